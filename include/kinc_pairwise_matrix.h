/*
 * kinc_pairwise_matrix.h -- KINC's pairwise matrix files (CCM cluster
 * matrix, CMX correlation matrix) and expression matrix (EMX) data, plus the
 * ordered block-by-block runner that writes them.
 *
 * Byte layout of a pairwise matrix (the data section KINC's classes write
 * through their stream):
 *   header, 30 bytes         src/core/pairwise_matrix.h:32-40, src/core/pairwise_matrix.cpp:12-57
 *     i32 geneSize, i32 maxClusterSize, i32 dataSize, i64 pairSize, i64 clusterSize, i16 offset
 *   sub-header, `offset` bytes
 *     CCM: i32 sampleSize          src/core/ccmatrix.h:21-23
 *     CMX: i8 correlationSize      src/core/correlationmatrix.h:21-23
 *   items, each 9 + dataSize bytes, in strictly increasing indent order
 *     i32 x, i32 y, i8 cluster     src/core/pairwise_matrix.cpp:122-151
 *     CCM payload: (sampleSize+1)/2 bytes, sample 2i in the low nibble, 2i+1 in the high nibble
 *                                  src/core/ccmatrix.cpp:223-243, dataSize src/core/ccmatrix.cpp:126
 *     CMX payload: correlationSize float32   src/core/correlationmatrix.cpp:231-242
 * EMX: i32 geneSize, i32 sampleSize, then float32 [gene][sample]   src/core/expressionmatrix.cpp:21-37
 *
 * The reference writes through ACE's stream class, which is not part of the
 * KINC tree; its byte order is a parameter here (big-endian, the Qt stream
 * default, unless little_endian is set).  Gene/sample names, which ACE keeps
 * as metadata, are not part of these files.
 */
#ifndef KINC_PAIRWISE_MATRIX_H
#define KINC_PAIRWISE_MATRIX_H

#include <stdint.h>

#include "kinc_sim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define KINC_PM_CCM 1
#define KINC_PM_CMX 2

typedef struct kinc_pm kinc_pm;

/* Pairwise::Matrix::initialize + writeNewData: a new CCM (subsize = samples) or
 * CMX (subsize = correlations per cluster) file. */
int kinc_pm_create(const char* path, int32_t type, int32_t genes, int32_t max_clusters, int32_t subsize,
                   int32_t little_endian, kinc_pm** out);

/* Append n items already in pair order: (x[i], y[i], c[i]) and the payload of
 * item i at payload + i*stride (CCM: samples int8 codes 0/1/6/7/8/9, packed to
 * nibbles here; CMX: subsize float32).  Matrix::write's rule holds: each indent
 * (x(x-1)/2 + y)*64 + c must exceed the last one written, else KINC_SIM_EORDER.
 * pairSize counts the distinct (x, y) pairs written. */
int kinc_pm_write_items(kinc_pm* m, int64_t n, const int32_t* x, const int32_t* y, const int8_t* c,
                        const void* payload);

/* The same with CCM payloads already packed ((samples + 1) / 2 bytes per item, as
 * kinc_sim_compact_block_device writes them); CMX payloads as above. */
int kinc_pm_write_items_packed(kinc_pm* m, int64_t n, const int32_t* x, const int32_t* y, const int8_t* c,
                               const void* payload);

/* Matrix::finish: rewrite the header counts and close. */
int kinc_pm_close(kinc_pm* m);

/* Open an existing file for reading; reports its header. */
int kinc_pm_open(const char* path, int32_t type, int32_t little_endian, kinc_pm** out, int32_t* genes,
                 int32_t* max_clusters, int32_t* subsize, int64_t* pairs, int64_t* clusters);

/* Read items [first, first+n): CCM payloads unpacked to one int8 code per sample. */
int kinc_pm_read_items(kinc_pm* m, int64_t first, int64_t n, int32_t* x, int32_t* y, int8_t* c, void* payload);

/* EMX data section. */
int kinc_emx_write(const char* path, const float* gem, int32_t genes, int32_t samples, int32_t little_endian);
int kinc_emx_read_header(const char* path, int32_t little_endian, int32_t* genes, int32_t* samples);
int kinc_emx_read(const char* path, int32_t little_endian, float* gem, int64_t capacity);

/*
 * Resume an interrupted kinc_sim_run_to_files: the runner appends work blocks in pair order and
 * rewrites the header counts only when it finishes, so an interrupted CCM/CMX file holds the
 * items of the finished blocks and possibly part of the next.  *resume_block is the work block of
 * the last whole item on disk -- the smallest over the two files -- or first_block for a file
 * without items or not yet created (either path may be NULL: that file is not written);
 * both files are cut back to the items of the blocks before *resume_block and their header
 * counts rewritten.  Running blocks [*resume_block, end) into new files and joining them after
 * these with kinc_pm_concat gives the files of the uninterrupted run.
 */
int kinc_pm_resume_point(const char* ccm_path, const char* cmx_path, int32_t little_endian, int64_t first_block,
                         int64_t* resume_block);

/*
 * The CCM or CMX files of a sharded run (each rank's contiguous range of work blocks) joined into
 * one, in the order given: the inputs must be of one type (detected from the first), agree on
 * genes, maximum clusters and payload size, and keep strictly increasing indent order across the
 * joins (else KINC_SIM_EINVAL / KINC_SIM_EORDER, and no output file is left).  The output may not
 * be one of the inputs.
 */
int kinc_pm_concat(const char* out_path, const char* const* in_paths, int32_t n, int32_t little_endian);

/*
 * ExportCorrelationMatrix (src/core/exportcorrelationmatrix.cpp:17-117): the CMX and CCM files as
 * tab-separated text, one line per CMX cluster: x, y, cluster, clusters of the pair, then the
 * counts of sample codes 1 (in the cluster), 9 (missing), 8 (post-outlier), 7 (pre-outlier) and
 * 6 (below minexpr) from the CCM cluster, the cluster's first correlation (%.6g) and the sample
 * mask ('0' + code per sample).  Pairs with a single CMX cluster take no CCM data: zero counts
 * and a mask of '0's, as the reference writes them.
 */
int kinc_pm_export_text(const char* ccm_path, const char* cmx_path, int32_t little_endian, const char* out_path);

/*
 * Extract (src/core/extract.cpp:24-274): the co-expression network of the CMX clusters whose first
 * correlation r has min_corr <= |r| <= max_corr (the reference's defaults: 0.85, 1.0), written as
 * a tab-separated edge list (tsv_path) and as GraphML (graphml_path); either may be NULL.
 * Multi-cluster pairs take their code counts and sample mask from the CCM; single-cluster pairs
 * take the mask from the EMX ('9' where either gene is NaN, else '1').  names_path: one gene name
 * per line (NULL: the gene indices).
 */
int kinc_pm_extract(const char* emx_path, const char* ccm_path, const char* cmx_path, const char* names_path,
                    int32_t little_endian, float min_corr, float max_corr, const char* tsv_path,
                    const char* graphml_path);

/*
 * ImportCorrelationMatrix (src/core/importcorrelationmatrix.cpp:22-141): the 11-column text that
 * kinc_pm_export_text writes (and any file of that shape), read back into a CCM and a CMX file.
 * Lines are split on white space.  A line of 11 fields is one cluster: fields 0 and 1 are the
 * pair (x, y), field 9 the correlation and field 10 the sample mask (one digit per sample); the
 * cluster number, cluster count and code counts are not read, the clusters of a pair being
 * numbered in line order.  Consecutive lines of one pair form one pair; the CMX
 * (one correlation per cluster) receives every pair, the CCM the pairs with
 * more than one cluster (codes = the mask's digits, any other character code 15).  Lines of 0
 * or 1 fields are skipped; any other field count, a mask whose length is not `samples`, a pair
 * out of increasing order or outside `genes`, or more than max_clusters clusters is an error
 * (KINC_SIM_EINVAL or KINC_SIM_EORDER) naming the line.  A field that is not a number reads as
 * 0, as Qt's toInt/toFloat return it.
 */
int kinc_pm_import_text(const char* in_path, const char* ccm_path, const char* cmx_path, int32_t genes,
                        int32_t max_clusters, int32_t samples, int32_t little_endian);

/* ExpressionMatrix::Transform (src/core/expressionmatrix.h), the element-wise transform an
 * expression matrix is imported with: "none", "natural logarithm", "logarithm base 2",
 * "logarithm base 10". */
#define KINC_EMX_TRANSFORM_NONE 0
#define KINC_EMX_TRANSFORM_NLOG 1
#define KINC_EMX_TRANSFORM_LOG2 2
#define KINC_EMX_TRANSFORM_LOG10 3

/*
 * ImportExpressionMatrix (src/core/importexpressionmatrix.cpp:20-180): white-space separated
 * text, one gene per line (name, then one value per sample), into an EMX file.  samples == 0:
 * the first line holds the sample names and sets the sample count; else the samples are named
 * 0..samples-1 and every line is a gene.  A value equal to nan_token (NULL or "": none) is NaN;
 * any other is read as a double, rounded to float, then transformed (the float functions
 * logf / log2f / log10f).  Blank lines are skipped.  A line whose field count is not
 * samples + 1, or a value that is not a number, is KINC_SIM_EINVAL.  Gene and sample names,
 * which KINC keeps as metadata, are written one per line to gene_names_path and
 * sample_names_path when those are not NULL.
 */
int kinc_emx_import_text(const char* in_path, const char* nan_token, int32_t samples, int32_t transform,
                         int32_t little_endian, const char* emx_path, const char* gene_names_path,
                         const char* sample_names_path);

/*
 * ExportExpressionMatrix (src/core/exportexpressionmatrix.cpp:20-100): the EMX as text.  First
 * line: each sample name followed by a tab; then per gene its name and, per sample, a tab and
 * either nan_token (NaN; NULL = "") or the value with the import's transform undone (expf(v);
 * 2^v, 10^v by pow in double, rounded to float) at 12 significant digits (%.12g).  Names are read one per
 * line from gene_names_path / sample_names_path, or are the indices when NULL.  transform is the
 * one the matrix was imported with (KINC stores it as metadata, which the EMX data section does
 * not hold).
 */
int kinc_emx_export_text(const char* emx_path, int32_t little_endian, const char* gene_names_path,
                         const char* sample_names_path, int32_t transform, const char* nan_token,
                         const char* out_path);

/* Message of the last failed kinc_pm_* / kinc_emx_* / kinc_sim_run_to_files call on this thread. */
const char* kinc_pm_last_error(void);

/*
 * The analytic's block loop (ACE's serial runner + Similarity::process,
 * src/core/similarity.cpp:17-39,66-127) on the worker: work blocks
 * [first_block, first_block + nblocks) are executed in order, filtered and
 * appended to the CCM and CMX files (either path may be NULL).  nblocks < 0
 * means all remaining blocks.  The files are created and finished here.
 */
int kinc_sim_run_to_files(kinc_sim_ctx* ctx, const char* ccm_path, const char* cmx_path, int32_t little_endian,
                          int64_t first_block, int64_t nblocks);

/*
 * The same with the device block size chosen by the caller: device_block pairs
 * (rounded down to whole work blocks; 0 = kinc_sim_max_device_block).  Both
 * forms run two result slots, so the GPU computes device block b while block
 * b-1's kept items come back through pinned buffers on a second stream and
 * are written.
 */
int kinc_sim_run_to_files_ex(kinc_sim_ctx* ctx, const char* ccm_path, const char* cmx_path, int32_t little_endian,
                             int64_t first_block, int64_t nblocks, int64_t device_block);

#ifdef __cplusplus
}
#endif

#endif
