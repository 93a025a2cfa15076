/*
 * kinc_rmt.h -- KINC's RMT analytic (random-matrix-theory thresholding of a
 * correlation matrix) on the GPU.  Replaces RMT::process
 * (src/core/rmt.cpp:33-122): for thresholds from threshold_start down in
 * threshold_step, the correlation matrix is pruned to the (gene, cluster) rows
 * whose largest |r| reaches the threshold (computePruneMatrix,
 * src/core/rmt.cpp:202-245), its eigenvalues are computed (computeEigenvalues,
 * :252-282), and the nearest-neighbour spacing distribution of the unfolded
 * eigenvalues is compared with the Poisson distribution by a chi-square test
 * averaged over unfolding paces (computeChiSquare / computePaceChiSquare /
 * degenerate / unfold, :289-439).  The search stops once a chi-square above
 * chi_square_threshold2 follows one below chi_square_threshold1; the last
 * threshold whose chi-square was below chi_square_threshold1 is the result.
 *
 * The pruned matrix is built on the GPU from the CMX items (no dense
 * genes x genes x clusters copy) and its eigenvalues come from cuSOLVER's
 * symmetric eigensolver in double precision, as the reference's solver works
 * in double; the unfolding (Akima spline) and the chi-square run on the host.
 */
#ifndef KINC_RMT_H
#define KINC_RMT_H

#include <stdint.h>

#include "kinc_sim.h"

#ifdef __cplusplus
extern "C" {
#endif

/* no threshold above threshold_stop passed the test (the reference's "RMT Threshold Error") */
#define KINC_RMT_ENOTHRESHOLD 6
/* the unfolding spline needs strictly increasing eigenvalues in |lambda| order (the
 * reference's spline library rejects them too) */
#define KINC_RMT_ESPLINE 7

/* Arguments of src/core/rmt_input.cpp, defaults src/core/rmt.h:31-39. */
typedef struct kinc_rmt_params
{
   float threshold_start;        /* 0.99 */
   float threshold_step;         /* 0.001 */
   float threshold_stop;         /* 0.5 */
   float chi_square_threshold1;  /* 99.607 */
   float chi_square_threshold2;  /* 200 */
   int32_t min_eigenvalue_size;  /* 50 */
   int32_t min_unfolding_pace;   /* 10 */
   int32_t max_unfolding_pace;   /* 40 */
   int32_t histogram_bin_size;   /* 60 */
} kinc_rmt_params;

void kinc_rmt_params_default(kinc_rmt_params* p);

/*
 * The analytic over CMX items already in memory: n items (x > y gene indices,
 * c cluster, r = the cluster's first correlation) of a matrix of `genes` genes
 * and `max_clusters` clusters per pair.  Writes the reference's log lines
 * ("threshold<TAB>size<TAB>chi" per step, then the final threshold) to log_path
 * when it is not NULL, and the final threshold to *out_threshold.  steps_out,
 * when not NULL, receives up to steps_cap (threshold, size, chi) triples.
 */
int kinc_rmt_run_items(int32_t genes, int32_t max_clusters, int64_t n, const int32_t* x, const int32_t* y,
                       const int8_t* c, const float* r, const kinc_rmt_params* p, const char* log_path,
                       float* out_threshold, float* steps_out, int32_t steps_cap, int32_t* steps);

/* The same reading a CMX file (include/kinc_pairwise_matrix.h). */
int kinc_rmt_run(const char* cmx_path, int32_t little_endian, const kinc_rmt_params* p, const char* log_path,
                 float* out_threshold);

/*
 * computeChiSquare (src/core/rmt.cpp:289-323) on the host for eigenvalues
 * already sorted by ascending |lambda| (float, as the reference converts
 * them): -1 when fewer than min_eigenvalue_size unique values remain.
 */
int kinc_rmt_chi_square(const float* eigens, int32_t n, const kinc_rmt_params* p, float* out_chi);

/* Eigenvalues of the pruned matrix at one threshold, sorted by ascending |lambda|;
 * *size receives the pruned dimension (eigens must hold genes * max_clusters floats). */
int kinc_rmt_prune_eigenvalues(int32_t genes, int32_t max_clusters, int64_t n, const int32_t* x, const int32_t* y,
                               const int8_t* c, const float* r, float threshold, float* eigens, int32_t* size);

/* Message of the last failed kinc_rmt_* call on this thread. */
const char* kinc_rmt_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
