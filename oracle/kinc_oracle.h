/*
 * kinc_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of KINC's CPU Similarity path (the serial worker and
 * the Pairwise:: models) used as the checker for the CUDA implementation.
 * Only tests, the smoke check and bench.py's CPU-baseline leg may load it.
 * Nothing in the product links or calls it.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the KINC source tree).  Float exp/log go through kinc_fmath.h so that the
 * oracle, the reference sources compiled by oracle/build_ref.py and the GPU
 * agree bit for bit; the oracle is pinned against the compiled reference
 * sources by tests/test_oracle_vs_ref.py and tests/golden/.
 */
#ifndef KINC_ORACLE_H
#define KINC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ko_params
{
   int32_t clus_method;   /* 0 none, 1 gmm, 2 kmeans */
   int32_t corr_method;   /* 0 pearson, 1 spearman, 2 both ([k][0] Pearson, [k][1] Spearman) */
   float   min_expr;
   int32_t min_samples;
   int32_t min_clusters;
   int32_t max_clusters;
   int32_t criterion;     /* 0 BIC, 1 ICL */
   int32_t pre_out;
   int32_t post_out;
   float   min_corr;
   float   max_corr;
   int32_t semantics;     /* 0 reference CPU path, 1 fixed gathers */
   int32_t rand_mode;     /* 0 glibc rand() stream (serial path); 1 the OpenCL worker's GMM: per-fit
                             POSIX LCG, float BIC/ICL, zero-determinant failure rule */
} ko_params;

/* glibc random_r TYPE_3 (the default rand()) restated from its published
 * description: r[0]=seed, r[i]=16807*r[i-1] mod (2^31-1) for i<31,
 * r[i]=r[i-31] for i in 31..33, r[i]=r[i-31]+r[i-3] mod 2^32, output k is
 * r[k+344]>>1. */
typedef struct ko_rand
{
   uint32_t r[34];
   int32_t  head;         /* index of the oldest of the 34 kept values */
   uint64_t drawn;        /* outputs produced so far */
} ko_rand;

void     ko_rand_seed(ko_rand* g, uint32_t seed);
int32_t  ko_rand_next(ko_rand* g);
void     ko_rand_skip(ko_rand* g, uint64_t n);
/* libc's own rand() after srand(seed): used by the tests to pin the restatement */
void     ko_libc_rand(uint32_t seed, int32_t n, int32_t* out);

/* draws of rand() one qualifying pair consumes (GMM: sum K; K-means: 10 sum K) */
int64_t  ko_draws_per_pair(const ko_params* p);
/* number of pairs with linear index < end whose usable-sample count N >= min_samples */
int64_t  ko_count_qualifying(const float* gem, int32_t G, int32_t S, const ko_params* p, int64_t end);

/* linear pair index -> (x, y), x > y  (src/core/pairwise_index.cpp:32-57) */
void     ko_pair_xy(int64_t index, int32_t* x, int32_t* y);

/*
 * Run one work block of `size` pairs starting at linear index `start` exactly
 * like Similarity::Serial::execute (src/core/similarity_serial.cpp:33-101).
 * `rng` must be positioned where the process-global rand() stream would be at
 * the block start (see ko_count_qualifying / ko_draws_per_pair).
 * Outputs per pair: K, labels[S] (valid when K > 1), corr[max_clusters]
 * (entries k < K valid), N (usable samples).  Any output may be NULL.
 */
int ko_run_block(const float* gem, int32_t G, int32_t S, const ko_params* p, ko_rand* rng,
                 int64_t start, int64_t size,
                 int8_t* out_K, int8_t* out_labels, float* out_corr, int32_t* out_N);

/* Same, over `nblocks` work blocks of 32768 pairs (block indices in `blocks`)
 * with `threads` POSIX threads, each block positioned on the rand() stream
 * independently.  Used by the CPU baseline.  Returns pairs processed. */
/* Segments [starts[s], starts[s]+sizes[s]) with `threads` POSIX threads, each
 * positioned at rand_pos[s] on the rand() stream; wall time of the compute in
 * *seconds.  The _out form also stores each segment's results back to back
 * (K [Σsizes], labels [Σsizes][S], corr [Σsizes][max_clusters]); any may be NULL. */
int64_t ko_run_segments_parallel(const float* gem, int32_t G, int32_t S, const ko_params* p,
                                 const int64_t* starts, const int64_t* sizes, const uint64_t* rand_pos,
                                 int32_t nseg, int32_t threads, double* seconds);
int64_t ko_run_segments_parallel_out(const float* gem, int32_t G, int32_t S, const ko_params* p,
                                     const int64_t* starts, const int64_t* sizes, const uint64_t* rand_pos,
                                     int32_t nseg, int32_t threads, double* seconds,
                                     int8_t* out_K, int8_t* out_labels, float* out_corr);

int64_t ko_run_blocks_parallel(const float* gem, int32_t G, int32_t S, const ko_params* p,
                               const int64_t* blocks, int32_t nblocks, int32_t threads);

/*
 * Similarity::process (src/core/similarity.cpp:66-127) for `size` pairs:
 * the kept clusters of each pair.  For each kept (pair, cluster) it appends
 * x, y, cluster (renumbered 0..c-1), r, and S sample codes.  Returns the
 * number of CMX items; *n_ccm receives the number of CCM items (clusters of
 * pairs with K > 1).  Arrays must hold size*max_clusters entries (codes:
 * times S).
 */
int64_t ko_process_block(int32_t S, const ko_params* p, int64_t start, int64_t size,
                         const int8_t* K, const int8_t* labels, const float* corr,
                         int32_t* cmx_x, int32_t* cmx_y, int8_t* cmx_c, float* cmx_r,
                         int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c, int8_t* ccm_codes,
                         int64_t* n_ccm);

/* FP64 pairwise-complete Pearson over all usable samples of pair (x, y) */
double ko_pearson_fp64(const float* gem, int32_t S, int32_t x, int32_t y, float min_expr,
                       int32_t min_samples);

/* the same for n pairs (xs[i], ys[i]) with `threads` POSIX threads */
void ko_pearson_fp64_batch(const float* gem, int32_t S, const int32_t* xs, const int32_t* ys, int64_t n,
                           float min_expr, int32_t min_samples, double* out, int32_t threads);

#ifdef __cplusplus
}
#endif

#endif
