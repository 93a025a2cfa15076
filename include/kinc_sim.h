/*
 * kinc_sim.h -- C ABI of the GB300 Similarity worker.
 *
 * This is the drop-in replacement for KINC's OpenCL Similarity worker: the
 * object that turns one work block {start, size} of gene pairs into one
 * result block {K, labels, correlations} per pair.  It replaces
 *
 *   Similarity::OpenCL::initialize(::OpenCL::Context*)     src/core/similarity_opencl.cpp:34-70
 *   Similarity::OpenCL::makeWorker()                         src/core/similarity_opencl.cpp:24-27
 *   Similarity::OpenCL::Worker::Worker(...)                  src/core/similarity_opencl_worker.cpp:50-86
 *   Similarity::OpenCL::Worker::execute(const Block*)        src/core/similarity_opencl_worker.cpp:93-271
 *
 * and computes what Similarity::Serial::execute computes
 * (src/core/similarity_serial.cpp:33-101) on the same inputs.
 *
 * Conventions: every call returns 0 on success and a non-zero KINC_SIM_E*
 * code otherwise (no exceptions cross the ABI); kinc_sim_last_error() gives
 * the message.  The context owns all device memory; callers own host
 * buffers.  A context is used by one host thread at a time.
 */
#ifndef KINC_SIM_H
#define KINC_SIM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KINC_SIM_OK 0
#define KINC_SIM_EINVAL 1      /* invalid argument */
#define KINC_SIM_ECUDA 2       /* CUDA runtime error */
#define KINC_SIM_ENOMEM 3      /* device or host allocation failed */
#define KINC_SIM_EKERNEL 4     /* a kernel reported an error status */
#define KINC_SIM_EORDER 5      /* out-of-order write to a pairwise matrix */
#define KINC_SIM_EIO 8         /* a file could not be written (codes 6 and 7: include/kinc_rmt.h) */

/* Work-block size the reference splits all pairs into (src/core/similarity.cpp:20). */
#define KINC_SIM_WORK_BLOCK_SIZE 32768

typedef struct kinc_sim_ctx kinc_sim_ctx;

/*
 * Analytic arguments: the Similarity CLI options (src/core/similarity_input.cpp:96-254)
 * with the member defaults of src/core/similarity.h:58-71, plus three
 * options of this implementation.
 */
typedef struct kinc_sim_params
{
   int32_t clus_method;   /* --clusmethod: 0 none, 1 gmm, 2 kmeans            (default 0) */
   int32_t corr_method;   /* --corrmethod: 0 pearson, 1 spearman              (default 0);
                             2 both (Pearson and Spearman per cluster in one pass; not in the reference,
                             which runs one method per analytic) */
   float   min_expr;      /* --minexpr                                        (default -inf) */
   int32_t min_samples;   /* --minsamp, >= 1                                  (default 30) */
   int32_t min_clusters;  /* --minclus, 1..64                                 (default 1) */
   int32_t max_clusters;  /* --maxclus, 1..64                                 (default 5) */
   int32_t criterion;     /* --crit: 0 BIC, 1 ICL                             (default 1) */
   int32_t pre_out;       /* --preout                                         (default 0) */
   int32_t post_out;      /* --postout                                        (default 0) */
   float   min_corr;      /* --mincorr, 0..1                                  (default 0.5) */
   float   max_corr;      /* --maxcorr, 0..1                                  (default 1) */
   int32_t ksize;         /* --ksize: accepted for CLI compatibility; pairs per launch are chosen here */
   int32_t semantics;     /* 0: the reference CPU path, including its packed-array indexing in
                                Pearson/Spearman (default); 1: each sample's own values */
   int32_t rand_mode;     /* 0: the process-global glibc rand() stream of a serial KINC run (default);
                             1: the OpenCL worker's GMM (src/opencl/gmm.cl): the POSIX LCG reset per
                                fit, BIC/ICL evaluated in float, a fit failing only on a zero
                                covariance determinant (K-means: the LCG with the CPU path's fit) */
   int32_t precision;     /* clusmethod none + pearson + semantics 1 only: 0 per-pair FP32 (default),
                             1 TF32 tensor cores, 2 3xBF16 tensor cores, 3 FP32 CUDA cores, 4 FP16
                             tensor cores with each gene's centred values scaled by a power of two
                             (1-4: the pairwise-complete Pearson as a tiled masked contraction; labels
                             are not written) */
} kinc_sim_params;

/* Fill `p` with the reference defaults. */
int kinc_sim_params_default(kinc_sim_params* p);

/*
 * Create a worker for an expression matrix `gem` (host, row-major [genes][samples]
 * float32, NaN = missing), as Similarity::OpenCL::initialize uploads the EMX once.
 */
int kinc_sim_create(const float* gem, int32_t genes, int32_t samples, const kinc_sim_params* params,
                    kinc_sim_ctx** out);

void kinc_sim_destroy(kinc_sim_ctx* ctx);

/* Message of the last failed call on `ctx`; with ctx NULL, of the calling thread's last failed call
 * that has no context (kinc_sim_create, kinc_sim_execute_block_noalloc). */
const char* kinc_sim_last_error(const kinc_sim_ctx* ctx);

/* The context's arguments and matrix shape (any output may be NULL). */
int kinc_sim_get_params(const kinc_sim_ctx* ctx, kinc_sim_params* params, int32_t* genes, int32_t* samples);

/* Total pairs G(G-1)/2 and the number of 32768-pair work blocks (Similarity::size). */
int64_t kinc_sim_total_pairs(const kinc_sim_ctx* ctx);
int32_t kinc_sim_num_work_blocks(const kinc_sim_ctx* ctx);

/*
 * Execute the pairs [start, start + size) in linear pair order (x > y,
 * index = x(x-1)/2 + y), writing HOST arrays:
 *   out_K[size]                  int8   number of clusters (0 = not enough samples / all fits failed)
 *   out_labels[size * samples]   int8   per-sample labels: cluster id >= 0, or -9 missing,
 *                                        -6 below minexpr, -7 pre-outlier, -8 post-outlier
 *                                        (meaningful when K > 1)
 *   out_corr[size * max_clusters * nc] float correlation per cluster k < K, NaN elsewhere;
 *                                  nc = 2 when corr_method is 2 (row [k][0] Pearson, [k][1] Spearman)
 * Any output pointer may be NULL.  Blocks may be executed in any order; the
 * position on the rand() stream is derived from `start`.
 */
int kinc_sim_execute_block(kinc_sim_ctx* ctx, int64_t start, int64_t size, int8_t* out_K,
                           int8_t* out_labels, float* out_corr);

/*
 * Same with DEVICE output arrays, stream-ordered on `stream` (a cudaStream_t,
 * 0 = the context's own stream); returns after enqueueing.  size must be
 * <= kinc_sim_max_device_block(ctx).
 */
int kinc_sim_execute_block_device(kinc_sim_ctx* ctx, int64_t start, int64_t size, int8_t* d_K,
                                  int8_t* d_labels, float* d_corr, void* stream);
int64_t kinc_sim_max_device_block(const kinc_sim_ctx* ctx);

/*
 * Same with HOST output arrays, stream-ordered on the context's stream: the
 * block is computed and its K, labels and correlations copied back (to pinned
 * arrays for the copies to run asynchronously) without waiting; the arrays
 * are complete after kinc_sim_synchronize.  size must be <=
 * kinc_sim_max_device_block(ctx), and one block may be in flight per context
 * (the context's device buffers hold it).
 */
int kinc_sim_execute_block_async(kinc_sim_ctx* ctx, int64_t start, int64_t size, int8_t* out_K,
                                 int8_t* out_labels, float* out_corr);

/* Synchronise the context's stream and report any kernel error status. */
int kinc_sim_synchronize(kinc_sim_ctx* ctx);

/*
 * Similarity::process (src/core/similarity.cpp:66-127) for one executed
 * block, on HOST arrays from kinc_sim_execute_block: the clusters whose
 * correlation passes !isnan(r) && mincorr <= |r| <= maxcorr, renumbered
 * 0..c-1 per pair.  CMX items: (x, y, cluster, r) for pairs with K > 0;
 * CCM items: (x, y, cluster, samples codes) for pairs with K > 1, the codes
 * being labels >= 0 ? (k == label) : -label.  Capacity arguments bound the
 * output arrays (items; codes hold cap_ccm * samples bytes).  *n_cmx and
 * *n_ccm receive the counts.
 */
int kinc_sim_process_block(const kinc_sim_ctx* ctx, int64_t start, int64_t size, const int8_t* K,
                           const int8_t* labels, const float* corr,
                           int32_t* cmx_x, int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int64_t cap_cmx,
                           int64_t* n_cmx,
                           int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c, int8_t* ccm_codes, int64_t cap_ccm,
                           int64_t* n_ccm);

/*
 * The same filter on the GPU for a block executed with kinc_sim_execute_block_device,
 * stream-ordered: DEVICE inputs d_K, d_labels (NULL: no CCM items), d_corr; DEVICE outputs
 * with room for cap_cmx / cap_ccm items (any output array may be NULL).  CCM payloads are
 * written packed, (samples + 1) / 2 bytes per item with sample 2i in the low nibble, as the
 * CCM file stores them.  d_counts[0] / d_counts[1] receive the numbers of CMX / CCM items,
 * even when they exceed the capacities (items beyond them are dropped).
 */
int kinc_sim_compact_block_device(kinc_sim_ctx* ctx, int64_t start, int64_t size, const int8_t* d_K,
                                  const int8_t* d_labels, const float* d_corr,
                                  int32_t* cmx_x, int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int64_t cap_cmx,
                                  int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c, uint8_t* ccm_packed,
                                  int64_t cap_ccm, uint64_t* d_counts, void* stream);

/* The same filter without a context (host code only; no GPU needed): the
 * caller passes the analytic arguments and the sample count. */
int kinc_sim_process_pairs(const kinc_sim_params* params, int32_t samples, int64_t start, int64_t size,
                           const int8_t* K, const int8_t* labels, const float* corr,
                           int32_t* cmx_x, int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int64_t cap_cmx,
                           int64_t* n_cmx,
                           int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c, int8_t* ccm_codes, int64_t cap_ccm,
                           int64_t* n_ccm);

/* Per-pair usable-sample counts N for [start, start+size) (diagnostics / binning checks). */
int kinc_sim_pair_counts(kinc_sim_ctx* ctx, int64_t start, int64_t size, int32_t* out_N);

/* Kernel launches made by the last kinc_sim_execute_block* call (for accounting). */
int32_t kinc_sim_last_launch_count(const kinc_sim_ctx* ctx);

/*
 * Launch shape of the per-pair kernel.  Every shape computes the same bits;
 * only the speed differs, so the shape is picked by measurement
 * (kinc_sim_autotune) rather than fixed.  Replaces the hand-set work-item
 * count of KINC's OpenCL worker (--ksize, src/core/similarity_input.cpp:241-251),
 * which this worker does not need for correctness.
 *   warps_per_cta  warps of one CTA: 4, 8 or 16 (GMM: 4, 10 or 20); the SM holds
 *                  16 warps (GMM: 20, at fewer registers each) either way
 *   rounds         1: a CTA's warps take their 32-pair tiles together, round by
 *                  round (they then run the same code region at the same time);
 *                  0: every warp takes its next tile as soon as it is done
 *   prefetch       0, 4, 8 or 16: samples ahead the clustering sweeps (GMM EM passes,
 *                  K-means Lloyd and log-likelihood passes) prefetch into L2
 * Pearson without clustering (clusmethod none, corrmethod pearson) runs one thread
 * per pair and takes no shape.
 */
typedef struct kinc_sim_launch
{
   int32_t warps_per_cta;
   int32_t rounds;
   int32_t prefetch;
   int32_t reserved;
} kinc_sim_launch;

/* One timed candidate of kinc_sim_autotune. */
typedef struct kinc_sim_tune_entry
{
   kinc_sim_launch launch;
   double ms;             /* device time of the sample block */
} kinc_sim_tune_entry;

int kinc_sim_get_launch(const kinc_sim_ctx* ctx, kinc_sim_launch* launch);
/* KINC_SIM_EINVAL for a shape outside the values above */
int kinc_sim_set_launch(kinc_sim_ctx* ctx, const kinc_sim_launch* launch);

/*
 * Pick the launch shape by timing: the pairs [start, start + size) (size is
 * capped at kinc_sim_max_device_block) run once per candidate on the context's
 * stream, timed with CUDA events, in a coordinate descent from the current
 * shape over prefetch (clustering only), warps_per_cta and rounds (not for GMM,
 * which keeps the current shape's rounds); the fastest is applied.  With use_cache, the shape is first looked up -- and afterwards
 * stored -- in a small text cache keyed by the clustering and correlation
 * arguments, max_clusters, the sample count rounded up to a power of two and
 * the GPU (file: $KINC_TUNE_CACHE, else $XDG_CACHE_HOME/kinc_gb300/launch.txt,
 * else ~/.cache/kinc_gb300/launch.txt); a cache hit times nothing.  Up to
 * `cap` timed candidates are written to `entries` (may be NULL) and their
 * count to *n.  Synchronises the context's stream; the per-pair outputs of the
 * timed runs are discarded.  Not available for the tensor-core precisions.
 */
int kinc_sim_autotune(kinc_sim_ctx* ctx, int64_t start, int64_t size, int32_t use_cache, kinc_sim_launch* chosen,
                      kinc_sim_tune_entry* entries, int32_t cap, int32_t* n);

/*
 * Dense tcgen05 MMA rate of the current device, in TFLOP/s, for the operand type of
 * precision 1 (TF32) or 2 (BF16): one CTA per SM issuing 128 x 256 MMAs back to back
 * on operands resident in shared memory, timed with CUDA events (best of two after a
 * warm-up).  The ceiling the tensor-core Pearson form is measured against.  No
 * counterpart in the reference (its OpenCL worker has no tensor-core path).
 * Synchronises the device.
 */
int kinc_sim_tensor_peak(int32_t precision, double* tflops);

/* Work done since the last reset: out[0] = clustering model units (sum over
 * fits of iterations x N x K), out[1] = fits run, out[2..3] reserved.
 * Synchronises the context's stream. */
int kinc_sim_work_counters(kinc_sim_ctx* ctx, uint64_t* out, int reset);

/*
 * Allocation-free form of kinc_sim_execute_block_device, for callers that may
 * not allocate device memory: hosts that give the whole device to their own
 * pool allocator and forbid raw cudaMalloc (which also synchronises the
 * device), or that run this step where allocating is not allowed.  No
 * counterpart in the reference.
 *
 * The caller passes the expression matrix already on the device (d_gem,
 * row-major [genes][samples] float32) and device outputs laid out as in
 * kinc_sim_execute_block.  All working memory is a 64 MiB static device array
 * inside the library, which every GPU that loads the library holds until the
 * process exits.  Limits: samples <= 4096 and size <= 262144 pairs per call,
 * and the per-gene masks, per-pair arrays and the working space of at least
 * one block of the kernel's warps (16; GMM 20) must fit in the 64 MiB; precision must be 0 (the per-pair FP32
 * path; corr_method 0, 1 or 2 as in kinc_sim_create).  Other requests are
 * rejected with KINC_SIM_EINVAL and a message from kinc_sim_last_error(NULL).
 *
 * The first call on a device does a one-time set-up with that device current:
 * it looks up the array's device address and uploads the rand() jump table.
 * Every call runs
 * its kernels on `stream` (a cudaStream_t, 0 = default stream), then waits
 * for them with cudaStreamSynchronize and copies a status word back to the
 * host before returning.  Every call shares the one array, which keeps the
 * last call's contents, so calls that overlap on the GPU race; the function
 * serialises callers on the host side.
 */
int kinc_sim_execute_block_noalloc(const float* d_gem, int32_t genes, int32_t samples,
                                   const kinc_sim_params* params, int64_t start, int64_t size, int8_t* d_K,
                                   int8_t* d_labels, float* d_corr, void* stream);

/*
 * Sharding across processes (one per GPU): the contiguous range of whole work blocks
 * [*first_block, *first_block + *nblocks) that rank `rank` of `world` runs, for
 * kinc_sim_run_to_files(..., first_block, nblocks); the ranks' ranges cover every block once,
 * in rank order.  by_cost 0: equal block counts.  by_cost 1: equal estimated cost, a block
 * costing the sum over its pairs of n_x * n_y / samples (n_g: gene g's samples that are present
 * and not below min_expr), the expected usable count every per-pair pass is proportional to;
 * gem is the host matrix, row-major [genes][samples] (unused for by_cost 0).  Replaces the
 * block farming of ACE's MPI runner with a static partition; no counterpart in KINC itself.
 */
int kinc_shard_blocks(const float* gem, int32_t genes, int32_t samples, float min_expr, int32_t world,
                      int32_t rank, int32_t by_cost, int64_t* first_block, int64_t* nblocks);

#ifdef __cplusplus
}
#endif

#endif
