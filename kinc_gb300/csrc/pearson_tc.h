/*
 * pearson_tc.h -- host interface of the tensor-core Pearson form
 * (pearson_gemm.cu), used by the worker context in kinc_sim.cu.
 */
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace kinc_tc {

struct TcMaps
{
   CUtensorMap x[5];                  /* 128-row boxes per operand plane */
   CUtensorMap y[5];                  /* 64-row boxes per operand plane */
   CUtensorMap y2[3];                 /* 32-row boxes (TF32, the CTA-pair kernel's y-side halves) */
};

}  // namespace kinc_tc

/* Operand planes and tensor maps of one expression matrix. */
struct TcState
{
   int mode = 0;                      /* 1 TF32, 2 3xBF16, 3 FP32 on the CUDA cores, 4 scaled FP16 */
   int Gp = 0, Sp = 0;                /* padded genes (x128, x256 for the CTA-pair TF32 kernel) and samples (x64) */
   void* ops = nullptr;               /* operand planes [Gp][Sp] */
   kinc_tc::TcMaps maps;
   /* tensor-core tile list of the last range enqueued (row tiles tiles_ia..tiles_ib, rows to tiles_xb) */
   int2* d_tiles = nullptr;
   int2* h_tiles = nullptr;           /* pinned */
   int64_t tiles_cap = 0;
   int ntiles = 0;
   int tiles_ia = -1, tiles_ib = -1;
   int64_t tiles_xb = -1;
   cudaEvent_t tiles_ev = nullptr;    /* the list's host-to-device copy */
};

/* centred/masked operands and their tensor maps for d_gem [G][S] */
cudaError_t tc_prepare(TcState& t, const float* d_gem, int G, int S, float min_expr, int mode, cudaStream_t st,
                       char* err, size_t errlen);
void tc_release(TcState& t);
/* pairs [start, start+size): K = 1, corr[.][0] = pairwise-complete Pearson, NaN in columns >= 1 */
cudaError_t tc_enqueue(TcState& t, int G, int S, int min_samples, int max_k, int64_t start, int64_t size,
                       int8_t* d_K, float* d_corr, int* d_status, cudaStream_t st, int* launches);
