/*
 * rmt.cu -- the RMT analytic (include/kinc_rmt.h).
 *
 * GPU: per-(gene, cluster) largest |r| from the CMX items (computeMaximums,
 * src/core/rmt.cpp:164-195), then per threshold the pruned matrix
 * (computePruneMatrix, :202-245) scattered straight from the items into a
 * dense m x m double array in HBM and its eigenvalues from cuSOLVER's
 * symmetric divide-and-conquer solver (computeEigenvalues, :252-282, which
 * solves the same double matrix).
 *
 * Host: the eigenvalues sorted by ascending |lambda| and converted to float,
 * the unique values (degenerate, :374-388), the Akima-spline unfolding
 * (unfold, :395-439) and the chi-square against the Poisson spacing
 * distribution averaged over unfolding paces (computeChiSquare /
 * computePaceChiSquare, :289-367), in the reference's float/double types.
 * The reference calls GSL for the spline (gsl_interp_akima; GSL is not part
 * of the KINC tree and no version is pinned): the spline here is Akima's
 * published method (H. Akima, J. ACM 17(4), 1970) with the usual end
 * extension of the slopes, written from that description.
 */
#include "../../include/kinc_rmt.h"
#include "../../include/kinc_pairwise_matrix.h"
#include "kinc_fmath.h"

#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

namespace {

thread_local std::string r_err;

int rmt_fail(int code, const char* fmt, ...)
{
   char buf[512];
   va_list ap;
   va_start(ap, fmt);
   vsnprintf(buf, sizeof buf, fmt, ap);
   va_end(ap);
   r_err = buf;
   return code;
}

/* ------------------------------------------------------------------ GPU */

/* largest |r| per (gene, cluster); |r| >= 0 so its bits order like the value; NaN never wins */
__global__ void k_rmt_max(int64_t n, int K, const int32_t* __restrict__ x, const int32_t* __restrict__ y,
                          const int8_t* __restrict__ c, const float* __restrict__ r, unsigned int* __restrict__ mx)
{
   for ( int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x )
   {
      const float a = fabsf(r[i]);
      if ( !(a == a) ) continue;
      atomicMax(&mx[(int64_t)x[i] * K + c[i]], __float_as_uint(a));
      atomicMax(&mx[(int64_t)y[i] * K + c[i]], __float_as_uint(a));
   }
}

/* rank of each (gene, cluster) row kept at this threshold (-1: pruned); one block, m in *count */
__global__ void k_rmt_rank(int64_t rows, const unsigned int* __restrict__ mx, float t, int32_t* __restrict__ rank,
                           int32_t* __restrict__ count)
{
   __shared__ int32_t part[1024];
   const int tid = threadIdx.x;
   const int64_t per = (rows + blockDim.x - 1) / blockDim.x;
   const int64_t a = tid * per;
   const int64_t b = a + per < rows ? a + per : rows;
   int32_t s = 0;
   for ( int64_t i = a; i < b; ++i ) s += __uint_as_float(mx[i]) >= t;
   part[tid] = s;
   __syncthreads();
   if ( tid == 0 )
   {
      int32_t run = 0;
      for ( int i = 0; i < (int)blockDim.x; ++i )
      {
         const int32_t v = part[i];
         part[i] = run;
         run += v;
      }
      *count = run;
   }
   __syncthreads();
   int32_t run = part[tid];
   for ( int64_t i = a; i < b; ++i ) rank[i] = __uint_as_float(mx[i]) >= t ? run++ : -1;
}

/* unit diagonal */
__global__ void k_rmt_diag(int32_t m, double* __restrict__ A)
{
   for ( int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x )
      A[i * m + i] = 1.0;
}

/* the items with |r| >= t between kept rows: row-major lower triangle (i > j: gene x > gene y) */
__global__ void k_rmt_scatter(int64_t n, int K, int32_t m, const int32_t* __restrict__ x,
                              const int32_t* __restrict__ y, const int8_t* __restrict__ c,
                              const float* __restrict__ r, float t, const int32_t* __restrict__ rank,
                              double* __restrict__ A)
{
   for ( int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x )
   {
      const float v = r[i];
      if ( !(fabsf(v) >= t) ) continue;
      const int32_t ri = rank[(int64_t)x[i] * K + c[i]];
      const int32_t rj = rank[(int64_t)y[i] * K + c[i]];
      if ( ri < 0 || rj < 0 ) continue;
      A[(int64_t)ri * m + rj] = (double)v;
   }
}

struct RmtDevice
{
   int32_t G = 0, K = 0;
   int64_t n = 0;
   int32_t *dx = nullptr, *dy = nullptr, *drank = nullptr, *dcount = nullptr, *dinfo = nullptr;
   int8_t* dc = nullptr;
   float* dr = nullptr;
   unsigned int* dmax = nullptr;
   double *dA = nullptr, *dW = nullptr, *dwork = nullptr;
   size_t capA = 0, capWork = 0;
   cudaStream_t st = nullptr;
   cusolverDnHandle_t solver = nullptr;

   ~RmtDevice()
   {
      cudaFree(dx); cudaFree(dy); cudaFree(drank); cudaFree(dcount); cudaFree(dinfo); cudaFree(dc); cudaFree(dr);
      cudaFree(dmax); cudaFree(dA); cudaFree(dW); cudaFree(dwork);
      if ( solver ) cusolverDnDestroy(solver);
      if ( st ) cudaStreamDestroy(st);
   }
};

#define RCK(call)                                                                                  \
   do                                                                                              \
   {                                                                                               \
      cudaError_t e_ = (call);                                                                     \
      if ( e_ != cudaSuccess )                                                                     \
         return rmt_fail(e_ == cudaErrorMemoryAllocation ? KINC_SIM_ENOMEM : KINC_SIM_ECUDA, "%s: %s", \
                         #call, cudaGetErrorString(e_));                                           \
   } while ( 0 )

int device_setup(RmtDevice& d, int32_t G, int32_t K, int64_t n, const int32_t* x, const int32_t* y, const int8_t* c,
                 const float* r)
{
   if ( G < 1 || K < 1 || n < 0 || (n > 0 && (!x || !y || !c || !r)) )
      return rmt_fail(KINC_SIM_EINVAL, "Did not get valid input or logfile arguments.");
   for ( int64_t i = 0; i < n; ++i )
      if ( x[i] <= y[i] || y[i] < 0 || x[i] >= G || c[i] < 0 || c[i] >= K )
         return rmt_fail(KINC_SIM_EINVAL, "item %lld (%d, %d, %d) outside %d genes x %d clusters", (long long)i, x[i],
                         y[i], c[i], G, K);
   d.G = G;
   d.K = K;
   d.n = n;
   const int64_t rows = (int64_t)G * K;
   RCK(cudaStreamCreateWithFlags(&d.st, cudaStreamNonBlocking));
   if ( cusolverDnCreate(&d.solver) != CUSOLVER_STATUS_SUCCESS || cusolverDnSetStream(d.solver, d.st) != CUSOLVER_STATUS_SUCCESS )
      return rmt_fail(KINC_SIM_ECUDA, "cannot create the eigensolver");
   RCK(cudaMalloc(&d.dx, std::max<int64_t>(n, 1) * 4));
   RCK(cudaMalloc(&d.dy, std::max<int64_t>(n, 1) * 4));
   RCK(cudaMalloc(&d.dc, std::max<int64_t>(n, 1)));
   RCK(cudaMalloc(&d.dr, std::max<int64_t>(n, 1) * 4));
   RCK(cudaMalloc(&d.dmax, rows * sizeof(unsigned int)));
   RCK(cudaMalloc(&d.drank, rows * sizeof(int32_t)));
   RCK(cudaMalloc(&d.dcount, sizeof(int32_t)));
   RCK(cudaMalloc(&d.dinfo, sizeof(int32_t)));
   RCK(cudaMalloc(&d.dW, rows * sizeof(double)));
   if ( n > 0 )
   {
      RCK(cudaMemcpyAsync(d.dx, x, n * 4, cudaMemcpyHostToDevice, d.st));
      RCK(cudaMemcpyAsync(d.dy, y, n * 4, cudaMemcpyHostToDevice, d.st));
      RCK(cudaMemcpyAsync(d.dc, c, n, cudaMemcpyHostToDevice, d.st));
      RCK(cudaMemcpyAsync(d.dr, r, n * 4, cudaMemcpyHostToDevice, d.st));
   }
   RCK(cudaMemsetAsync(d.dmax, 0, rows * sizeof(unsigned int), d.st));   /* the reference starts every maximum at 0 */
   if ( n > 0 )
   {
      const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
      k_rmt_max<<<blocks, 256, 0, d.st>>>(n, K, d.dx, d.dy, d.dc, d.dr, d.dmax);
      RCK(cudaGetLastError());
   }
   return KINC_SIM_OK;
}

/* eigenvalues of the pruned matrix at threshold t, ascending |lambda|, as floats */
int device_eigenvalues(RmtDevice& d, float t, std::vector<float>& eig, int32_t& m)
{
   const int64_t rows = (int64_t)d.G * d.K;
   k_rmt_rank<<<1, 1024, 0, d.st>>>(rows, d.dmax, t, d.drank, d.dcount);
   RCK(cudaGetLastError());
   RCK(cudaMemcpyAsync(&m, d.dcount, sizeof(int32_t), cudaMemcpyDeviceToHost, d.st));
   RCK(cudaStreamSynchronize(d.st));
   eig.clear();
   if ( m == 0 ) return KINC_SIM_OK;
   const size_t need = (size_t)m * m;
   if ( need > d.capA )
   {
      cudaFree(d.dA);
      d.dA = nullptr;
      d.capA = 0;
      RCK(cudaMalloc(&d.dA, need * sizeof(double)));
      d.capA = need;
   }
   RCK(cudaMemsetAsync(d.dA, 0, need * sizeof(double), d.st));
   k_rmt_diag<<<(int)std::min<int64_t>((m + 255) / 256, 1024), 256, 0, d.st>>>(m, d.dA);
   if ( d.n > 0 )
      k_rmt_scatter<<<(int)std::min<int64_t>((d.n + 255) / 256, 4096), 256, 0, d.st>>>(
         d.n, d.K, m, d.dx, d.dy, d.dc, d.dr, t, d.drank, d.dA);
   RCK(cudaGetLastError());
   /* row-major with the lower triangle set = column-major with the upper triangle set */
   int lwork = 0;
   if ( cusolverDnDsyevd_bufferSize(d.solver, CUSOLVER_EIG_MODE_NOVECTOR, CUBLAS_FILL_MODE_UPPER, m, d.dA, m, d.dW,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS )
      return rmt_fail(KINC_SIM_ECUDA, "eigensolver workspace query failed for m = %d", m);
   if ( (size_t)lwork > d.capWork )
   {
      cudaFree(d.dwork);
      d.dwork = nullptr;
      d.capWork = 0;
      RCK(cudaMalloc(&d.dwork, (size_t)lwork * sizeof(double)));
      d.capWork = (size_t)lwork;
   }
   if ( cusolverDnDsyevd(d.solver, CUSOLVER_EIG_MODE_NOVECTOR, CUBLAS_FILL_MODE_UPPER, m, d.dA, m, d.dW, d.dwork,
                         lwork, d.dinfo) != CUSOLVER_STATUS_SUCCESS )
      return rmt_fail(KINC_SIM_ECUDA, "eigensolver failed for m = %d", m);
   std::vector<double> w((size_t)m);
   int32_t info = 0;
   RCK(cudaMemcpyAsync(w.data(), d.dW, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost, d.st));
   RCK(cudaMemcpyAsync(&info, d.dinfo, sizeof(int32_t), cudaMemcpyDeviceToHost, d.st));
   RCK(cudaStreamSynchronize(d.st));
   if ( info != 0 ) return rmt_fail(KINC_SIM_ECUDA, "eigensolver did not converge (info %d, m = %d)", info, m);
   /* GSL_EIGEN_SORT_ABS_ASC: ascending |lambda| (stable among equal magnitudes) */
   std::stable_sort(w.begin(), w.end(), [](double a, double b) { return std::fabs(a) < std::fabs(b); });
   eig.resize((size_t)m);
   for ( int32_t i = 0; i < m; ++i ) eig[(size_t)i] = (float)w[(size_t)i];
   return KINC_SIM_OK;
}

/* ----------------------------------------------------------------- host */

/* Akima spline through (x[i], y[i]), x strictly increasing, n >= 5 */
struct Akima
{
   std::vector<double> x, y, b, c, d;

   bool init(const double* xs, const double* ys, int n)
   {
      x.assign(xs, xs + n);
      y.assign(ys, ys + n);
      for ( int i = 0; i + 1 < n; ++i )
         if ( !(x[(size_t)i] < x[(size_t)i + 1]) ) return false;
      /* slopes m[-2 .. n] stored at m[j + 2] */
      std::vector<double> m((size_t)n + 3);
      for ( int i = 0; i + 1 < n; ++i )
         m[(size_t)i + 2] = (y[(size_t)i + 1] - y[(size_t)i]) / (x[(size_t)i + 1] - x[(size_t)i]);
      m[1] = 2.0 * m[2] - m[3];
      m[0] = 3.0 * m[2] - 2.0 * m[3];
      m[(size_t)n + 1] = 2.0 * m[(size_t)n] - m[(size_t)n - 1];
      m[(size_t)n + 2] = 3.0 * m[(size_t)n] - 2.0 * m[(size_t)n - 1];
      auto M = [&](int j) { return m[(size_t)(j + 2)]; };
      /* derivative at each knot: weights from the slope differences on either side */
      std::vector<double> tk((size_t)n);
      for ( int i = 0; i < n; ++i )
      {
         const double w1 = std::fabs(M(i + 1) - M(i));
         const double w2 = std::fabs(M(i - 1) - M(i - 2));
         const double ne = w1 + w2;
         if ( ne == 0.0 )
         {
            tk[(size_t)i] = 0.5 * (M(i - 1) + M(i));
         }
         else
         {
            const double alpha = w2 / ne;
            tk[(size_t)i] = (1.0 - alpha) * M(i - 1) + alpha * M(i);
         }
      }
      b.assign((size_t)n, 0.0);
      c.assign((size_t)n, 0.0);
      d.assign((size_t)n, 0.0);
      for ( int i = 0; i + 1 < n; ++i )
      {
         const double h = x[(size_t)i + 1] - x[(size_t)i];
         b[(size_t)i] = tk[(size_t)i];
         c[(size_t)i] = (3.0 * M(i) - 2.0 * tk[(size_t)i] - tk[(size_t)i + 1]) / h;
         d[(size_t)i] = (tk[(size_t)i] + tk[(size_t)i + 1] - 2.0 * M(i)) / (h * h);
      }
      return true;
   }

   double eval(double v) const
   {
      /* interval i with x[i] <= v < x[i+1]; v == x[n-1] takes the last interval */
      const int n = (int)x.size();
      int lo = 0, hi = n - 1;
      while ( hi - lo > 1 )
      {
         const int mid = (lo + hi) / 2;
         if ( x[(size_t)mid] > v ) hi = mid; else lo = mid;
      }
      const double dx = v - x[(size_t)lo];
      return y[(size_t)lo] + dx * (b[(size_t)lo] + dx * (c[(size_t)lo] + dx * d[(size_t)lo]));
   }
};

/* unique eigenvalues: skips the first, drops values within 1e-6 of the last kept (degenerate) */
std::vector<float> unique_eigens(const float* e, int n)
{
   const float EPSILON = 1e-6f;
   std::vector<float> u;
   for ( int i = 1; i < n; ++i )
      if ( u.empty() || std::fabs(e[i] - u.back()) > EPSILON ) u.push_back(e[i]);
   return u;
}

/* unfold: spacings of the spline-unfolded eigenvalues; false when the spline rejects the knots */
bool unfold(const std::vector<float>& e, int pace, std::vector<float>& spacings)
{
   const int n = (int)e.size();
   const int ns = n / pace;
   std::vector<double> x((size_t)ns), y((size_t)ns);
   for ( int i = 0; i < ns; ++i )
   {
      x[(size_t)i] = (double)e[(size_t)i * pace];
      y[(size_t)i] = (double)(i * pace + 1) / n;
   }
   x[(size_t)ns - 1] = e.back();
   y[(size_t)ns - 1] = 1.0;
   Akima s;
   if ( !s.init(x.data(), y.data(), ns) ) return false;
   std::vector<float> se((size_t)n);
   se[0] = 0.0f;
   se[(size_t)n - 1] = 1.0f;
   for ( int i = 1; i < n - 1; ++i )
   {
      const double v = (double)e[(size_t)i];
      if ( v < x.front() || v > x.back() ) return false;   /* outside the spline's range */
      se[(size_t)i] = (float)s.eval(v);
   }
   spacings.resize((size_t)n - 1);
   for ( int i = 0; i < n - 1; ++i ) spacings[(size_t)i] = (se[(size_t)i + 1] - se[(size_t)i]) * n;
   return true;
}

/* computePaceChiSquare: NNSD histogram on [0, 3) against the Poisson spacing law */
bool pace_chi(const std::vector<float>& e, int pace, int bins, float& chi)
{
   std::vector<float> sp;
   if ( !unfold(e, pace, sp) ) return false;
   const float hmin = 0.0f, hmax = 3.0f;
   const float w = (hmax - hmin) / bins;
   std::vector<float> hist((size_t)bins, 0.0f);
   for ( float s : sp )
   {
      if ( hmin <= s && s < hmax )
      {
         const int b = (int)((s - hmin) / w);
         if ( b < bins ) ++hist[(size_t)b];   /* a spacing just below 3 can round into bin `bins` */
      }
   }
   chi = 0.0f;
   const int n = (int)e.size();
   for ( int i = 0; i < bins; ++i )
   {
      const float O = hist[(size_t)i];
      const float E = (kinc_expf(-i * w) - kinc_expf(-(i + 1) * w)) * n;
      chi += (O - E) * (O - E) / E;
   }
   return true;
}

int chi_square(const float* eigens, int n, const kinc_rmt_params& p, float& chi)
{
   const std::vector<float> u = unique_eigens(eigens, n);
   if ( (int)u.size() < p.min_eigenvalue_size )
   {
      chi = -1.0f;
      return KINC_SIM_OK;
   }
   chi = 0.0f;
   int count = 0;
   for ( int pace = p.min_unfolding_pace; pace <= p.max_unfolding_pace; ++pace )
   {
      if ( (int)u.size() / pace < 5 ) break;
      float c = 0.0f;
      if ( !pace_chi(u, pace, p.histogram_bin_size, c) )
         return rmt_fail(KINC_RMT_ESPLINE, "unfolding at pace %d: eigenvalues not increasing in |lambda| order", pace);
      chi += c;
      ++count;
   }
   chi /= count;
   return KINC_SIM_OK;
}

int check_params(const kinc_rmt_params* p)
{
   if ( !p ) return rmt_fail(KINC_SIM_EINVAL, "no parameters");
   if ( p->threshold_start <= p->threshold_stop )
      return rmt_fail(KINC_SIM_EINVAL, "Starting threshold must be greater than stopping threshold.");
   if ( p->min_unfolding_pace >= p->max_unfolding_pace )
      return rmt_fail(KINC_SIM_EINVAL, "Minimum unfolding pace must be less than maximum unfolding pace.");
   if ( p->min_unfolding_pace < 1 || p->histogram_bin_size < 1 || !(p->threshold_step > 0.0f) )
      return rmt_fail(KINC_SIM_EINVAL, "An integer argument given is less than the minimum.");
   return KINC_SIM_OK;
}

}  // namespace

extern "C" void kinc_rmt_params_default(kinc_rmt_params* p)
{
   if ( !p ) return;
   p->threshold_start = 0.99f;
   p->threshold_step = 0.001f;
   p->threshold_stop = 0.5f;
   p->chi_square_threshold1 = 99.607f;
   p->chi_square_threshold2 = 200.0f;
   p->min_eigenvalue_size = 50;
   p->min_unfolding_pace = 10;
   p->max_unfolding_pace = 40;
   p->histogram_bin_size = 60;
}

extern "C" const char* kinc_rmt_last_error(void)
{
   return r_err.c_str();
}

extern "C" int kinc_rmt_chi_square(const float* eigens, int32_t n, const kinc_rmt_params* p, float* out_chi)
{
   if ( !out_chi || n < 0 || (n > 0 && !eigens) ) return rmt_fail(KINC_SIM_EINVAL, "invalid arguments");
   int rc = check_params(p);
   if ( rc ) return rc;
   return chi_square(eigens, n, *p, *out_chi);
}

extern "C" int kinc_rmt_prune_eigenvalues(int32_t genes, int32_t max_clusters, int64_t n, const int32_t* x,
                                          const int32_t* y, const int8_t* c, const float* r, float threshold,
                                          float* eigens, int32_t* size)
{
   if ( !eigens || !size ) return rmt_fail(KINC_SIM_EINVAL, "invalid arguments");
   RmtDevice d;
   int rc = device_setup(d, genes, max_clusters, n, x, y, c, r);
   if ( rc ) return rc;
   std::vector<float> e;
   int32_t m = 0;
   if ( (rc = device_eigenvalues(d, threshold, e, m)) ) return rc;
   std::copy(e.begin(), e.end(), eigens);
   *size = m;
   return KINC_SIM_OK;
}

extern "C" int kinc_rmt_run_items(int32_t genes, int32_t max_clusters, int64_t n, const int32_t* x, const int32_t* y,
                                  const int8_t* c, const float* r, const kinc_rmt_params* p, const char* log_path,
                                  float* out_threshold, float* steps_out, int32_t steps_cap, int32_t* steps)
{
   int rc = check_params(p);
   if ( rc ) return rc;
   if ( !out_threshold ) return rmt_fail(KINC_SIM_EINVAL, "out_threshold must not be NULL");
   RmtDevice d;
   if ( (rc = device_setup(d, genes, max_clusters, n, x, y, c, r)) ) return rc;
   FILE* log = nullptr;
   if ( log_path && !(log = fopen(log_path, "wb")) ) return rmt_fail(KINC_SIM_EINVAL, "cannot open %s", log_path);

   /* RMT::process: thresholds downwards until a large chi-square follows a small one */
   float finalThreshold = 0.0f;
   float finalChi = std::numeric_limits<float>::infinity();
   float maxChi = -std::numeric_limits<float>::infinity();
   float threshold = p->threshold_start;
   int32_t nsteps = 0;
   std::vector<float> eig;
   while ( maxChi < p->chi_square_threshold2 )
   {
      int32_t m = 0;
      if ( (rc = device_eigenvalues(d, threshold, eig, m)) ) break;
      float chi = -1.0f;
      if ( m > 0 && (rc = chi_square(eig.data(), m, *p, chi)) ) break;
      if ( chi != -1.0f )
      {
         if ( chi < p->chi_square_threshold1 )
         {
            finalChi = chi;
            finalThreshold = threshold;
         }
         if ( finalChi < p->chi_square_threshold1 && chi > finalChi ) maxChi = chi;
      }
      if ( log ) fprintf(log, "%.6g\t%d\t%.6g\n", (double)threshold, m, (double)chi);
      if ( steps_out && nsteps < steps_cap )
      {
         steps_out[3 * nsteps] = threshold;
         steps_out[3 * nsteps + 1] = (float)m;
         steps_out[3 * nsteps + 2] = chi;
      }
      ++nsteps;
      threshold -= p->threshold_step;
      if ( threshold < p->threshold_stop )
      {
         rc = rmt_fail(KINC_RMT_ENOTHRESHOLD, "Could not find non-random threshold above stopping threshold.");
         break;
      }
   }
   if ( log )
   {
      if ( rc == KINC_SIM_OK ) fprintf(log, "%.6g\n", (double)finalThreshold);
      fclose(log);
   }
   if ( steps ) *steps = nsteps;
   *out_threshold = finalThreshold;
   return rc;
}

extern "C" int kinc_rmt_run(const char* cmx_path, int32_t little_endian, const kinc_rmt_params* p, const char* log_path,
                            float* out_threshold)
{
   kinc_pm* m = nullptr;
   int32_t G = 0, K = 0, nc = 0;
   int64_t pairs = 0, n = 0;
   int rc = kinc_pm_open(cmx_path, KINC_PM_CMX, little_endian, &m, &G, &K, &nc, &pairs, &n);
   if ( rc ) return rmt_fail(rc, "%s", kinc_pm_last_error());
   std::vector<int32_t> x((size_t)std::max<int64_t>(n, 1)), y((size_t)std::max<int64_t>(n, 1));
   std::vector<int8_t> c((size_t)std::max<int64_t>(n, 1));
   std::vector<float> all((size_t)std::max<int64_t>(n, 1) * std::max(nc, 1)), r((size_t)std::max<int64_t>(n, 1));
   rc = n > 0 ? kinc_pm_read_items(m, 0, n, x.data(), y.data(), c.data(), all.data()) : KINC_SIM_OK;
   kinc_pm_close(m);
   if ( rc ) return rmt_fail(rc, "%s", kinc_pm_last_error());
   for ( int64_t i = 0; i < n; ++i ) r[(size_t)i] = all[(size_t)i * nc];   /* the first correlation */
   return kinc_rmt_run_items(G, K, n, x.data(), y.data(), c.data(), r.data(), p, log_path, out_threshold, nullptr, 0,
                             nullptr);
}
