/*
 * kinc_oracle.c -- TEST INFRASTRUCTURE ONLY: the CPU checker for the CUDA
 * Similarity path.  Never linked into the product.
 *
 * A plain-C restatement of KINC's serial Similarity worker and Pairwise::
 * models (paths relative to the KINC source tree):
 *   fetch-pair             src/core/similarity_serial.cpp:108-141
 *   serial block loop      src/core/similarity_serial.cpp:33-101
 *   clustering driver      src/core/pairwise_clustering.cpp:23-103
 *   Tukey outliers         src/core/pairwise_clustering.cpp:110-148
 *   BIC / ICL              src/core/pairwise_clustering.cpp:155-172
 *   GMM (2-D EM)           src/core/pairwise_gmm.cpp:11-445
 *   K-means                src/core/pairwise_kmeans.cpp:12-127
 *   Pearson                src/core/pairwise_pearson.cpp:12-52
 *   Spearman               src/core/pairwise_spearman.cpp:27-166
 *   process (CCM/CMX)      src/core/similarity.cpp:66-127
 *   2x2 linear algebra     src/core/pairwise_linalg.cpp:97-230
 *
 * Expression semantics follow the reference as compiled with the float
 * overloads of exp/log/sqrt/fabs (libstdc++ <math.h> style) and with no
 * floating-point contraction; double appears exactly where the reference's
 * expressions promote to double (M_PI, log of an int, 1.0/6.0 literals).
 * Float exp/log are kinc_expf/kinc_logf (kinc_fmath.h).  Build with
 * -ffp-contract=off.
 */
#define _GNU_SOURCE
#include "kinc_oracle.h"
#include "../kinc_gb300/csrc/kinc_fmath.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct { float s[2]; } v2;

/* ---------------------------------------------------------------- rand() */

void ko_rand_seed(ko_rand* g, uint32_t seed)
{
   int32_t r[34];
   int i;
   if ( seed == 0 )
   {
      seed = 1;
   }
   r[0] = (int32_t)seed;
   for ( i = 1; i < 31; ++i )
   {
      /* 16807 * r[i-1] mod (2^31 - 1) by Schrage's method */
      const int32_t hi = r[i - 1] / 127773;
      const int32_t lo = r[i - 1] % 127773;
      int32_t word = 16807 * lo - 2836 * hi;
      if ( word < 0 )
      {
         word += 2147483647;
      }
      r[i] = word;
   }
   for ( i = 31; i < 34; ++i )
   {
      r[i] = r[i - 31];
   }
   for ( i = 0; i < 34; ++i )
   {
      g->r[i] = (uint32_t)r[i];
   }
   g->head = 34;          /* absolute index of the next value to generate */
   g->drawn = 0;
   /* discard r[34..343] */
   for ( i = 34; i < 344; ++i )
   {
      const uint32_t v = g->r[(i - 31) % 34] + g->r[(i - 3) % 34];
      g->r[i % 34] = v;
   }
   g->head = 344;
}

int32_t ko_rand_next(ko_rand* g)
{
   /* head counts in absolute indices; the ring is indexed modulo 34 */
   const uint64_t i = (uint64_t)g->head + g->drawn;
   const uint32_t v = g->r[(i - 31) % 34] + g->r[(i - 3) % 34];
   g->r[i % 34] = v;
   g->drawn++;
   return (int32_t)(v >> 1);
}

void ko_rand_skip(ko_rand* g, uint64_t n)
{
   while ( n-- )
   {
      (void)ko_rand_next(g);
   }
}

void ko_libc_rand(uint32_t seed, int32_t n, int32_t* out)
{
   int32_t i;
   srand(seed);
   for ( i = 0; i < n; ++i )
   {
      out[i] = rand();
   }
}

/* POSIX example rand() with a 64-bit state (src/opencl/outlier.cl:14-18) */
static int32_t lcg_next(uint64_t* state)
{
   *state = (*state) * 1103515245ull + 12345ull;
   return (int32_t)((uint32_t)((*state) / 65536ull) % 32768u);
}

typedef struct
{
   int mode;
   ko_rand* g;
   uint64_t lcg;
} draw_src;

static int32_t draw(draw_src* d)
{
   return d->mode == 0 ? ko_rand_next(d->g) : lcg_next(&d->lcg);
}

int64_t ko_draws_per_pair(const ko_params* p)
{
   int64_t s = 0;
   int k;
   if ( p->clus_method == 0 || p->rand_mode != 0 )
   {
      return 0;
   }
   for ( k = p->min_clusters; k <= p->max_clusters; ++k )
   {
      s += k;
   }
   return p->clus_method == 2 ? 10 * s : s;
}

/* ------------------------------------------------------------- pair index */

void ko_pair_xy(int64_t index, int32_t* px, int32_t* py)
{
   /* src/core/pairwise_index.cpp:32-57 */
   int64_t x = 1;
   int64_t pos = 0;
   while ( pos <= index )
   {
      ++x;
      pos = x * (x - 1) / 2;
   }
   --x;
   pos = x * (x - 1) / 2;
   *px = (int32_t)x;
   *py = (int32_t)(index - pos);
}

static void pair_next(int32_t* x, int32_t* y)
{
   /* src/core/pairwise_index.cpp:85-94 */
   if ( ++(*y) >= *x )
   {
      *y = 0;
      ++(*x);
   }
}

/* ------------------------------------------------------------- fetch pair */

static int fetch_pair(const float* gem, int S, int x, int y, float minexpr, v2* X, int8_t* labels)
{
   const float* g1 = gem + (int64_t)x * S;
   const float* g2 = gem + (int64_t)y * S;
   int n = 0;
   int i;
   for ( i = 0; i < S; ++i )
   {
      if ( isnan(g1[i]) || isnan(g2[i]) )
      {
         labels[i] = -9;
      }
      else if ( g1[i] < minexpr || g2[i] < minexpr )
      {
         labels[i] = -6;
      }
      else
      {
         X[n].s[0] = g1[i];
         X[n].s[1] = g2[i];
         n++;
         labels[i] = 0;
      }
   }
   return n;
}

/* --------------------------------------------------------------- outliers */

static int cmp_float(const void* a, const void* b)
{
   const float fa = *(const float*)a;
   const float fb = *(const float*)b;
   return (fa > fb) - (fa < fb);
}

static void mark_outliers(const v2* X, int N, int j, int8_t* labels, int8_t cluster, int8_t marker,
                          float* work)
{
   int n = 0;
   int i;
   float Q1, Q3, T_min, T_max;
   for ( i = 0; i < N; i++ )
   {
      if ( labels[i] == cluster || labels[i] == marker )
      {
         work[n++] = X[i].s[j];
      }
   }
   if ( n == 0 )
   {
      return;
   }
   qsort(work, (size_t)n, sizeof(float), cmp_float);
   Q1 = work[n * 1 / 4];
   Q3 = work[n * 3 / 4];
   T_min = Q1 - 1.5f * (Q3 - Q1);
   T_max = Q3 + 1.5f * (Q3 - Q1);
   for ( i = 0; i < N; ++i )
   {
      if ( labels[i] == cluster && (X[i].s[j] < T_min || T_max < X[i].s[j]) )
      {
         labels[i] = marker;
      }
   }
}

/* -------------------------------------------------------------------- GMM */

typedef struct
{
   float pi;
   float mu[2];
   float sigma[4];
   float sinv[4];
   float norm;
} gcomp;


static int comp_prepare(gcomp* c, int opencl)
{
   /* matrixInverse (pairwise_linalg.cpp:163-173) then prepareCovariance (pairwise_gmm.cpp:31-47).
    * The CPU code fails on det <= 0; the OpenCL kernel's GMM_Component_prepareCovariance
    * (src/opencl/gmm.cl:46-64) only on fabs(det) <= 0, and goes on with the NaN normaliser of
    * a negative determinant. */
   const float det = c->sigma[0] * c->sigma[3] - c->sigma[1] * c->sigma[2];
   c->sinv[0] = +c->sigma[3] / det;
   c->sinv[1] = -c->sigma[1] / det;
   c->sinv[2] = -c->sigma[2] / det;
   c->sinv[3] = +c->sigma[0] / det;
   if ( opencl ? (fabsf(det) <= 0) : (det <= 0) )
   {
      return 0;
   }
   /* -0.5f * (D * log(2.0f * M_PI) + log(det)): the first log takes a double */
   c->norm = (float)(-0.5 * (2 * log(2.0f * M_PI) + (double)kinc_logf(det)));
   return 1;
}

typedef struct
{
   gcomp comp[64];
   float logpi[64];
   float logGamma[64];
   float* loggamma;   /* K * N */
} gmm_ws;

static int gmm_fit(const v2* X, int N, int K, int8_t* labels, float* out_logL, float* out_E,
                   draw_src* rnd, gmm_ws* w)
{
   int k, i, t;
   float prevLogL = -INFINITY;
   float currentLogL = -INFINITY;
   float* lg = w->loggamma;
   gcomp* C = w->comp;
   float* logpi = w->logpi;
   float* logGamma = w->logGamma;

   if ( rnd->mode == 1 )
   {
      rnd->lcg = 1;   /* src/opencl/gmm.cl:432 */
   }
   /* pairwise_gmm.cpp:370-380: random means, uniform pi, identity sigma */
   for ( k = 0; k < K; ++k )
   {
      const int ii = draw(rnd) % N;
      C[k].pi = 1.0f / K;
      C[k].mu[0] = X[ii].s[0];
      C[k].mu[1] = X[ii].s[1];
      C[k].sigma[0] = 1; C[k].sigma[1] = 0; C[k].sigma[2] = 0; C[k].sigma[3] = 1;
      C[k].sinv[0] = 0; C[k].sinv[1] = 0; C[k].sinv[2] = 0; C[k].sinv[3] = 0;
      C[k].norm = 0;
      comp_prepare(&C[k], rnd->mode == 1);
   }
   /* GMM::kmeans is a no-op: its loop condition `diff > TOLERANCE` starts with diff = 0
    * (pairwise_gmm.cpp:88-95) */
   for ( k = 0; k < K; ++k )
   {
      logpi[k] = kinc_logf(C[k].pi);
   }

   for ( t = 0; t < 100; ++t )
   {
      /* E step: calcLogMvNorm (pairwise_gmm.cpp:54-77,143-151) */
      for ( k = 0; k < K; ++k )
      {
         const gcomp* c = &C[k];
         for ( i = 0; i < N; ++i )
         {
            const float xm0 = X[i].s[0] - c->mu[0];
            const float xm1 = X[i].s[1] - c->mu[1];
            const float b0 = c->sinv[0] * xm0 + c->sinv[1] * xm1;
            const float b1 = c->sinv[2] * xm0 + c->sinv[3] * xm1;
            const float dot = xm0 * b0 + xm1 * b1;
            lg[k * N + i] = c->norm - 0.5f * dot;
         }
      }
      /* calcLogLikelihoodAndGammaNK (pairwise_gmm.cpp:158-187) */
      prevLogL = currentLogL;
      {
         float logL = 0.0f;
         for ( i = 0; i < N; ++i )
         {
            float maxArg = -INFINITY;
            float sum = 0.0f;
            float logpx;
            for ( k = 0; k < K; ++k )
            {
               const float lp = logpi[k] + lg[k * N + i];
               if ( lp > maxArg )
               {
                  maxArg = lp;
               }
            }
            for ( k = 0; k < K; ++k )
            {
               const float lp = logpi[k] + lg[k * N + i];
               sum += kinc_expf(lp - maxArg);
            }
            logpx = maxArg + kinc_logf(sum);
            logL += logpx;
            for ( k = 0; k < K; ++k )
            {
               lg[k * N + i] += -logpx;
            }
         }
         currentLogL = logL;
      }
      if ( fabsf(currentLogL - prevLogL) < 1e-8f )
      {
         break;
      }
      /* calcLogGammaK (pairwise_gmm.cpp:194-221) */
      for ( k = 0; k < K; ++k )
      {
         float maxArg = -INFINITY;
         float sum = 0;
         for ( i = 0; i < N; ++i )
         {
            if ( lg[k * N + i] > maxArg )
            {
               maxArg = lg[k * N + i];
            }
         }
         for ( i = 0; i < N; ++i )
         {
            sum += kinc_expf(lg[k * N + i] - maxArg);
         }
         logGamma[k] = maxArg + kinc_logf(sum);
      }
      /* calcLogGammaSum (pairwise_gmm.cpp:228-248) + performMStep (pairwise_gmm.cpp:255-316) */
      {
         float maxArg = -INFINITY;
         float sum = 0;
         float logGammaSum;
         for ( k = 0; k < K; ++k )
         {
            const float arg = logpi[k] + logGamma[k];
            if ( arg > maxArg )
            {
               maxArg = arg;
            }
         }
         for ( k = 0; k < K; ++k )
         {
            const float arg = logpi[k] + logGamma[k];
            sum += kinc_expf(arg - maxArg);
         }
         logGammaSum = maxArg + kinc_logf(sum);

         for ( k = 0; k < K; ++k )
         {
            logpi[k] += logGamma[k] - logGammaSum;
            C[k].pi = kinc_expf(logpi[k]);
         }
      }
      for ( k = 0; k < K * N; ++k )
      {
         lg[k] = kinc_expf(lg[k]);
      }
      for ( k = 0; k < K; ++k )
      {
         logGamma[k] = kinc_expf(logGamma[k]);
      }
      for ( k = 0; k < K; ++k )
      {
         gcomp* c = &C[k];
         float sc;
         c->mu[0] = 0;
         c->mu[1] = 0;
         for ( i = 0; i < N; ++i )
         {
            c->mu[0] += lg[k * N + i] * X[i].s[0];
            c->mu[1] += lg[k * N + i] * X[i].s[1];
         }
         sc = 1.0f / logGamma[k];
         c->mu[0] *= sc;
         c->mu[1] *= sc;

         c->sigma[0] = 0; c->sigma[1] = 0; c->sigma[2] = 0; c->sigma[3] = 0;
         for ( i = 0; i < N; ++i )
         {
            const float xm0 = X[i].s[0] - c->mu[0];
            const float xm1 = X[i].s[1] - c->mu[1];
            const float o00 = xm0 * xm0;
            const float o01 = xm0 * xm1;
            const float o10 = xm1 * xm0;
            const float o11 = xm1 * xm1;
            const float g = lg[k * N + i];
            c->sigma[0] += g * o00;
            c->sigma[1] += g * o01;
            c->sigma[2] += g * o10;
            c->sigma[3] += g * o11;
         }
         sc = 1.0f / logGamma[k];
         c->sigma[0] *= sc; c->sigma[1] *= sc; c->sigma[2] *= sc; c->sigma[3] *= sc;
         if ( !comp_prepare(c, rnd->mode == 1) )
         {
            return 0;   /* prepareCovariance throws; fit() reports failure */
         }
      }
   }

   *out_logL = currentLogL;
   /* calcLabels (pairwise_gmm.cpp:323-341) */
   for ( i = 0; i < N; ++i )
   {
      int max_k = -1;
      float max_gamma = -INFINITY;
      for ( k = 0; k < K; ++k )
      {
         if ( max_gamma < lg[k * N + i] )
         {
            max_k = k;
            max_gamma = lg[k * N + i];
         }
      }
      labels[i] = (int8_t)max_k;
   }
   /* calcEntropy (pairwise_gmm.cpp:348-360).  A label of -1 (every value NaN)
    * indexes before the array in the reference; that only happens when logL is
    * NaN, so the fit is never selected and the value does not matter. */
   {
      float E = 0;
      for ( i = 0; i < N; ++i )
      {
         const int kk = labels[i];
         E += kk >= 0 ? kinc_logf(lg[kk * N + i]) : NAN;
      }
      *out_E = E;
   }
   return 1;
}

/* ---------------------------------------------------------------- K-means */

static float diff_norm(const v2* a, const float* b)
{
   /* vectorDiffNorm (pairwise_linalg.cpp:97-104) */
   float dist = 0;
   dist += (a->s[0] - b[0]) * (a->s[0] - b[0]);
   dist += (a->s[1] - b[1]) * (a->s[1] - b[1]);
   return sqrtf(dist);
}

static int kmeans_fit(const v2* X, int N, int K, int8_t* labels, float* out_logL, draw_src* rnd,
                      int8_t* y, int8_t* y_next)
{
   int init, k, i, t;
   float means[64][2];
   float bestLogL = -INFINITY;

   if ( rnd->mode == 1 )
   {
      rnd->lcg = 1;
   }
   for ( init = 0; init < 10; ++init )
   {
      int8_t* ya = y;
      int8_t* yb = y_next;
      float S = 0;
      float logL;
      for ( k = 0; k < K; ++k )
      {
         const int ii = draw(rnd) % N;
         means[k][0] = X[ii].s[0];
         means[k][1] = X[ii].s[1];
      }
      memset(ya, 0, (size_t)N);
      memset(yb, 0, (size_t)N);
      for ( t = 0; t < 300; ++t )
      {
         int same = 1;
         for ( i = 0; i < N; ++i )
         {
            int min_k = -1;
            float min_dist = 0;
            for ( k = 0; k < K; ++k )
            {
               const float dist = diff_norm(&X[i], means[k]);
               if ( min_k == -1 || dist < min_dist )
               {
                  min_k = k;
                  min_dist = dist;
               }
            }
            yb[i] = (int8_t)min_k;
            same &= (yb[i] == ya[i]);
         }
         if ( same )
         {
            break;
         }
         {
            int8_t* tmp = ya;
            ya = yb;
            yb = tmp;
         }
         for ( k = 0; k < K; ++k )
         {
            int n_k = 0;
            float sc;
            means[k][0] = 0;
            means[k][1] = 0;
            for ( i = 0; i < N; ++i )
            {
               if ( ya[i] == k )
               {
                  means[k][0] += X[i].s[0];
                  means[k][1] += X[i].s[1];
                  n_k++;
               }
            }
            sc = 1.0f / n_k;
            means[k][0] *= sc;
            means[k][1] *= sc;
         }
      }
      /* computeLogLikelihood (pairwise_kmeans.cpp:106-127) */
      for ( k = 0; k < K; ++k )
      {
         for ( i = 0; i < N; ++i )
         {
            float dist;
            if ( ya[i] != k )
            {
               continue;
            }
            dist = diff_norm(&X[i], means[k]);
            S += dist * dist;
         }
      }
      logL = -S;
      if ( bestLogL < logL )
      {
         bestLogL = logL;
         memcpy(labels, ya, (size_t)N);
      }
   }
   *out_logL = bestLogL;
   return 1;
}

/* ------------------------------------------------------------- clustering */

typedef struct
{
   v2* X;             /* S entries, kept for a whole block (stale tail) */
   int8_t* labels;    /* S */
   int8_t* work;      /* S: the model's work labels */
   int8_t* y;
   int8_t* y_next;
   float* fwork;      /* max(S, pow2) floats */
   float* sx;
   float* sy;
   float* srank;
   gmm_ws gmm;
} pair_ws;

static float criterion_value(const ko_params* p, int K, float logL, int N, float E)
{
   /* computeBIC / computeICL (pairwise_clustering.cpp:155-172): log(N) of an int is
    * double, 2*logL stays float, the difference is double, the return is float.
    * The OpenCL worker's GMM (rand_mode 1) evaluates them in float, with log of (float)N
    * (GMM_computeBIC / GMM_computeICL, src/opencl/gmm.cl:511-530). */
   const int D = 2;
   const int pp = K * (1 + D + D * D);
   if ( p->rand_mode == 1 && p->clus_method == 1 )
   {
      float v = kinc_logf((float)N) * (float)pp - 2.0f * logL;
      if ( p->criterion == 1 ) v = v - 2.0f * E;
      return v;
   }
   if ( p->criterion == 0 )
   {
      return (float)(log((double)N) * pp - (double)(2 * logL));
   }
   return (float)(log((double)N) * pp - (double)(2 * logL) - (double)(2 * E));
}

static int cluster_pair(const ko_params* p, pair_ws* w, int N, draw_src* rnd)
{
   /* Clustering::compute (pairwise_clustering.cpp:23-103) */
   int8_t* labels = w->labels;
   int bestK = 0;
   if ( p->pre_out )
   {
      mark_outliers(w->X, N, 0, labels, 0, -7, w->fwork);
      mark_outliers(w->X, N, 1, labels, 0, -7, w->fwork);
   }
   if ( N >= p->min_samples )
   {
      float bestValue = INFINITY;
      int K;
      for ( K = p->min_clusters; K <= p->max_clusters; ++K )
      {
         float logL = 0, E = 0, value;
         int ok;
         if ( p->clus_method == 1 )
         {
            ok = gmm_fit(w->X, N, K, w->work, &logL, &E, rnd, &w->gmm);
         }
         else
         {
            ok = kmeans_fit(w->X, N, K, w->work, &logL, rnd, w->y, w->y_next);
            E = 0;
         }
         if ( !ok )
         {
            continue;
         }
         value = criterion_value(p, K, logL, N, E);
         if ( value < bestValue )
         {
            int i, j;
            bestK = K;
            bestValue = value;
            for ( i = 0, j = 0; i < N; ++i )
            {
               if ( labels[i] >= 0 )
               {
                  labels[i] = w->work[j];
                  ++j;
               }
            }
         }
      }
   }
   if ( bestK > 1 && p->post_out )
   {
      int k;
      for ( k = 0; k < bestK; ++k )
      {
         mark_outliers(w->X, N, 0, labels, (int8_t)k, -8, w->fwork);
         mark_outliers(w->X, N, 1, labels, (int8_t)k, -8, w->fwork);
      }
   }
   return bestK;
}

/* ------------------------------------------------------------ correlation */

static float pearson_cluster(const ko_params* p, const pair_ws* w, const float* g1, const float* g2,
                             int S, int8_t cluster)
{
   /* Pearson::computeCluster (pairwise_pearson.cpp:12-52).  The reference reads
    * the packed X at the sample position i; semantics 1 reads sample i itself. */
   int n = 0;
   float sumx = 0, sumy = 0, sumx2 = 0, sumy2 = 0, sumxy = 0;
   int i;
   for ( i = 0; i < S; ++i )
   {
      if ( w->labels[i] == cluster )
      {
         const float x_i = p->semantics == 0 ? w->X[i].s[0] : g1[i];
         const float y_i = p->semantics == 0 ? w->X[i].s[1] : g2[i];
         sumx += x_i;
         sumy += y_i;
         sumx2 += x_i * x_i;
         sumy2 += y_i * y_i;
         sumxy += x_i * y_i;
         ++n;
      }
   }
   if ( n >= p->min_samples )
   {
      return (n * sumxy - sumx * sumy) / sqrtf((n * sumx2 - sumx * sumx) * (n * sumy2 - sumy * sumy));
   }
   return NAN;
}

static int next_pow2(int n)
{
   int pow2 = 2;
   while ( pow2 < n )
   {
      pow2 *= 2;
   }
   return pow2;
}

static void bitonic_sort(int size, float* sortList, float* extraList)
{
   /* Spearman::bitonicSort (pairwise_spearman.cpp:109-134) */
   const int bsize = size / 2;
   int ob, ib, i;
   for ( ob = 2; ob <= size; ob *= 2 )
   {
      for ( ib = ob; ib >= 2; ib /= 2 )
      {
         const int t = ib / 2;
         for ( i = 0; i < bsize; ++i )
         {
            const int dir = -((i / (ob / 2)) & 0x1);
            const int a = (i / t) * ib + (i % t);
            const int b = a + t;
            if ( ((sortList[a] > sortList[b]) && !dir) || ((sortList[a] < sortList[b]) && dir) )
            {
               float tmp = sortList[a];
               sortList[a] = sortList[b];
               sortList[b] = tmp;
               tmp = extraList[a];
               extraList[a] = extraList[b];
               extraList[b] = tmp;
            }
         }
      }
   }
}

static float spearman_cluster(const ko_params* p, pair_ws* w, const float* g1, const float* g2, int S,
                              int8_t cluster)
{
   /* Spearman::computeCluster (pairwise_spearman.cpp:27-86) */
   const int N_pow2 = next_pow2(S);
   int n = 0;
   int i, j;
   for ( i = 0, j = 0; i < S; ++i )
   {
      if ( p->semantics == 0 )
      {
         if ( w->labels[i] >= 0 )
         {
            if ( w->labels[i] == cluster )
            {
               w->sx[n] = w->X[j].s[0];
               w->sy[n] = w->X[j].s[1];
               w->srank[n] = (float)(n + 1);
               ++n;
            }
            ++j;
         }
      }
      else if ( w->labels[i] == cluster )
      {
         w->sx[n] = g1[i];
         w->sy[n] = g2[i];
         w->srank[n] = (float)(n + 1);
         ++n;
      }
   }
   for ( i = n; i < N_pow2; ++i )
   {
      w->sx[i] = INFINITY;
      w->sy[i] = INFINITY;
      w->srank[i] = 0;
   }
   if ( n >= p->min_samples )
   {
      const int n_pow2 = next_pow2(n);
      uint32_t diff = 0;
      int32_t denom;
      bitonic_sort(n_pow2, w->sx, w->sy);
      bitonic_sort(n_pow2, w->sy, w->srank);
      for ( i = 0; i < n; ++i )
      {
         const int tmp = (int)((float)(i + 1) - w->srank[i]);
         diff += (uint32_t)(tmp * tmp);    /* int arithmetic; wraps like the reference */
      }
      denom = (int32_t)((uint32_t)n * ((uint32_t)n * (uint32_t)n - 1u));
      return (float)(1.0 - 6.0 * (double)(int32_t)diff / (double)denom);
   }
   return NAN;
}

/* ------------------------------------------------------------- block loop */

static void ws_alloc(pair_ws* w, int S, int maxK)
{
   const int P2 = next_pow2(S);
   w->X = (v2*)calloc((size_t)S, sizeof(v2));
   w->labels = (int8_t*)calloc((size_t)S, 1);
   w->work = (int8_t*)calloc((size_t)S, 1);
   w->y = (int8_t*)calloc((size_t)S, 1);
   w->y_next = (int8_t*)calloc((size_t)S, 1);
   w->fwork = (float*)calloc((size_t)(P2 > S ? P2 : S), sizeof(float));
   w->sx = (float*)calloc((size_t)P2, sizeof(float));
   w->sy = (float*)calloc((size_t)P2, sizeof(float));
   w->srank = (float*)calloc((size_t)P2, sizeof(float));
   w->gmm.loggamma = (float*)calloc((size_t)maxK * (size_t)S, sizeof(float));
}

static void ws_free(pair_ws* w)
{
   free(w->X); free(w->labels); free(w->work); free(w->y); free(w->y_next);
   free(w->fwork); free(w->sx); free(w->sy); free(w->srank); free(w->gmm.loggamma);
}

int ko_run_block(const float* gem, int32_t G, int32_t S, const ko_params* p, ko_rand* rng,
                 int64_t start, int64_t size,
                 int8_t* out_K, int8_t* out_labels, float* out_corr, int32_t* out_N)
{
   pair_ws w;
   int32_t x, y;
   int64_t q;
   const int maxK = p->max_clusters;
   draw_src rnd;

   if ( size <= 0 )
   {
      return 0;
   }
   if ( p->min_clusters < 1 || p->max_clusters > 64 || p->max_clusters < p->min_clusters
        || p->min_samples < 1 || S < 1 || G < 2 )
   {
      return -1;
   }
   rnd.mode = p->rand_mode;
   rnd.g = rng;
   rnd.lcg = 1;
   ws_alloc(&w, S, maxK);
   (void)G;
   /* Serial::execute allocates X once per 32768-pair work block; when `start`
    * is inside a block, replay the fetches of the block's earlier pairs so
    * the packed array holds what the reference would have left in it. */
   ko_pair_xy((start / 32768) * 32768, &x, &y);
   for ( q = (start / 32768) * 32768; q < start; ++q )
   {
      fetch_pair(gem, S, x, y, p->min_expr, w.X, w.labels);
      pair_next(&x, &y);
   }

   for ( q = 0; q < size; ++q )
   {
      const float* g1 = gem + (int64_t)x * S;
      const float* g2 = gem + (int64_t)y * S;
      int N;
      if ( q > 0 && (start + q) % 32768 == 0 )
      {
         /* a new work block: Serial::execute starts from fresh zeroed arrays */
         memset(w.X, 0, (size_t)S * sizeof(v2));
         memset(w.labels, 0, (size_t)S);
      }
      N = fetch_pair(gem, S, x, y, p->min_expr, w.X, w.labels);
      int K = 1;
      int k;
      if ( p->clus_method != 0 )
      {
         K = cluster_pair(p, &w, N, &rnd);
      }
      if ( out_corr && p->corr_method == 2 )
      {
         /* both methods of one clustering, [k][0] Pearson and [k][1] Spearman: what two KINC runs
          * with the same arguments and the two --corrmethod values give (the worker computes both
          * in one pass) */
         for ( k = 0; k < maxK; ++k )
         {
            float rp = NAN, rs = NAN;
            if ( k < K )
            {
               rp = pearson_cluster(p, &w, g1, g2, S, (int8_t)k);
               rs = spearman_cluster(p, &w, g1, g2, S, (int8_t)k);
            }
            out_corr[(q * maxK + k) * 2] = rp;
            out_corr[(q * maxK + k) * 2 + 1] = rs;
         }
      }
      else if ( out_corr )
      {
         for ( k = 0; k < maxK; ++k )
         {
            float r = NAN;
            if ( k < K )
            {
               r = p->corr_method == 0 ? pearson_cluster(p, &w, g1, g2, S, (int8_t)k)
                                       : spearman_cluster(p, &w, g1, g2, S, (int8_t)k);
            }
            out_corr[q * maxK + k] = r;
         }
      }
      if ( out_K )
      {
         out_K[q] = (int8_t)K;
      }
      if ( out_labels )
      {
         memcpy(out_labels + q * S, w.labels, (size_t)S);
      }
      if ( out_N )
      {
         out_N[q] = N;
      }
      pair_next(&x, &y);
   }
   ws_free(&w);
   return 0;
}

/* ------------------------------------------------------ qualifying counts */

int64_t ko_count_qualifying(const float* gem, int32_t G, int32_t S, const ko_params* p, int64_t end)
{
   const int W = (S + 31) / 32;
   uint32_t* mask = (uint32_t*)calloc((size_t)G * W, sizeof(uint32_t));
   int64_t count = 0;
   int32_t x, y, i;
   int64_t q;
   for ( x = 0; x < G; ++x )
   {
      for ( i = 0; i < S; ++i )
      {
         const float v = gem[(int64_t)x * S + i];
         if ( !isnan(v) && !(v < p->min_expr) )
         {
            mask[(int64_t)x * W + i / 32] |= 1u << (i % 32);
         }
      }
   }
   x = 1;
   y = 0;
   for ( q = 0; q < end; ++q )
   {
      int n = 0;
      int w;
      for ( w = 0; w < W; ++w )
      {
         n += __builtin_popcount(mask[(int64_t)x * W + w] & mask[(int64_t)y * W + w]);
      }
      count += (n >= p->min_samples);
      pair_next(&x, &y);
   }
   free(mask);
   return count;
}

/* --------------------------------------------------------------- parallel */

typedef struct
{
   const float* gem;
   int32_t G, S;
   const ko_params* p;
   const int64_t* starts;
   const int64_t* sizes;
   const uint64_t* rand_pos;
   int8_t* out_K;
   int8_t* out_labels;
   float* out_corr;
   const int64_t* out_off;
   int32_t nseg;
   int32_t next;
   pthread_mutex_t lock;
   pthread_barrier_t barrier;
   int64_t done;
} par_state;

typedef struct
{
   par_state* st;
   int32_t tid;
   int32_t nthreads;
} par_arg;

static void* par_worker(void* argp)
{
   par_arg* a = (par_arg*)argp;
   par_state* st = a->st;
   int32_t s;
   /* position one rand() stream per segment owned by this thread before timing starts */
   int32_t mine = 0;
   ko_rand* rngs = (ko_rand*)calloc((size_t)st->nseg, sizeof(ko_rand));
   for ( s = a->tid; s < st->nseg; s += a->nthreads )
   {
      ko_rand_seed(&rngs[s], 1);
      ko_rand_skip(&rngs[s], st->rand_pos ? st->rand_pos[s] : 0);
      ++mine;
   }
   pthread_barrier_wait(&st->barrier);
   for ( s = a->tid; s < st->nseg; s += a->nthreads )
   {
      const int64_t o = st->out_off ? st->out_off[s] : 0;
      ko_run_block(st->gem, st->G, st->S, st->p, &rngs[s], st->starts[s], st->sizes[s],
                   st->out_K ? st->out_K + o : NULL,
                   st->out_labels ? st->out_labels + o * st->S : NULL,
                   st->out_corr ? st->out_corr + o * st->p->max_clusters * (st->p->corr_method == 2 ? 2 : 1)
                                : NULL, NULL);
      pthread_mutex_lock(&st->lock);
      st->done += st->sizes[s];
      pthread_mutex_unlock(&st->lock);
   }
   (void)mine;
   free(rngs);
   return NULL;
}

int64_t ko_run_segments_parallel_out(const float* gem, int32_t G, int32_t S, const ko_params* p,
                                     const int64_t* starts, const int64_t* sizes, const uint64_t* rand_pos,
                                     int32_t nseg, int32_t threads, double* seconds,
                                     int8_t* out_K, int8_t* out_labels, float* out_corr)
{
   par_state st;
   pthread_t* th;
   par_arg* args;
   int32_t t;
   struct timespec t0, t1;
   int64_t* offs = NULL;
   if ( threads < 1 )
   {
      threads = 1;
   }
   if ( out_K || out_labels || out_corr )
   {
      int32_t s;
      offs = (int64_t*)calloc((size_t)nseg + 1, sizeof(int64_t));
      for ( s = 0; s < nseg; ++s )
      {
         offs[s + 1] = offs[s] + sizes[s];
      }
   }
   st.gem = gem; st.G = G; st.S = S; st.p = p; st.starts = starts; st.sizes = sizes;
   st.rand_pos = rand_pos; st.nseg = nseg; st.next = 0; st.done = 0;
   st.out_K = out_K; st.out_labels = out_labels; st.out_corr = out_corr; st.out_off = offs;
   pthread_mutex_init(&st.lock, NULL);
   pthread_barrier_init(&st.barrier, NULL, (unsigned)threads + 1);
   th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
   args = (par_arg*)calloc((size_t)threads, sizeof(par_arg));
   for ( t = 0; t < threads; ++t )
   {
      args[t].st = &st;
      args[t].tid = t;
      args[t].nthreads = threads;
      pthread_create(&th[t], NULL, par_worker, &args[t]);
   }
   pthread_barrier_wait(&st.barrier);
   clock_gettime(CLOCK_MONOTONIC, &t0);
   for ( t = 0; t < threads; ++t )
   {
      pthread_join(th[t], NULL);
   }
   clock_gettime(CLOCK_MONOTONIC, &t1);
   if ( seconds )
   {
      *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
   }
   pthread_barrier_destroy(&st.barrier);
   pthread_mutex_destroy(&st.lock);
   free(th);
   free(args);
   free(offs);
   return st.done;
}

int64_t ko_run_segments_parallel(const float* gem, int32_t G, int32_t S, const ko_params* p,
                                 const int64_t* starts, const int64_t* sizes, const uint64_t* rand_pos,
                                 int32_t nseg, int32_t threads, double* seconds)
{
   return ko_run_segments_parallel_out(gem, G, S, p, starts, sizes, rand_pos, nseg, threads, seconds, NULL, NULL,
                                       NULL);
}

int64_t ko_run_blocks_parallel(const float* gem, int32_t G, int32_t S, const ko_params* p,
                               const int64_t* blocks, int32_t nblocks, int32_t threads)
{
   int64_t* starts = (int64_t*)calloc((size_t)nblocks, sizeof(int64_t));
   int64_t* sizes = (int64_t*)calloc((size_t)nblocks, sizeof(int64_t));
   const int64_t total = (int64_t)G * (G - 1) / 2;
   int64_t done;
   int32_t b;
   for ( b = 0; b < nblocks; ++b )
   {
      starts[b] = blocks[b] * 32768;
      sizes[b] = total - starts[b] < 32768 ? total - starts[b] : 32768;
   }
   done = ko_run_segments_parallel(gem, G, S, p, starts, sizes, NULL, nblocks, threads, NULL);
   free(starts);
   free(sizes);
   return done;
}

/* ---------------------------------------------------------------- process */

int64_t ko_process_block(int32_t S, const ko_params* p, int64_t start, int64_t size,
                         const int8_t* K, const int8_t* labels, const float* corr,
                         int32_t* cmx_x, int32_t* cmx_y, int8_t* cmx_c, float* cmx_r,
                         int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c, int8_t* ccm_codes,
                         int64_t* n_ccm)
{
   int64_t q, ncmx = 0, nccm = 0;
   int32_t x, y;
   const int maxK = p->max_clusters;
   ko_pair_xy(start, &x, &y);
   for ( q = 0; q < size; ++q )
   {
      const int Kq = K[q];
      int k, i;
      if ( Kq > 1 )
      {
         int c = 0;
         for ( k = 0; k < Kq; ++k )
         {
            const float r = corr[q * maxK + k];
            if ( !isnan(r) && p->min_corr <= fabsf(r) && fabsf(r) <= p->max_corr )
            {
               ccm_x[nccm] = x;
               ccm_y[nccm] = y;
               ccm_c[nccm] = (int8_t)c++;
               for ( i = 0; i < S; ++i )
               {
                  const int8_t l = labels[q * S + i];
                  ccm_codes[nccm * S + i] = (int8_t)(l >= 0 ? (k == l) : -l);
               }
               ++nccm;
            }
         }
      }
      if ( Kq > 0 )
      {
         int c = 0;
         for ( k = 0; k < Kq; ++k )
         {
            const float r = corr[q * maxK + k];
            if ( !isnan(r) && p->min_corr <= fabsf(r) && fabsf(r) <= p->max_corr )
            {
               cmx_x[ncmx] = x;
               cmx_y[ncmx] = y;
               cmx_c[ncmx] = (int8_t)c++;
               cmx_r[ncmx] = r;
               ++ncmx;
            }
         }
      }
      pair_next(&x, &y);
   }
   if ( n_ccm )
   {
      *n_ccm = nccm;
   }
   return ncmx;
}

/* ------------------------------------------------------------------- FP64 */

double ko_pearson_fp64(const float* gem, int32_t S, int32_t x, int32_t y, float min_expr,
                       int32_t min_samples)
{
   const float* g1 = gem + (int64_t)x * S;
   const float* g2 = gem + (int64_t)y * S;
   double mx = 0, my = 0, sxy = 0, sxx = 0, syy = 0;
   int n = 0, i;
   for ( i = 0; i < S; ++i )
   {
      if ( isnan(g1[i]) || isnan(g2[i]) || g1[i] < min_expr || g2[i] < min_expr )
      {
         continue;
      }
      mx += g1[i];
      my += g2[i];
      ++n;
   }
   if ( n < min_samples || n == 0 )
   {
      return NAN;
   }
   mx /= n;
   my /= n;
   for ( i = 0; i < S; ++i )
   {
      double dx, dy;
      if ( isnan(g1[i]) || isnan(g2[i]) || g1[i] < min_expr || g2[i] < min_expr )
      {
         continue;
      }
      dx = g1[i] - mx;
      dy = g2[i] - my;
      sxy += dx * dy;
      sxx += dx * dx;
      syy += dy * dy;
   }
   return sxy / sqrt(sxx * syy);
}

typedef struct
{
   const float* gem;
   int32_t S;
   const int32_t* xs;
   const int32_t* ys;
   int64_t lo, hi;
   float min_expr;
   int32_t min_samples;
   double* out;
} fp64_job;

static void* fp64_worker(void* p)
{
   fp64_job* j = (fp64_job*)p;
   int64_t i;
   for ( i = j->lo; i < j->hi; ++i )
   {
      j->out[i] = ko_pearson_fp64(j->gem, j->S, j->xs[i], j->ys[i], j->min_expr, j->min_samples);
   }
   return NULL;
}

void ko_pearson_fp64_batch(const float* gem, int32_t S, const int32_t* xs, const int32_t* ys, int64_t n,
                           float min_expr, int32_t min_samples, double* out, int32_t threads)
{
   pthread_t th[256];
   fp64_job jobs[256];
   int32_t t;
   if ( threads < 1 ) threads = 1;
   if ( threads > 256 ) threads = 256;
   for ( t = 0; t < threads; ++t )
   {
      jobs[t].gem = gem; jobs[t].S = S; jobs[t].xs = xs; jobs[t].ys = ys;
      jobs[t].lo = n * t / threads; jobs[t].hi = n * (t + 1) / threads;
      jobs[t].min_expr = min_expr; jobs[t].min_samples = min_samples; jobs[t].out = out;
      pthread_create(&th[t], NULL, fp64_worker, &jobs[t]);
   }
   for ( t = 0; t < threads; ++t )
   {
      pthread_join(th[t], NULL);
   }
}
