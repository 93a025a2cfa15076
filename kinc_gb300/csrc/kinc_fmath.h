/*
 * kinc_fmath.h -- portable single-precision exp and log, bit-identical on the
 * host (C/C++) and on the GPU (CUDA).
 *
 * Why these exist.  The reference's clustering code calls unqualified exp()
 * and log() on float arguments (src/core/pairwise_gmm.cpp:177,219,262,271,356
 * and the convergence/entropy paths).  Which function that resolves to --
 * glibc expf, glibc exp(double) rounded to float, or something else -- is
 * decided by the headers the reference happens to be built with, and the
 * EM trajectory (100 iterations of sequential float sums) is sensitive to the
 * last bit of every call.  To make "the reference's results" a defined thing,
 * the oracle, the compiled reference sources and the CUDA kernels all route
 * float exp/log through the two functions below, which use only IEEE-754
 * binary32 add/sub/mul/div and fused multiply-add.  Those operations are
 * correctly rounded on every conforming host and on the GPU, so the results
 * are identical everywhere as long as callers do not let the compiler contract
 * a*b+c on their own (host: -ffp-contract=off; device: --fmad=false).
 *
 * Methods (written from the mathematics, not from any vendor library):
 *   exp:  n = rint(x/ln2) by the 1.5*2^23 shifter (one fused multiply-add,
 *         whose sum also holds n in its low mantissa bits); Cody-Waite
 *         argument reduction x = n*ln2 + r with a two-part ln2 whose leading
 *         part has 16 significant bits (so n*LN2_HI and x - n*LN2_HI are
 *         exact for |n| <= 2^8), |r| <= ln2/2; then
 *         e^r ~ 1 + r + r^2 (c2 + c3 r + ... + c6 r^4), the coefficients a
 *         minimax fit of the relative error on [-ln2/2, ln2/2] found with
 *         the Remez exchange algorithm (max relative error 4.3e-9 before
 *         rounding), evaluated by Horner's rule in fused multiply-adds; then
 *         scaling by 2^n with one integer add of n to the exponent field
 *         when the result is a normal float, in two steps otherwise.
 *         Max error 0.92 ulp over every float input with a normal result;
 *         99.52 % of results are correctly rounded.
 *   log:  the table-driven method of P. T. P. Tang (ACM TOMS 16(4), 1990)
 *         in single precision: x = 2^e * m with m in [0.703125, 1.40625),
 *         the reduction offset chosen so that 1.0 starts one of 32 equal
 *         steps of the mantissa bits; entry i holds c_i = 1/invc_i with invc_i
 *         a multiple of 1/64 (1 on the two steps around 1), and
 *         log(c_i) = hi_i + lo_i with hi_i a multiple of 2^-16.  Then
 *         z = m * invc_i - 1 is exact (|z| < 2^-5 and a multiple of 2^-30),
 *         e*LN2_HI + hi_i is exact, that sum plus z is carried as a
 *         two-float sum, and log1p(z) = z + z^2 (-1/2 + z/3 - z^2/4 + z^3/5)
 *         supplies the rest (Taylor series, truncation below 2^-27
 *         relative).  No division.  Max error 0.60 ulp over every positive
 *         normal float; all but 0.0005 % correctly rounded.
 */
#ifndef KINC_FMATH_H
#define KINC_FMATH_H

#ifdef __CUDACC__
#define KINC_HD __host__ __device__ __forceinline__
#else
#define KINC_HD static inline
#endif

#ifdef __cplusplus
#include <cstdint>
#include <cstring>
#include <cmath>
#define KINC_FMAF(a, b, c) ::fmaf((a), (b), (c))
#else
#include <stdint.h>
#include <string.h>
#include <math.h>
#define KINC_FMAF(a, b, c) fmaf((a), (b), (c))
#endif

#define KINC_F_LOG2E 1.44269502162933349609375f      /* float nearest to 1/ln2 */
#define KINC_F_LN2_HI 0.693145751953125f             /* 0x3f317200 */
#define KINC_F_LN2_LO 1.428606765330187045037746429e-06f /* ln2 - LN2_HI */
#define KINC_F_SQRT2 1.41421353816986083984375f      /* float nearest to sqrt(2) */
/* kinc_expf's polynomial (minimax on [-ln2/2, ln2/2], see the method note) */
#define KINC_EXP_C6 1.3893402647227049e-3f
#define KINC_EXP_C5 8.370262570679188e-3f
#define KINC_EXP_C4 4.1667088866233826e-2f
#define KINC_EXP_C3 1.6666506230831146e-1f
#define KINC_EXP_C2 4.999999701976776e-1f

/* kinc_logf's reduction table: { invc_i, hi_i, lo_i, 0 } for the 32 steps of
 * the mantissa bits above 0x3f340000 (see the method note above) */
#define KINC_LOG_TABLE_INIT \
   { \
   { 1.40625f, -0.3409271240234375f, 5.370528697e-07f, 0.0f }, \
   { 1.375f, -0.318450927734375f, -2.803384177e-06f, 0.0f }, \
   { 1.34375f, -0.29547119140625f, 6.978512374e-06f, 0.0f }, \
   { 1.3125f, -0.2719268798828125f, -6.835600743e-06f, 0.0f }, \
   { 1.296875f, -0.2599639892578125f, 6.464820672e-06f, 0.0f }, \
   { 1.265625f, -0.235565185546875f, -8.857658713e-07f, 0.0f }, \
   { 1.25f, -0.22314453125f, 9.799357485e-07f, 0.0f }, \
   { 1.21875f, -0.1978302001953125f, 4.456865554e-06f, 0.0f }, \
   { 1.203125f, -0.1849212646484375f, -1.073845624e-06f, 0.0f }, \
   { 1.171875f, -0.158599853515625f, -5.176661034e-06f, 0.0f }, \
   { 1.15625f, -0.1451873779296875f, 5.368085112e-06f, 0.0f }, \
   { 1.125f, -0.1177825927734375f, -4.428829357e-07f, 0.0f }, \
   { 1.109375f, -0.103790283203125f, -6.510478670e-06f, 0.0f }, \
   { 1.09375f, -0.0896148681640625f, 2.709474302e-06f, 0.0f }, \
   { 1.078125f, -0.075225830078125f, 2.408840601e-06f, 0.0f }, \
   { 1.0625f, -0.0606231689453125f, -1.452871174e-06f, 0.0f }, \
   { 1.046875f, -0.045806884765625f, -2.651265731e-06f, 0.0f }, \
   { 1.03125f, -0.0307769775390625f, 5.318872354e-06f, 0.0f }, \
   { 1.0f, 0.0f, 0.0f, 0.0f }, \
   { 1.0f, 0.0f, 0.000000000e+00f, 0.0f }, \
   { 0.953125f, 0.048004150390625f, 5.068795872e-06f, 0.0f }, \
   { 0.921875f, 0.0813446044921875f, 1.034961770e-06f, 0.0f }, \
   { 0.90625f, 0.0984344482421875f, 5.624571259e-06f, 0.0f }, \
   { 0.875f, 0.1335296630859375f, 1.729538553e-06f, 0.0f }, \
   { 0.859375f, 0.15155029296875f, -3.948415497e-07f, 0.0f }, \
   { 0.828125f, 0.1885986328125f, -7.463004749e-06f, 0.0f }, \
   { 0.8125f, 0.2076416015625f, -2.236784212e-06f, 0.0f }, \
   { 0.796875f, 0.22705078125f, 6.669385129e-06f, 0.0f }, \
   { 0.765625f, 0.267059326171875f, 3.459077107e-06f, 0.0f }, \
   { 0.75f, 0.287689208984375f, -7.136532531e-06f, 0.0f }, \
   { 0.734375f, 0.3087310791015625f, 4.402548257e-06f, 0.0f }, \
   { 0.71875f, 0.3302459716796875f, -4.284809165e-06f, 0.0f }, \
   }

typedef struct
{
   float inv, hi, lo, pad;
} kinc_log_entry;

#ifdef __CUDACC__
static __device__ const __align__(16) kinc_log_entry kinc_log_table_d[32] = KINC_LOG_TABLE_INIT;
#endif
static const kinc_log_entry kinc_log_table_h[32] = KINC_LOG_TABLE_INIT;

KINC_HD uint32_t kinc_f2u(float x)
{
#ifdef __CUDA_ARCH__
   return (uint32_t)__float_as_uint(x);
#else
   uint32_t u;
   memcpy(&u, &x, sizeof u);
   return u;
#endif
}

KINC_HD float kinc_u2f(uint32_t u)
{
#ifdef __CUDA_ARCH__
   return __uint_as_float(u);
#else
   float x;
   memcpy(&x, &u, sizeof x);
   return x;
#endif
}

/* slow path of kinc_expf: NaN, overflow, underflow and subnormal results */
KINC_HD float kinc_expf_tail(float x, float n, float p)
{
   if ( !(x == x) )
   {
      return x + x;
   }
   if ( x > 88.72283172607421875f )   /* 0x42b17217: largest x with finite e^x */
   {
      return kinc_u2f(0x7f800000u);
   }
   if ( x < -104.0f )                 /* e^x < 2^-150: rounds to zero */
   {
      return 0.0f;
   }
   const int in = (int)n;
   if ( in >= -126 && in <= 127 )
   {
      return p * kinc_u2f((uint32_t)(in + 127) << 23);
   }
   if ( in > 127 )
   {
      /* only n = 128 reaches here: p * 2^127 * 2 */
      return (p * kinc_u2f(0x7f000000u)) * kinc_u2f((uint32_t)(in - 127 + 127) << 23);
   }
   /* n in [-151, -127]: p * 2^(n+64) is a normal float, the second step rounds once */
   return (p * kinc_u2f((uint32_t)(in + 64 + 127) << 23)) * kinc_u2f((uint32_t)(-64 + 127) << 23);
}

/* e^x, single precision. */
KINC_HD float kinc_expf(float x)
{
   /* n = rint(x / ln2): adding and removing 1.5 * 2^23 rounds to the nearest
    * integer (ties to even) for |x / ln2| < 2^22, which covers every x that
    * reaches the scaling below; the sum's low mantissa bits hold n itself */
   const float shifted = KINC_FMAF(x, KINC_F_LOG2E, 12582912.0f);
   const float n = shifted - 12582912.0f;
   float r = KINC_FMAF(-n, KINC_F_LN2_HI, x);
   r = KINC_FMAF(-n, KINC_F_LN2_LO, r);

   /* 1 + r + r^2 (c2 + r (c3 + r (c4 + r (c5 + r c6)))) */
   float p = KINC_EXP_C6;
   p = KINC_FMAF(p, r, KINC_EXP_C5);
   p = KINC_FMAF(p, r, KINC_EXP_C4);
   p = KINC_FMAF(p, r, KINC_EXP_C3);
   p = KINC_FMAF(p, r, KINC_EXP_C2);
   p = KINC_FMAF(p, r, 1.0f);
   p = KINC_FMAF(p, r, 1.0f);

   /* |x| <= 86 keeps n in [-125, 125] and p in [0.70, 1.42]: p * 2^n is a
    * normal float, formed exactly by adding n to p's exponent field -- the
    * low bits of `shifted` shifted up by 23 are n * 2^23 modulo 2^32 (NaN
    * fails the comparison and takes the tail) */
   if ( (x < 0.0f ? -x : x) <= 86.0f )
   {
      return kinc_u2f(kinc_f2u(p) + (kinc_f2u(shifted) << 23));
   }
   return kinc_expf_tail(x, n, p);
}

/* natural logarithm of the positive normal float with bits b, times 2^eoff */
KINC_HD float kinc_logf_normal(uint32_t b, int eoff)
{
   const uint32_t tmp = b - 0x3f340000u;
   const int e = (int)((int32_t)tmp >> 23) + eoff;
   const int i = (int)((tmp >> 18) & 31u);
   const float m = kinc_u2f(b - (tmp & 0xff800000u));   /* in [0.703125, 1.40625) */
#ifdef __CUDA_ARCH__
   const kinc_log_entry t = kinc_log_table_d[i];
#else
   const kinc_log_entry t = kinc_log_table_h[i];
#endif
   const float z = KINC_FMAF(m, t.inv, -1.0f);           /* exact */
   float q = 0.2f;
   q = KINC_FMAF(q, z, -0.25f);
   q = KINC_FMAF(q, z, 0.333333343267440796f);          /* float nearest to 1/3 */
   q = KINC_FMAF(q, z, -0.5f);
   const float z2 = z * z;
   const float ef = (float)e;
   const float hi = KINC_FMAF(ef, KINC_F_LN2_HI, t.hi);   /* exact: a multiple of 2^-16 below 2^7 */
   /* hi + z as s + err (|hi| >= |z| or hi = 0: Dekker's fast two-sum) */
   const float s = hi + z;
   const float err = (hi - s) + z;
   const float lo = KINC_FMAF(ef, KINC_F_LN2_LO, t.lo) + err;
   return s + KINC_FMAF(z2, q, lo);
}

/* natural logarithm, single precision. */
KINC_HD float kinc_logf(float x)
{
   const uint32_t b = kinc_f2u(x);
   if ( b - 0x00800000u < 0x7f000000u )
   {
      return kinc_logf_normal(b, 0);
   }
   if ( !(x == x) )
   {
      return x + x;
   }
   if ( x < 0.0f )
   {
      return kinc_u2f(0x7fc00000u);
   }
   if ( x == 0.0f )
   {
      return kinc_u2f(0xff800000u);
   }
   if ( x == kinc_u2f(0x7f800000u) )
   {
      return x;
   }
   /* subnormal: scale into the normal range first (exact) */
   return kinc_logf_normal(kinc_f2u(x * 8388608.0f), -23);
}

#endif
