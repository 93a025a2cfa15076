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
 *   exp:  n = rint(x/ln2) by the 1.5*2^23 shifter; Cody-Waite argument
 *         reduction x = n*ln2 + r with a two-part ln2
 *         whose leading part has 16 significant bits (so n*LN2_HI and
 *         x - n*LN2_HI are exact for |n| <= 2^8), |r| <= ln2/2; then the
 *         degree-7 Taylor polynomial of e^r by Horner's rule in fused
 *         multiply-adds; then scaling by 2^n through the exponent field,
 *         split in two steps when 2^n itself is not a normal float.
 *   log:  x = 2^e * m with m in [sqrt(1/2), sqrt(2)); with f = m - 1 and
 *         s = f/(2+f), log(m) = 2 atanh(s) = f - (f^2/2 - s*(f^2/2 + R)),
 *         R = sum_{k>=1} 2 s^{2k}/(2k+1) (Taylor series of atanh, truncated
 *         after s^10), and log(x) = e*ln2 + log(m) with the same two-part ln2.
 * Both are within ~1 ulp of the true value (checked against libm double in
 * the CPU tests and against all float inputs of the used range on the GPU).
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
#ifdef __CUDA_ARCH__
   const float shifted = __fadd_rn(__fmul_rn(x, KINC_F_LOG2E), 12582912.0f);   /* never contracted */
#else
   const float shifted = x * KINC_F_LOG2E + 12582912.0f;   /* hosts build with -ffp-contract=off */
#endif
   const float n = shifted - 12582912.0f;
   float r = KINC_FMAF(-n, KINC_F_LN2_HI, x);
   r = KINC_FMAF(-n, KINC_F_LN2_LO, r);

   /* 1 + r + r^2/2! + ... + r^7/7! */
   float p = 1.98412698412698412698e-4f;                /* 1/5040 */
   p = KINC_FMAF(p, r, 1.38888888888888888889e-3f);     /* 1/720 */
   p = KINC_FMAF(p, r, 8.33333333333333333333e-3f);     /* 1/120 */
   p = KINC_FMAF(p, r, 4.16666666666666666667e-2f);     /* 1/24 */
   p = KINC_FMAF(p, r, 1.66666666666666666667e-1f);     /* 1/6 */
   p = KINC_FMAF(p, r, 0.5f);
   p = KINC_FMAF(p, r, 1.0f);
   p = KINC_FMAF(p, r, 1.0f);

   /* |x| <= 87 keeps n in [-126, 126]: 2^n is a normal float and the product
    * rounds once (NaN fails the comparison and takes the tail) */
   if ( (x < 0.0f ? -x : x) <= 87.0f )
   {
      /* bits(shifted) - bits(1.5 * 2^23) = n; 2^n has exponent field n + 127 */
      return p * kinc_u2f((kinc_f2u(shifted) - 0x4b400000u + 127u) << 23);
   }
   return kinc_expf_tail(x, n, p);
}

/* natural logarithm of the positive normal float with bits b, times 2^eoff */
KINC_HD float kinc_logf_normal(uint32_t b, int eoff)
{
   int e = (int)(b >> 23) - 127 + eoff;
   float m = kinc_u2f((b & 0x007fffffu) | 0x3f800000u);
   if ( m > KINC_F_SQRT2 )
   {
      m = m * 0.5f;
      e += 1;
   }

   const float f = m - 1.0f;                 /* exact: m in [0.70, 1.42] */
   const float s = f / (2.0f + f);
   const float z = s * s;
   float R = 0.181818181818181818182f;                   /* 2/11 */
   R = KINC_FMAF(R, z, 0.222222222222222222222f);        /* 2/9 */
   R = KINC_FMAF(R, z, 0.285714285714285714286f);        /* 2/7 */
   R = KINC_FMAF(R, z, 0.4f);                            /* 2/5 */
   R = KINC_FMAF(R, z, 0.666666666666666666667f);        /* 2/3 */
   R = R * z;
   const float hfsq = (0.5f * f) * f;
   const float ef = (float)e;

   /* log(m) = f - (hfsq - s*(hfsq + R)); the e*ln2 tail joins the small terms */
   const float small = KINC_FMAF(s, hfsq + R, ef * KINC_F_LN2_LO);
   const float logm = f - (hfsq - small);
   return KINC_FMAF(ef, KINC_F_LN2_HI, logm);
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
