/*
 * kinc_f2.h -- two single-precision values in one 64-bit register, operated on
 * by the packed FP32 instructions of sm_100-class GPUs (add/sub/mul/fma
 * .rn.f32x2).  Each half is rounded exactly as the scalar instruction rounds
 * it, so a computation written with F2 gives, element by element, the bits of
 * the same computation written with float -- the packed form only halves the
 * instructions issued -- provided no product is contracted into a following
 * sum (see mulz).  The GMM fit pairs its mixture components this way: every
 * per-component accumulator is still summed in sample order.
 *
 * kinc_expf2 is kinc_expf (kinc_fmath.h) on both halves: the same shifter,
 * reduction, polynomial and exponent-field scaling, packed where the scalar
 * form uses a float operation; a half outside the fast path's range takes the
 * scalar function, so every result equals kinc_expf of that half.
 */
#pragma once

#include <cstdint>

#include "kinc_fmath.h"

namespace kinc {

struct F2
{
   unsigned long long v;
};

__device__ __forceinline__ F2 f2(float lo, float hi)
{
   F2 r;
   asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
   return r;
}

__device__ __forceinline__ F2 f2(float s)
{
   return f2(s, s);
}

__device__ __forceinline__ void split(F2 a, float& lo, float& hi)
{
   asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}

__device__ __forceinline__ float lo(F2 a)
{
   float l, h;
   split(a, l, h);
   return l;
}

__device__ __forceinline__ float hi(F2 a)
{
   float l, h;
   split(a, l, h);
   return h;
}

__device__ __forceinline__ F2 operator+(F2 a, F2 b)
{
   F2 r;
   asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
   return r;
}

__device__ __forceinline__ F2 operator-(F2 a, F2 b)
{
   F2 r;
   asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
   return r;
}

__device__ __forceinline__ F2 operator*(F2 a, F2 b)
{
   F2 r;
   asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
   return r;
}

__device__ __forceinline__ F2& operator+=(F2& a, F2 b)
{
   a = a + b;
   return a;
}

/* a * b + c with one rounding, per half */
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c)
{
   F2 r;
   asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
   return r;
}

/*
 * A product that feeds a sum.  ptxas contracts a packed multiply followed by a packed add into one
 * packed fused multiply-add even when the PTX asks for rounded steps (and with --fmad=false), which
 * would skip the product's own rounding.  fma(a, b, -0) is bitwise a * b -- the exact product plus
 * -0 rounds once, and a zero product keeps its sign -- and a fused product cannot be contracted
 * again; z must be -0.0 held where the compiler cannot see its value (a kernel argument), or the
 * fma would fold back into a multiply.  Scalar floats need none of this: the per-pair units build
 * with --fmad=false, which ptxas honours for scalar instructions.
 */
__device__ __forceinline__ F2 mulz(F2 a, F2 b, F2 z)
{
   return fma2(a, b, z);
}

__device__ __forceinline__ float mulz(float a, float b, float)
{
   return a * b;
}

__device__ __forceinline__ float fma_t(float a, float b, float c)
{
   return fmaf(a, b, c);
}

__device__ __forceinline__ F2 fma_t(F2 a, F2 b, F2 c)
{
   return fma2(a, b, c);
}

/* a constant of type T (float, or both halves of an F2) */
template <class T> __device__ __forceinline__ T cst(float c);
template <> __device__ __forceinline__ float cst<float>(float c)
{
   return c;
}
template <> __device__ __forceinline__ F2 cst<F2>(float c)
{
   return f2(c);
}

/* 1: one range test for both halves of kinc_expf2; measured slower in the GMM fits (2,142 vs
 * 2,004 ms per 262,144-pair block of the 5,000 x 1,000 workload) */
#ifndef KINC_EXPF2_ONE_BRANCH
#define KINC_EXPF2_ONE_BRANCH 0
#endif

/* the fast path of kinc_expf (kinc_fmath.h) on one half: exponent-field scaling */
__device__ __forceinline__ float expf_scale(float x, float p, float shifted)
{
   if ( fabsf(x) <= 86.0f ) return __uint_as_float(__float_as_uint(p) + (__float_as_uint(shifted) << 23));
   return kinc_expf(x);
}

/* kinc_expf on both halves */
__device__ __forceinline__ F2 kinc_expf2(F2 x)
{
   const F2 shifted = fma2(x, f2(KINC_F_LOG2E), f2(12582912.0f));
   const F2 n = shifted - f2(12582912.0f);
   /* fma(-n, c, x) == fma(n, -c, x): the product's sign flips exactly */
   F2 r = fma2(n, f2(-KINC_F_LN2_HI), x);
   r = fma2(n, f2(-KINC_F_LN2_LO), r);
   F2 p = f2(KINC_EXP_C6);
   p = fma2(p, r, f2(KINC_EXP_C5));
   p = fma2(p, r, f2(KINC_EXP_C4));
   p = fma2(p, r, f2(KINC_EXP_C3));
   p = fma2(p, r, f2(KINC_EXP_C2));
   p = fma2(p, r, f2(1.0f));
   p = fma2(p, r, f2(1.0f));
   float x0, x1, p0, p1, s0, s1;
   split(x, x0, x1);
   split(p, p0, p1);
   split(shifted, s0, s1);
#if KINC_EXPF2_ONE_BRANCH
   /* one test for both halves (NaN fails it), the rare slow path out of line */
   if ( __builtin_expect(!(fabsf(x0) <= 86.0f && fabsf(x1) <= 86.0f), 0) )
      return f2(expf_scale(x0, p0, s0), expf_scale(x1, p1, s1));
   return f2(__uint_as_float(__float_as_uint(p0) + (__float_as_uint(s0) << 23)),
             __uint_as_float(__float_as_uint(p1) + (__float_as_uint(s1) << 23)));
#else
   return f2(expf_scale(x0, p0, s0), expf_scale(x1, p1, s1));
#endif
}

__device__ __forceinline__ float kinc_exp_t(float x)
{
   return kinc_expf(x);
}

__device__ __forceinline__ F2 kinc_exp_t(F2 x)
{
   return kinc_expf2(x);
}

} /* namespace kinc */
