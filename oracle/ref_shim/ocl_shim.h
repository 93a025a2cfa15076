/*
 * TEST INFRASTRUCTURE ONLY.  Forced-include for compiling KINC's OpenCL kernels
 * (src/opencl/{linalg,fetchpair,sort,outlier,gmm,kmeans,pearson,spearman}.cl, concatenated
 * in that order) as C++ on the host, so that the OpenCL worker's semantics -- the per-fit
 * POSIX LCG initialisation among them -- can be run on the CPU as a second reference.
 *
 * It stands in for the parts of OpenCL C those files use: the address-space qualifiers, the
 * vector types float2 / float4 / int2 (only their .x/.y members and the (a, b) constructor are
 * used; the build recipe rewrites the one OpenCL vector literal "(float2)(a, b)" into a
 * constructor call), get_global_id, and the float overloads of the math built-ins.  The float
 * exp/log are routed to kinc_expf/kinc_logf, the math the GPU kernels and the CPU oracle use,
 * so differences in results come from the kernels' logic, not from a math library.
 */
#ifndef KINC_OCL_SHIM_H
#define KINC_OCL_SHIM_H

#include <cmath>
#include <cstdint>

#include "kinc_fmath.h"

#define __kernel
#define __global
#define __local
#define __constant const

typedef unsigned long ulong;
typedef unsigned int uint;

struct float2
{
   float x, y;
   float2() = default;
   float2(float a, float b) : x(a), y(b) {}
};

struct float4
{
   float x, y, z, w;
};

struct int2
{
   int x, y;
};

/* the work-item index of the kernel call in progress (set by the driver) */
extern thread_local int kocl_global_id;

inline int get_global_id(int) { return kocl_global_id; }

inline float exp(float x) { return kinc_expf(x); }
inline float log(float x) { return kinc_logf(x); }
inline float sqrt(float x) { return ::sqrtf(x); }
inline float fabs(float x) { return ::fabsf(x); }
using std::isnan;

#endif
