/*
 * TEST INFRASTRUCTURE ONLY.  A minimal stand-in for the ACE framework header
 * <ace/core/core.h>, sufficient to compile KINC's CPU Pairwise:: sources
 * (src/core/pairwise_{linalg,clustering,gmm,kmeans,correlation,pearson,
 * spearman}.cpp) unmodified for use as the parity reference.  ACE itself is
 * not part of the KINC tree; only the few Qt/ACE types those files touch are
 * provided here.
 *
 * KINC_REF_MATH selects how the sources' unqualified exp/log/sqrt/fabs on
 * float arguments resolve -- the reference's results depend on it and its
 * real headers do not pin it:
 *   0 (default) float overloads routed to kinc_expf/kinc_logf (the math the
 *     GPU kernels use), sqrtf and fabsf; log of an int is double (as in
 *     libstdc++);
 *   1 the float overloads of the C++ library (glibc expf/logf/sqrtf/fabsf);
 *   2 only the C library's double functions, so float arguments are promoted
 *     and the surrounding expressions are evaluated partly in double.
 */
#ifndef KINC_REF_SHIM_ACE_CORE_H
#define KINC_REF_SHIM_ACE_CORE_H

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "kinc_fmath.h"

typedef int8_t qint8;
typedef int16_t qint16;
typedef int32_t qint32;
typedef int64_t qint64;

template<class T>
class QVector : public std::vector<T>
{
public:
   using std::vector<T>::vector;
   int size() const { return (int)std::vector<T>::size(); }
   void append(const T& v) { this->push_back(v); }
};

class QString : public std::string
{
public:
   using std::string::string;
};

#ifndef KINC_REF_MATH
#define KINC_REF_MATH 0
#endif

#if KINC_REF_MATH == 0
inline float exp(float x) { return kinc_expf(x); }
inline float log(float x) { return kinc_logf(x); }
inline double log(int x) { return ::log((double)x); }
inline float sqrt(float x) { return ::sqrtf(x); }
inline float fabs(float x) { return ::fabsf(x); }
#elif KINC_REF_MATH == 1
using std::exp;
using std::fabs;
using std::log;
using std::sqrt;
#endif

#endif
