/*
 * Host-compilation shim for building the reference's Thrust sources as plain C++
 * on the serial (CPP) Thrust backend.  It supplies host versions of the handful of
 * CUDA device intrinsics those sources call and an lvalue overload of
 * thrust::make_pair that CCCL 3 no longer provides.  Part of the checker only.
 */
#pragma once
#include <cuda_runtime_api.h>
#include <cmath>
#include <thrust/pair.h>

template <typename T> static inline T __ldg(const T *p) { return *p; }
static inline int __float2int_rd(float x) { return (int)std::floor(x); }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline float norm3df(float a, float b, float c) { return std::sqrt(a * a + b * b + c * c); }

namespace thrust
{
template <class T1, class T2> inline pair<T1, T2> make_pair(const T1 &a, const T2 &b)
{
    return pair<T1, T2>(a, b);
}
} // namespace thrust
