// ct_internal.h -- host-side error plumbing and small exact conversions shared
// by the translation units of libcelltree_gb300.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "celltree_gb300.h"

// Records a readable reason for the last failure (thread-local) and returns
// the status code.
int ct_fail(int status, const char* msg);

#define CT_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) return ct_fail(CT_ERR_CUDA, cudaGetErrorString(e_));    \
    } while (0)

#define CT_CHECK_LAUNCH(what)                                                          \
    do {                                                                               \
        cudaError_t e_ = cudaGetLastError();                                           \
        if (e_ != cudaSuccess) return ct_fail(CT_ERR_CUDA, cudaGetErrorString(e_));    \
    } while (0)

#ifdef __CUDACC__
// Exact int -> double built with integer operations only (GB300 runs float64
// conversions on its narrow float64 pipe).  Valid for |x| < 2^31.
__device__ __forceinline__ double exact_i2d(int x) {
    if (x == 0) return 0.0;
    unsigned long long sign = x < 0 ? 0x8000000000000000ull : 0ull;
    unsigned int a = x < 0 ? (unsigned int)(-(long long)x) : (unsigned int)x;
    int lz = __clz(a);
    int e = 31 - lz;                                  // floor(log2 a)
    unsigned long long mant = ((unsigned long long)a << (52 - e)) & 0x000fffffffffffffull;
    unsigned long long bits = sign | ((unsigned long long)(e + 1023) << 52) | mant;
    return __longlong_as_double((long long)bits);
}
// 1 / n for a power of two n (exact).
__device__ __forceinline__ double exact_pow2_inv(int n) {
    int e = 31 - __clz((unsigned int)n);
    return __longlong_as_double((long long)((unsigned long long)(1023 - e) << 52));
}
#endif
