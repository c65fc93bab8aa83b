// Shared helpers for the SophT GB300 flow-step library (sm_103a).
//
// Every exported entry point returns an int status (SG_OK = 0) and records a
// message retrievable with sg_last_error().  Step entry points take an explicit
// cudaStream_t (passed as void*), never allocate and never synchronise.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>
#include <string>

#include "../../include/sopht_gb300.h"

namespace sg {

void set_last_error(const char* fmt, ...);

inline int cuda_status(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return SG_OK;
    set_last_error("%s: %s", where, cudaGetErrorString(e));
    return SG_ERR_CUDA;
}

// status of the most recent launch on this thread
inline int launch_status(const char* where) { return cuda_status(cudaGetLastError(), where); }

#define SG_TRY(expr)                 \
    do {                             \
        int _s = (expr);             \
        if (_s != SG_OK) return _s;  \
    } while (0)

#define SG_REQUIRE(cond, code, ...)          \
    do {                                     \
        if (!(cond)) {                       \
            ::sg::set_last_error(__VA_ARGS__); \
            return (code);                   \
        }                                    \
    } while (0)

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };
template <typename T> using cplx_t = typename cplx_of<T>::type;

template <typename C> __host__ __device__ __forceinline__ C cmake(decltype(C::x) re, decltype(C::x) im) {
    C c;
    c.x = re;
    c.y = im;
    return c;
}
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
    return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// fp32 complex sums on the device as packed two-lane instructions (one FADD2 / FFMA2 for both
// parts, half the issue slots of two scalar adds): the FFT butterflies are mostly these.  a - b is
// fma(b, -1, a), which rounds the exact difference once, as a - b does.
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
template <> __host__ __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) { return __fadd2_rn(a, b); }
template <> __host__ __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
#endif
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { return cmake<C>(a.x, -a.y); }
template <typename C, typename T> __host__ __device__ __forceinline__ C cscale(C a, T s) { return cmake<C>(a.x * s, a.y * s); }
// multiply by (0 + i*s): i*(x + i y) = -y + i x
template <typename C> __host__ __device__ __forceinline__ C cmul_i(C a) { return cmake<C>(-a.y, a.x); }

inline int dtype_size(int dtype) { return dtype == SG_F64 ? 8 : 4; }

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace sg
