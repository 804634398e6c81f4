// Shared helpers for the phase-linking kernels: status plumbing, IEEE-exact
// float helpers (no FMA contraction where bit-exactness against numpy matters),
// complex arithmetic and warp utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/dpl.h"

namespace dpl {

// ----------------------------------------------------------------------------------
// host-side status plumbing
// ----------------------------------------------------------------------------------
void set_error(const std::string& msg);
dpl_status fail(dpl_status st, const std::string& msg);
dpl_status check_launch(const char* what);

#define DPL_CUDA_TRY(expr)                                                              \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess)                                                          \
            return ::dpl::fail(DPL_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

constexpr int kMaxNslc = 64;
constexpr int kWarp = 32;

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Bump allocator over a caller-provided workspace.
struct Workspace {
    char* base;
    size_t size;
    size_t used = 0;
    template <class T>
    T* take(size_t count) {
        used = align_up(used, 256);
        T* p = reinterpret_cast<T*>(base + used);
        used += count * sizeof(T);
        return p;
    }
    bool ok() const { return used <= size; }
};

// ----------------------------------------------------------------------------------
// device helpers
// ----------------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// interleaved complex64, 8-byte aligned so that one element is one 64-bit access
struct __align__(8) cfloat {
    float re, im;
};

// complex arrays handed in through the C ABI must keep complex64's 8-byte alignment
inline bool misaligned_c8(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) != 0; }

__device__ __forceinline__ cfloat cmake(float r, float i) { return {r, i}; }
__device__ __forceinline__ cfloat cadd(cfloat a, cfloat b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cfloat csub(cfloat a, cfloat b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cfloat cmul(cfloat a, cfloat b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
// a * conj(b)
__device__ __forceinline__ cfloat cmulc(cfloat a, cfloat b) {
    return {a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im};
}
// acc + x * y and acc - x * conj(y) as four fused multiply-adds
__device__ __forceinline__ cfloat cfma(cfloat acc, cfloat x, cfloat y) {
    return {fmaf(x.re, y.re, fmaf(-x.im, y.im, acc.re)), fmaf(x.re, y.im, fmaf(x.im, y.re, acc.im))};
}
__device__ __forceinline__ cfloat cfms_conj(cfloat acc, cfloat x, cfloat y) {
    return {fmaf(-x.re, y.re, fmaf(-x.im, y.im, acc.re)), fmaf(-x.im, y.re, fmaf(x.re, y.im, acc.im))};
}
__device__ __forceinline__ cfloat cconj(cfloat a) { return {a.re, -a.im}; }
__device__ __forceinline__ cfloat cscale(cfloat a, float s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ float cabs2(cfloat a) { return a.re * a.re + a.im * a.im; }
__device__ __forceinline__ float cabs(cfloat a) { return hypotf(a.re, a.im); }
__device__ __forceinline__ bool cisnan(cfloat a) { return isnan(a.re) || isnan(a.im); }
// Complex division with scaling (Smith's method) to avoid overflow/underflow.
__device__ __forceinline__ cfloat cdiv(cfloat a, cfloat b) {
    if (fabsf(b.re) >= fabsf(b.im)) {
        float r = b.im / b.re;
        float d = b.re + b.im * r;
        return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
    } else {
        float r = b.re / b.im;
        float d = b.re * r + b.im;
        return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
    }
}
// exp(i * angle(a)): unit phasor with angle(0) = 0 and NaN preserved.
__device__ __forceinline__ cfloat cphasor(cfloat a) {
    if (cisnan(a)) return {nanf(""), nanf("")};
    float m = hypotf(a.re, a.im);
    if (m == 0.f) {
        // angle(+-0 + 0j) is 0 or pi depending on the sign of the real zero
        return {signbit(a.re) ? -1.f : 1.f, 0.f};
    }
    return {a.re / m, a.im / m};
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ bool warp_any(bool v) { return __any_sync(0xffffffffu, v); }

__device__ __forceinline__ cfloat shfl_c(cfloat v, int src) {
    return {__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src)};
}

// Input pixel flags written by the preparation kernel.
enum PixFlag : uint8_t {
    kNodata = 1,  // user nodata or any NaN in the stack (phase_link/_core.py:181)
    kPs = 2,      // PS after removing nodata (:183)
    kIgnore = 4,  // masked to NaN before covariance (:186-191)
};

}  // namespace dpl
