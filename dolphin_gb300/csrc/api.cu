// Status plumbing and library-level queries for the C ABI.
#include "dpl_common.cuh"

namespace dpl {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

dpl_status fail(dpl_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

dpl_status check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DPL_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return DPL_OK;
}

}  // namespace dpl

extern "C" const char* dpl_last_error_message(void) { return dpl::g_last_error.c_str(); }

extern "C" int dpl_version(void) { return 1000; }

extern "C" int dpl_max_nslc(void) { return dpl::kMaxNslc; }

// FP32 fused multiply-add throughput, for the FP32 roofline of the CUDA-core kernels:
// each thread runs 8 independent chains of `iters` FMAs (enough independent work for
// every SM sub-partition to issue one FFMA per cycle) and writes one value, which keeps
// the chains live.
__global__ void __launch_bounds__(256) k_fma_peak(float* out, int iters) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3f + (float)k;
#pragma unroll 8
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], 0.999999f, 1e-7f);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" dpl_status dpl_fp32_fma_probe(float* out, int blocks, int iters, dpl_stream_t stream) {
    if (!out || blocks < 1 || iters < 1) return dpl::fail(DPL_ERR_INVALID_ARGUMENT, "dpl_fp32_fma_probe: bad argument");
    k_fma_peak<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters);
    return dpl::check_launch("k_fma_peak");
}

// FP64 counterpart of k_fma_peak: 8 independent chains of double FMAs per thread.
__global__ void __launch_bounds__(256) k_fma64_peak(double* out, int iters) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3 + (double)k;
#pragma unroll 8
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], 0.999999999, 1e-12);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" dpl_status dpl_fp64_fma_probe(double* out, int blocks, int iters, dpl_stream_t stream) {
    if (!out || blocks < 1 || iters < 1) return dpl::fail(DPL_ERR_INVALID_ARGUMENT, "dpl_fp64_fma_probe: bad argument");
    k_fma64_peak<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters);
    return dpl::check_launch("k_fma64_peak");
}
