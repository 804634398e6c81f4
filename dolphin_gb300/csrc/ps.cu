// Amplitude dispersion and PS selection: calc_ps_block (ps.py:169-244).
//
// One thread per pixel streams the N magnitudes once (coalesced across the warp,
// date-major input) and keeps them in registers for the second (variance) pass.
// The arithmetic reproduces numpy's float32 nanmean / nanstd exactly: sequential
// sums along axis 0, NaN entries replaced by 0, divisions by the count rounded
// once, no FMA contraction.  The kernel is HBM-bound: 4N bytes in, 9 bytes out.
#include "dpl_common.cuh"

namespace dpl {

template <int NMAX>
__global__ void __launch_bounds__(256) k_ps_block(const float* __restrict__ mag, int n, int64_t npix,
                                                  float thr, int thr_is_f64, double thr64, int64_t min_count,
                                                  float* __restrict__ mean_out, float* __restrict__ disp_out,
                                                  uint8_t* __restrict__ ps_out) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float x[NMAX > 0 ? NMAX : 1];
    uint64_t nanbits = 0;
    float sum = 0.f;
    int cnt = 0;
    if (NMAX > 0) {
#pragma unroll
        for (int t = 0; t < (NMAX > 0 ? NMAX : 1); ++t) {
            if (t < n) {
                float v = __ldg(mag + (int64_t)t * npix + p);
                bool nan = isnan(v);
                x[t] = nan ? 0.f : v;
                nanbits |= (uint64_t)nan << t;
                cnt += nan ? 0 : 1;
                sum = t == 0 ? x[0] : fadd(sum, x[t]);
            }
        }
    } else {
        for (int t = 0; t < n; ++t) {
            float v = __ldg(mag + (int64_t)t * npix + p);
            bool nan = isnan(v);
            float xv = nan ? 0.f : v;
            cnt += nan ? 0 : 1;
            sum = t == 0 ? xv : fadd(sum, xv);
        }
    }
    float mean = fdiv(sum, (float)cnt);
    float ss = 0.f;
    if (NMAX > 0) {
#pragma unroll
        for (int t = 0; t < (NMAX > 0 ? NMAX : 1); ++t) {
            if (t < n) {
                float d = ((nanbits >> t) & 1) ? 0.f : fsub(x[t], mean);
                float sq = fmul(d, d);
                ss = t == 0 ? sq : fadd(ss, sq);
            }
        }
    } else {
        for (int t = 0; t < n; ++t) {
            float v = __ldg(mag + (int64_t)t * npix + p);
            float d = isnan(v) ? 0.f : fsub(v, mean);
            float sq = fmul(d, d);
            ss = t == 0 ? sq : fadd(ss, sq);
        }
    }
    float var = fdiv(ss, (float)cnt);
    float sd = fsqrt(var);
    float disp = fdiv(sd, mean);
    if (cnt < min_count) disp = nanf("");
    if (!isfinite(mean)) mean = 0.f;
    if (!isfinite(disp)) disp = 0.f;
    bool ps = thr_is_f64 ? ((double)disp < thr64) : (disp < thr);
    if (disp == 0.f) ps = false;
    mean_out[p] = mean;
    disp_out[p] = disp;
    ps_out[p] = ps ? 1 : 0;
}

}  // namespace dpl

using namespace dpl;

extern "C" dpl_status dpl_ps_block(const float* stack_mag, int64_t nslc, int64_t npix, float threshold,
                                   int threshold_is_f64, double threshold64, int64_t min_count, float* mean,
                                   float* amp_disp, uint8_t* ps, dpl_stream_t stream) {
    if (nslc <= 0 || npix < 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_ps_block: bad shape");
    if (npix == 0) return DPL_OK;
    if (!stack_mag || !mean || !amp_disp || !ps) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_ps_block: null pointer");
    dim3 block(256), grid(ceil_div(npix, 256));
    cudaStream_t s = (cudaStream_t)stream;
    int n = (int)nslc;
    if (n <= 16)
        k_ps_block<16><<<grid, block, 0, s>>>(stack_mag, n, npix, threshold, threshold_is_f64, threshold64, min_count, mean, amp_disp, ps);
    else if (n <= 32)
        k_ps_block<32><<<grid, block, 0, s>>>(stack_mag, n, npix, threshold, threshold_is_f64, threshold64, min_count, mean, amp_disp, ps);
    else if (n <= 64)
        k_ps_block<64><<<grid, block, 0, s>>>(stack_mag, n, npix, threshold, threshold_is_f64, threshold64, min_count, mean, amp_disp, ps);
    else
        k_ps_block<0><<<grid, block, 0, s>>>(stack_mag, n, npix, threshold, threshold_is_f64, threshold64, min_count, mean, amp_disp, ps);
    return check_launch("k_ps_block");
}
