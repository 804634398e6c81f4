// Compressed SLC: compress (phase_link/_compress.py:11-65) on the GPU.
//
// One thread per full-resolution pixel, coalesced along columns for every SLC: the
// phase-linked phase of the pixel's block (nearest upsampling, utils.py:281-324),
// re-referenced if asked, projects the non-compressed SLCs; the magnitude is the given
// mean (or mean |z|), NaN where the projected phase is exactly 0.  HBM-bound: reads the
// stack once (8 B per SLC per pixel) and writes 8 B per pixel.
#include <cstdio>

#include "dpl_common.cuh"

namespace dpl {

struct CompressArgs {
    int n, rows, cols, pl_rows, pl_cols, ry, rx, first, has_ref, ref;
    const cfloat* slc;  // (n, rows, cols)
    const cfloat* pl;   // (n, pl_rows, pl_cols)
    float* mean;        // (rows, cols) in/out or null
    cfloat* out;        // (rows, cols)
};

__global__ void __launch_bounds__(256) k_compress(CompressArgs a) {
    const int64_t npix = (int64_t)a.rows * a.cols;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int r = (int)(p / a.cols), c = (int)(p - (int64_t)r * a.cols);
    // upsampled phase-linked pixel: identical shapes map 1:1, otherwise block repeats,
    // zero beyond them
    int64_t q = -1;
    if (a.pl_rows == a.rows && a.pl_cols == a.cols) {
        q = p;
    } else if (r < a.pl_rows * a.ry && c < a.pl_cols * a.rx) {
        q = (int64_t)(r / a.ry) * a.pl_cols + c / a.rx;
    }
    const int64_t plane = (int64_t)a.pl_rows * a.pl_cols;
    cfloat refc = cmake(1.f, 0.f);
    if (a.has_ref && q >= 0) refc = cconj(a.pl[(int64_t)a.ref * plane + q]);
    float sre = 0.f, sim = 0.f, msum = 0.f;
    for (int t = a.first; t < a.n; ++t) {
        const cfloat z = a.slc[(int64_t)t * npix + p];
        cfloat w = cmake(0.f, 0.f);
        if (q >= 0) {
            w = a.pl[(int64_t)t * plane + q];
            if (a.has_ref) w = cmul(w, refc);
        }
        const cfloat prod = cmulc(z, w);  // z conj(w)
        if (!cisnan(prod)) {
            sre += prod.re;
            sim += prod.im;
        }
        msum = t == a.first ? hypotf(z.re, z.im) : fadd(msum, hypotf(z.re, z.im));
    }
    const float phase = atan2f(sim, sre);
    float m = a.mean ? a.mean[p] : fdiv(msum, (float)(a.n - a.first));
    if (phase == 0.f) m = nanf("");
    if (a.mean) a.mean[p] = m;
    float sn, cs;
    sincosf(phase, &sn, &cs);
    a.out[p] = cmake(m * cs, m * sn);
}

}  // namespace dpl

using namespace dpl;

extern "C" dpl_status dpl_compress(const float* slc, int64_t nslc, int64_t rows, int64_t cols,
                                   const float* pl_cpx_phase, int64_t pl_rows, int64_t pl_cols,
                                   int first_real_slc_idx, float* slc_mean, int has_reference,
                                   int reference_idx, float* comp_slc, dpl_stream_t stream) {
    if (nslc <= 0 || rows < 0 || cols < 0 || pl_rows < 0 || pl_cols < 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_compress: bad shape");
    if (first_real_slc_idx < 0 || first_real_slc_idx > nslc)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_compress: first_real_slc_idx out of range");
    if (has_reference && (reference_idx < 0 || reference_idx >= nslc))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_compress: reference_idx out of range");
    if (rows * cols == 0) return DPL_OK;
    if (!slc || !pl_cpx_phase || !comp_slc) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_compress: null pointer");
    if (misaligned_c8(slc) || misaligned_c8(pl_cpx_phase) || misaligned_c8(comp_slc))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_compress: complex arrays must be 8-byte aligned");
    if (rows > INT32_MAX || cols > INT32_MAX) return fail(DPL_ERR_UNSUPPORTED, "dpl_compress: image too large");
    CompressArgs a{};
    a.n = (int)nslc;
    a.rows = (int)rows;
    a.cols = (int)cols;
    a.pl_rows = (int)pl_rows;
    a.pl_cols = (int)pl_cols;
    a.ry = pl_rows > 0 ? (int)(rows / pl_rows) : 0;
    a.rx = pl_cols > 0 ? (int)(cols / pl_cols) : 0;
    a.first = first_real_slc_idx;
    a.has_ref = has_reference != 0;
    a.ref = reference_idx;
    a.slc = reinterpret_cast<const cfloat*>(slc);
    a.pl = reinterpret_cast<const cfloat*>(pl_cpx_phase);
    a.mean = slc_mean;
    a.out = reinterpret_cast<cfloat*>(comp_slc);
    const int64_t npix = rows * cols;
    k_compress<<<(unsigned)ceil_div(npix, 256), 256, 0, (cudaStream_t)stream>>>(a);
    return check_launch("k_compress");
}
