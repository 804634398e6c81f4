// Statistically homogeneous pixel (SHP) selection.
//
// GLRT (shp/_glrt.py:13-130): the Rayleigh scale^2 = (var + mean^2)/2 is written to a
// pitched buffer, and each CTA stages its input region into shared memory with one
// TMA tiled copy (cp.async.bulk.tensor.2d, completion on an mbarrier with a bounded
// wait).  log(scale^2) is taken once per staged sample; each (pixel, offset) test
// needs one more log, of the pooled scale.  Window starts follow lax.dynamic_slice
// (clamped into the image: windows shift at the edges), validity follows the
// unclamped origin and the window centre is always False -- the reference's
// semantics.  The statistic is the reference's float32 expression
// nslc * (2*log(pooled) - log(s1) - log(s2)) without FMA contraction; its three logs
// cancel, so its rounding is a few 1e-6 of the cutoff.  Where it lands within 1e-5
// (relative) of the cutoff, the decision is taken on the same statistic evaluated in
// double precision as nslc * log1p((s1 - s2)^2 / (4 s1 s2)) (algebraically equal, no
// cancellation), so every mask bit is the exact comparison on the float32 scale^2.
//
// KS (shp/_ks.py:22-239): amplitudes are sorted per pixel (NaN last, like np.sort);
// each (pixel, neighbour) pair walks the two-sample merge exactly as
// _get_max_cdf_dist does.  The reference accumulates the ECDFs by repeated float64
// additions of 1/n, so after i steps an ECDF equals T[i] (the i-fold sum); the walk
// only needs the integer positions and a host-built table of the admissible
// partner range {i2 : |T[i1] - T[i2]| < cutoff}, an interval because T increases.
// The decision is therefore bit-identical to the float64 walk.
#include <cuda.h>

#include <algorithm>
#include <vector>

#include "dpl_common.cuh"
#include "shp.cuh"

namespace dpl {

// ---------------------------------------------------------------------------------
// TMA / mbarrier helpers (inline PTX)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

constexpr uint32_t kWaitLimit = 1u << 24;  // bounded mbarrier wait (iterations)

__device__ __forceinline__ int clamp_start(int center, int half, int size, int dim) {
    int s = center - half;
    s = s < 0 ? 0 : s;
    return s > dim - size ? dim - size : s;
}

// ---------------------------------------------------------------------------------
// GLRT
// ---------------------------------------------------------------------------------
__global__ void k_glrt_scale(const float* __restrict__ mean, const float* __restrict__ var, int64_t rows,
                             int64_t cols, int64_t pitch, float* __restrict__ scale2) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    int64_t r = i / cols, c = i - r * cols;
    float m = mean[i];
    scale2[r * pitch + c] = fdiv(fadd(var[i], fmul(m, m)), 2.f);
}

// One (pixel, offset) test: threshold > statistic, the float32 statistic refined in
// double precision near the cutoff (see above).  NaN statistics stay False.
__device__ __forceinline__ bool glrt_test(float s1, float s2, float l1, float l2, float nslc, float thr) {
    // (s1 + s2) / 2 == (s1 + s2) * 0.5 exactly in IEEE arithmetic
    const float pooled = fmul(fadd(s1, s2), 0.5f);
    const float stat = fmul(nslc, fsub(fsub(fmul(2.f, logf(pooled)), l1), l2));
    bool shp = thr > stat;
    if (fabsf(stat - thr) <= 1e-5f * thr) {
        const double d = (double)s1 - (double)s2;
        const double t = (double)nslc * log1p(d * d / (4.0 * (double)s1 * (double)s2));
        shp = (double)thr > t;
    }
    return shp;
}

template <bool kBits>
__global__ void __launch_bounds__(256) k_glrt(const __grid_constant__ CUtensorMap tmap, GlrtArgs a) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    // 128-byte aligned base (TMA destination), offset within the shared array so that
    // the accesses below stay shared-memory accesses
    const uint32_t mis = (uint32_t)__cvta_generic_to_shared(smem_raw) & 127u;
    float* raw = reinterpret_cast<float*>(smem_raw + ((128u - mis) & 127u));
    const int n_tile = a.box_w * a.box_h;
    float* lg = raw + n_tile;
    const int wy = 2 * a.hy + 1, wx = 2 * a.hx + 1;
    const int or0 = blockIdx.y * a.tile_r, oc0 = blockIdx.x * a.tile_c;
    const int or1 = min(or0 + a.tile_r, a.out_rows), oc1 = min(oc0 + a.tile_c, a.out_cols);
    const int rr0 = clamp_start(a.sy / 2 + or0 * a.sy, a.hy, wy, a.rows);
    const int cc0 = clamp_start(a.sx / 2 + oc0 * a.sx, a.hx, wx, a.cols);
    const int x0 = cc0 & ~3;  // TMA inner coordinate: multiple of 4 floats (16 bytes)
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, (uint32_t)(n_tile * sizeof(float)));
        tma_load_2d(raw, &tmap, x0, rr0, &bar);
    }
    bool timed_out = false;
    for (uint32_t spins = 0; !mbar_try_wait(&bar, 0);) {
        if (++spins > kWaitLimit) {
            timed_out = true;
            break;
        }
    }
    if (__syncthreads_or(timed_out)) {
        if (threadIdx.x == 0) {
            atomicExch(a.status, (int)DPL_ERR_TIMEOUT);
            // the copy may still be in flight: give it a second bounded wait before exit
            for (uint32_t more = 0; !mbar_try_wait(&bar, 0) && more < kWaitLimit; ++more) {
            }
        }
        __syncthreads();
        return;
    }
    for (int i = threadIdx.x; i < n_tile; i += blockDim.x) lg[i] = logf(raw[i]);
    __syncthreads();

    const float nslc = (float)a.nslc;
    const int W = wy * wx;
    if (!kBits) {
        // per output row of the tile: one item per (pixel, window row) computes the
        // row's wx bytes into shared memory (index arithmetic once per item, the valid
        // column range hoisted), then the row's contiguous segment of the output is
        // written with consecutive bytes per consecutive threads (coalesced)
        uint8_t* ob = reinterpret_cast<uint8_t*>(lg + n_tile);
        const int tc = oc1 - oc0;
        for (int orow = or0; orow < or1; ++orow) {
            const int in_r = a.sy / 2 + orow * a.sy;
            const int r0 = clamp_start(in_r, a.hy, wy, a.rows);
            const int ur0 = in_r - a.hy;
            for (int it = threadIdx.x; it < tc * wy; it += blockDim.x) {
                const int pix = it / wy, wa = it - pix * wy;
                const int in_c = a.sx / 2 + (oc0 + pix) * a.sx;
                const int c0 = clamp_start(in_c, a.hx, wx, a.cols);
                const int uc0 = in_c - a.hx;
                uint8_t* dst = ob + pix * W + wa * wx;
                const bool row_ok = (wa >= -ur0) && (wa < a.rows - ur0);
                // valid window columns of the unclamped origin
                const int wb0 = row_ok ? max(0, -uc0) : wx, wb1 = row_ok ? min(wx, a.cols - uc0) : wx;
                const int i1 = (in_r - rr0) * a.box_w + (in_c - x0);
                const float s1 = raw[i1], l1 = lg[i1];
                const float* rraw = raw + (r0 + wa - rr0) * a.box_w + (c0 - x0);
                const float* rlg = lg + (r0 + wa - rr0) * a.box_w + (c0 - x0);
                for (int wb = 0; wb < wx; ++wb) {
                    bool shp = false;
                    if (wb >= wb0 && wb < wb1 && !(wa == a.hy && wb == a.hx))
                        shp = glrt_test(s1, rraw[wb], l1, rlg[wb], nslc, a.thr);
                    dst[wb] = shp ? 1 : 0;
                }
            }
            __syncthreads();
            const int64_t seg0 = ((int64_t)orow * a.out_cols + oc0) * W;
            for (int k = threadIdx.x; k < tc * W; k += blockDim.x) a.is_shp[seg0 + k] = ob[k];
            __syncthreads();
        }
    } else {
        // one window row (<= 64 offsets) per iteration, packed into words_per_row words
        const int tc = oc1 - oc0;
        const int items = (or1 - or0) * tc * wy;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int wa = it % wy;
            const int pix = it / wy;
            const int orow = or0 + pix / tc, ocol = oc0 + pix % tc;
            const int in_r = a.sy / 2 + orow * a.sy, in_c = a.sx / 2 + ocol * a.sx;
            const int r0 = clamp_start(in_r, a.hy, wy, a.rows), c0 = clamp_start(in_c, a.hx, wx, a.cols);
            const int ur0 = in_r - a.hy, uc0 = in_c - a.hx;
            const bool row_ok = (wa >= -ur0) && (wa < a.rows - ur0);
            const int i1 = (in_r - rr0) * a.box_w + (in_c - x0);
            const float s1 = raw[i1], l1 = lg[i1];
            uint32_t w0 = 0, w1 = 0;
            if (row_ok) {
                const float* rraw = raw + (r0 + wa - rr0) * a.box_w + (c0 - x0);
                const float* rlg = lg + (r0 + wa - rr0) * a.box_w + (c0 - x0);
                for (int wb = 0; wb < wx; ++wb) {
                    const bool valid = (wb >= -uc0) && (wb < a.cols - uc0) && !(wa == a.hy && wb == a.hx);
                    if (!valid) continue;
                    if (glrt_test(s1, rraw[wb], l1, rlg[wb], nslc, a.thr)) {
                        if (wb < 32) w0 |= 1u << wb;
                        else w1 |= 1u << (wb - 32);
                    }
                }
            }
            uint32_t* dst = a.bits + (((int64_t)orow * a.out_cols + ocol) * wy + wa) * a.words_per_row;
            dst[0] = w0;
            if (a.words_per_row > 1) dst[1] = w1;
        }
    }
}

// ---------------------------------------------------------------------------------
// KS
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool nan_last_greater(float a, float b) {
    // np.sort order: NaN after every number
    return (isnan(a) && !isnan(b)) || a > b;
}

template <int NMAX>
__global__ void __launch_bounds__(128) k_sort_pixels(const float* __restrict__ in, int n, int64_t npix,
                                                     float* __restrict__ out) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float v[NMAX];
#pragma unroll
    for (int t = 0; t < NMAX; ++t) v[t] = t < n ? in[(int64_t)t * npix + p] : __int_as_float(0x7fc00000);
    // odd-even transposition sort (NMAX passes) on a fixed-size register array; the
    // padding NaNs sort to the end and are never stored
#pragma unroll
    for (int pass = 0; pass < NMAX; ++pass) {
#pragma unroll
        for (int i = pass & 1; i + 1 < NMAX; i += 2) {
            float x = v[i], y = v[i + 1];
            bool sw = nan_last_greater(x, y);
            v[i] = sw ? y : x;
            v[i + 1] = sw ? x : y;
        }
    }
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n) out[(int64_t)t * npix + p] = v[t];
}

__global__ void __launch_bounds__(256) k_ks(KsArgs a) {
    extern __shared__ float ks_smem[];
    // layout: lo[n+1], hi[n+1] (int), then the staged sorted samples [region][n]
    int* lo = reinterpret_cast<int*>(ks_smem);
    int* hi = lo + (a.n + 1);
    float* samp = reinterpret_cast<float*>(hi + (a.n + 1));
    const int n = a.n;
    for (int i = threadIdx.x; i <= n; i += blockDim.x) {
        lo[i] = a.lo[i];
        hi[i] = a.hi[i];
    }
    const int wy = 2 * a.hy + 1, wx = 2 * a.hx + 1;
    const int or0 = blockIdx.y * a.tile_r, oc0 = blockIdx.x * a.tile_c;
    const int or1 = min(or0 + a.tile_r, a.out_rows), oc1 = min(oc0 + a.tile_c, a.out_cols);
    // input region of the (unclamped) windows, intersected with the image
    const int rr0 = max(0, a.sy / 2 + or0 * a.sy - a.hy), cc0 = max(0, a.sx / 2 + oc0 * a.sx - a.hx);
    const int rr1 = min(a.rows, a.sy / 2 + (or1 - 1) * a.sy + a.hy + 1);
    const int cc1 = min(a.cols, a.sx / 2 + (oc1 - 1) * a.sx + a.hx + 1);
    const int rw = cc1 - cc0, rh = rr1 - rr0;
    for (int i = threadIdx.x; i < rw * rh * n; i += blockDim.x) {
        const int pix = i % (rw * rh), t = i / (rw * rh);  // pixel-fastest: coalesced reads
        const int r = rr0 + pix / rw, c = cc0 + pix % rw;
        samp[pix * n + t] = a.sorted[((int64_t)t * a.rows + r) * a.cols + c];
    }
    __syncthreads();
    const int W = wy * wx;
    const int tc = oc1 - oc0;
    const int items = (or1 - or0) * tc * W;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int off = it % W, pix = it / W;
        const int orow = or0 + pix / tc, ocol = oc0 + pix % tc;
        const int in_r = a.sy / 2 + orow * a.sy, in_c = a.sx / 2 + ocol * a.sx;
        const int wa = off / wx, wb = off - wa * wx;
        bool shp = false;
        const bool full = in_r - a.hy >= 0 && in_r + a.hy + 1 <= a.rows && in_c - a.hx >= 0 &&
                          in_c + a.hx + 1 <= a.cols;
        if (full && !(wa == a.hy && wb == a.hx)) {
            const float* x1 = samp + ((in_r - rr0) * rw + (in_c - cc0)) * n;
            const float* x2 = samp + ((in_r - a.hy + wa - rr0) * rw + (in_c - a.hx + wb - cc0)) * n;
            int i1 = 0, i2 = 0;
            shp = true;
            for (int iout = 0; iout < 2 * n;) {
                if (i1 == n) {
                    ++i2;
                } else if (i2 == n || x1[i1] < x2[i2]) {
                    ++i1;
                } else if (x1[i1] > x2[i2]) {
                    ++i2;
                } else {  // a tie (or a comparison with NaN): both step
                    ++i1;
                    ++i2;
                    ++iout;
                }
                ++iout;
                if (i2 < lo[i1] || i2 > hi[i1]) {
                    shp = false;
                    break;
                }
            }
        }
        a.is_shp[((int64_t)orow * a.out_cols + ocol) * W + off] = shp ? 1 : 0;
    }
}

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

int64_t glrt_pitch(int64_t cols) { return (cols + 3) / 4 * 4; }

size_t glrt_workspace_size(int64_t rows, int64_t cols) {
    return align_up(256, 256) + align_up((size_t)rows * glrt_pitch(cols) * sizeof(float), 256);
}

dpl_status launch_glrt(const float* mean, const float* var, int64_t rows, int64_t cols, int hy, int hx, int sy,
                       int sx, int nslc, float threshold, uint8_t* is_shp, uint32_t* bits, int* status,
                       float* scale2, cudaStream_t s) {
    const int wy = 2 * hy + 1, wx = 2 * hx + 1;
    if (wy > rows || wx > cols) return fail(DPL_ERR_INVALID_ARGUMENT, "GLRT window larger than the image");
    if (bits && wx > 64) return fail(DPL_ERR_UNSUPPORTED, "packed GLRT masks need 2*hx+1 <= 64");
    const int64_t pitch = glrt_pitch(cols);
    const int64_t npix = rows * cols;
    k_glrt_scale<<<ceil_div(npix, 256), 256, 0, s>>>(mean, var, rows, cols, pitch, scale2);
    DPL_CUDA_TRY(cudaGetLastError());

    GlrtArgs a{};
    a.rows = (int)rows;
    a.cols = (int)cols;
    a.hy = hy;
    a.hx = hx;
    a.sy = sy;
    a.sx = sx;
    a.out_rows = (int)(rows / sy);
    a.out_cols = (int)(cols / sx);
    a.nslc = nslc;
    a.thr = threshold;
    a.is_shp = is_shp;
    a.bits = bits;
    a.words_per_row = wx > 32 ? 2 : 1;
    a.status = status;
    if (a.out_rows == 0 || a.out_cols == 0) return DPL_OK;
    // pick the largest tile whose TMA box fits the 256-element box limit and ~96 KB smem
    int tr = 16, tc = 32;
    auto box_w = [&](int t) { return (int)((((int64_t)(t - 1) * sx + wx + 3) + 3) / 4 * 4); };
    auto box_h = [&](int t) { return (t - 1) * sy + wy; };
    while (tc > 1 && box_w(tc) > 256) tc /= 2;
    while (tr > 1 && box_h(tr) > 256) tr /= 2;
    while ((size_t)2 * box_w(tc) * box_h(tr) * 4 > 96 * 1024 && (tr > 1 || tc > 1)) {
        if (tr >= tc && tr > 1) tr /= 2;
        else tc /= 2;
    }
    if (box_w(tc) > 256 || box_h(tr) > 256) return fail(DPL_ERR_UNSUPPORTED, "GLRT window too large for a TMA box");
    a.tile_r = tr;
    a.tile_c = tc;
    a.box_w = box_w(tc);
    a.box_h = box_h(tr);

    EncodeTiledFn enc = get_encode_fn();
    if (!enc) return fail(DPL_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    CUtensorMap map;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(pitch * sizeof(float))};
    cuuint32_t box[2] = {(cuuint32_t)a.box_w, (cuuint32_t)a.box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, scale2, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(DPL_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    // staged scale^2 and its log, then one output row of byte masks
    size_t smem = (size_t)2 * a.box_w * a.box_h * sizeof(float) + 128 + (bits ? 0 : (size_t)tc * wy * wx);
    if (smem > (size_t)227 * 1024) return fail(DPL_ERR_UNSUPPORTED, "GLRT window too large for shared memory");
    dim3 grid(ceil_div(a.out_cols, tc), ceil_div(a.out_rows, tr));
    if (bits) {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_glrt<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_glrt<true><<<grid, 256, smem, s>>>(map, a);
    } else {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_glrt<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_glrt<false><<<grid, 256, smem, s>>>(map, a);
    }
    return check_launch("k_glrt");
}

}  // namespace dpl

using namespace dpl;

extern "C" size_t dpl_shp_glrt_workspace_size(int64_t rows, int64_t cols) { return glrt_workspace_size(rows, cols); }

extern "C" dpl_status dpl_shp_glrt(const float* mean, const float* var, int64_t rows, int64_t cols, int hy, int hx,
                                   int sy, int sx, int nslc, float threshold, uint8_t* is_shp, void* workspace,
                                   size_t workspace_bytes, dpl_stream_t stream) {
    if (rows <= 0 || cols <= 0 || hy < 0 || hx < 0 || sy <= 0 || sx <= 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_shp_glrt: bad shape");
    if (rows > INT32_MAX || cols > INT32_MAX) return fail(DPL_ERR_UNSUPPORTED, "dpl_shp_glrt: image too large");
    if (!mean || !var || !is_shp || !workspace) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_shp_glrt: null pointer");
    if (workspace_bytes < glrt_workspace_size(rows, cols))
        return fail(DPL_ERR_WORKSPACE, "dpl_shp_glrt: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    Workspace ws{(char*)workspace, workspace_bytes};
    int* status = ws.take<int>(64);
    float* scale2 = ws.take<float>((size_t)rows * glrt_pitch(cols));
    DPL_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
    return launch_glrt(mean, var, rows, cols, hy, hx, sy, sx, nslc, threshold, is_shp, nullptr, status, scale2, s);
}

size_t dpl::ks_workspace_size(int64_t nslc, int64_t rows, int64_t cols) {
    return 256 + align_up((size_t)(2 * (nslc + 1)) * sizeof(int), 256) +
           align_up((size_t)nslc * rows * cols * sizeof(float), 256);
}

extern "C" size_t dpl_shp_ks_workspace_size(int64_t nslc, int64_t rows, int64_t cols) {
    return ks_workspace_size(nslc, rows, cols);
}

extern "C" dpl_status dpl_shp_ks(const float* amp_stack, int64_t nslc, int64_t rows, int64_t cols, int hy, int hx,
                                 int sy, int sx, double cutoff, int is_sorted, uint8_t* is_shp, void* workspace,
                                 size_t workspace_bytes, dpl_stream_t stream) {
    if (nslc <= 0 || rows <= 0 || cols <= 0 || hy < 0 || hx < 0 || sy <= 0 || sx <= 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_shp_ks: bad shape");
    if (nslc > kMaxNslc) return fail(DPL_ERR_UNSUPPORTED, "dpl_shp_ks: nslc > 64");
    if (rows > INT32_MAX || cols > INT32_MAX) return fail(DPL_ERR_UNSUPPORTED, "dpl_shp_ks: image too large");
    if (!amp_stack || !is_shp || !workspace) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_shp_ks: null pointer");
    if (workspace_bytes < ks_workspace_size(nslc, rows, cols))
        return fail(DPL_ERR_WORKSPACE, "dpl_shp_ks: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)nslc;
    const int wy = 2 * hy + 1, wx = 2 * hx + 1;
    const int out_rows = (int)(rows / sy), out_cols = (int)(cols / sx);
    if (out_rows == 0 || out_cols == 0) return DPL_OK;
    // ECDF tables: T[k] = k-fold float64 sum of 1/n; admissible partner interval per i1
    std::vector<double> T(n + 1, 0.0);
    const double step = 1.0 / n;
    for (int k = 1; k <= n; ++k) T[k] = T[k - 1] + step;
    std::vector<int> lo(n + 1), hi(n + 1);
    for (int i1 = 0; i1 <= n; ++i1) {
        int l = n + 1, h = -1;
        for (int i2 = 0; i2 <= n; ++i2) {
            if (std::fabs(T[i1] - T[i2]) < cutoff) {
                l = std::min(l, i2);
                h = std::max(h, i2);
            }
        }
        lo[i1] = l;
        hi[i1] = h;
    }
    Workspace ws{(char*)workspace, workspace_bytes};
    int* tables = ws.take<int>(2 * (n + 1));
    float* sorted = ws.take<float>((size_t)n * rows * cols);
    std::vector<int> host(2 * (n + 1));
    std::copy(lo.begin(), lo.end(), host.begin());
    std::copy(hi.begin(), hi.end(), host.begin() + (n + 1));
    // pageable source: cudaMemcpyAsync stages it before returning
    DPL_CUDA_TRY(cudaMemcpyAsync(tables, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    const int64_t npix = rows * cols;
    const float* src = amp_stack;
    if (!is_sorted) {
        dim3 g(ceil_div(npix, 128));
        if (n <= 16) k_sort_pixels<16><<<g, 128, 0, s>>>(amp_stack, n, npix, sorted);
        else if (n <= 32) k_sort_pixels<32><<<g, 128, 0, s>>>(amp_stack, n, npix, sorted);
        else k_sort_pixels<64><<<g, 128, 0, s>>>(amp_stack, n, npix, sorted);
        DPL_CUDA_TRY(cudaGetLastError());
        src = sorted;
    }
    KsArgs a{};
    a.sorted = src;
    a.lo = tables;
    a.hi = tables + (n + 1);
    a.n = n;
    a.rows = (int)rows;
    a.cols = (int)cols;
    a.hy = hy;
    a.hx = hx;
    a.sy = sy;
    a.sx = sx;
    a.out_rows = out_rows;
    a.out_cols = out_cols;
    a.is_shp = is_shp;
    int tr = 8, tc = 16;
    auto smem_for = [&](int r, int c) {
        size_t rh = (size_t)(r - 1) * sy + wy, rw = (size_t)(c - 1) * sx + wx;
        return 2 * (n + 1) * sizeof(int) + rh * rw * n * sizeof(float);
    };
    while (smem_for(tr, tc) > 96 * 1024 && (tr > 1 || tc > 1)) {
        if (tc >= tr && tc > 1) tc /= 2;
        else tr /= 2;
    }
    if (smem_for(tr, tc) > 200 * 1024) return fail(DPL_ERR_UNSUPPORTED, "dpl_shp_ks: window too large");
    a.tile_r = tr;
    a.tile_c = tc;
    size_t smem = smem_for(tr, tc);
    DPL_CUDA_TRY(cudaFuncSetAttribute(k_ks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_ks<<<dim3(ceil_div(out_cols, tc), ceil_div(out_rows, tr)), 256, smem, s>>>(a);
    return check_launch("k_ks");
}
