// SHP-masked coherence matrices on the 5th-generation tensor cores (tcgen05).
//
// For a tile of 128 output pixels the sample covariance is one GEMM:
//
//     D[p][e] = sum_s  A[p][s] * B[e][s]
//
//   A[p][s]  0/1: sample s of the tile's input region lies in pixel p's (clamped)
//            window and is an SHP of p (exact in bf16)
//   B[e][s]  the real outputs of the per-sample outer product z(s) z(s)^H:
//            e <  N                  |z_i|^2                     (diagonal)
//            e =  N + 2o, N + 2o + 1 Re, Im of z_i conj(z_j) for the lower pair
//                                    o = i(i-1)/2 + j, i > j
//
// B is split into bf16 hi + lo parts (x = hi + lo + O(2^-17 x)); both products
// accumulate into one fp32 accumulator in tensor memory.  The N^2 real outputs are
// computed in passes of at most 512 TMEM columns, split at pair boundaries; the
// diagonal is in the first pass, so every pass is normalised on the fly
// (covariance.py:131-142: C = numer / sqrt(amp_i amp_j) where that is > 1e-6,
// evaluated as numer * r_i * r_j with r = 1 / sqrt(amp), valid where r_i r_j < 1e6).
//
// Pipeline per K chunk of 32 samples (16 warps, one CTA per SM, persistent):
//   the chunk's samples were prefetched into shared memory by cp.async while the
//   previous chunk was built; all warps build A (mask bits -> bf16) and B (products,
//   hi/lo split with paired conversions) into one of two stages in the canonical
//   K-major no-swizzle layout (8-row x 16-byte core matrices, LBO 128 B, SBO 512 B);
//   one thread issues the MMAs and commits them to the stage's mbarrier, and the
//   next build overlaps them.  Every wait is bounded.
// Epilogue: each warp reads 32 pixels x 32 columns from TMEM (tcgen05.ld), transposes
// through its own shared buffer and writes 128-byte rows of the planar output.
//
// Output: planar per pixel, Cg[p][0 .. N^2): diagonal, then (Re, Im) per lower pair.
#pragma once

#include <cuda_bf16.h>

namespace dpl {

constexpr int kTcM = 128;        // pixels per tile (MMA M)
constexpr int kTcKC = 32;        // samples per K chunk
constexpr int kTcThreads = 512;  // 16 warps
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kTcMaxPW = 512;    // TMEM columns per pass
constexpr int kTcMaxPass = 12;
constexpr int kTcTileR = 8, kTcTileC = 16;  // output pixels per tile (rows x cols), kTcTileR * kTcTileC = kTcM
constexpr int kTcTbufBytes = kTcWarps * 32 * 33 * 4;  // epilogue transpose buffers
constexpr uint32_t kTcWaitLimit = 1u << 26;

struct TcArgs {
    int n, rows, cols, hy, hx, sy, sx, out_rows, out_cols;
    int tile_r, tile_c, tiles_r, tiles_c;
    int region_r, region_c;  // max region extent of a tile
    int kpad;                // region samples padded to a multiple of kTcKC
    int npass;
    int pair0[kTcMaxPass + 1];  // pass p covers pairs [pair0[p], pair0[p+1]); pass 0 also the diagonal
    int pcols[kTcMaxPass];      // TMEM columns of pass p (multiple of 16)
    int ld_r;                   // row stride of the per-pixel r = 1/sqrt(amp) table (odd)
    const cfloat* zt;           // (rows, cols, n) masked, pixel-major
    const uint32_t* bits;       // (out_rows, out_cols, wy, wpr) or null (rectangular window)
    const uint8_t* nb_u8;       // alternative mask input (out_rows, out_cols, wy, wx)
    int wpr;
    float* Cg;                  // (out_rows * out_cols, n * n) planar output
    int32_t* counts;            // (out_rows * out_cols) or null
    int* status;
    // shared-memory carve (bytes from the 1024-aligned base)
    int off_stage, stage_bytes, stage_a_bytes, plane_bytes;
    int off_z, z_bytes, off_r, off_pair, off_mask, off_win, off_bar, smem_bytes;
};

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; swizzle none
    return d;
}

__device__ __forceinline__ uint32_t tc_idesc_bf16(int m, int nn) {
    uint32_t d = 0;
    d |= 1u << 4;   // D: f32
    d |= 1u << 7;   // A: bf16
    d |= 1u << 10;  // B: bf16
    d |= (uint32_t)(nn >> 3) << 17;
    d |= (uint32_t)(m >> 4) << 24;
    return d;
}

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool tc_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(tc_smem(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; returns false on timeout
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kTcWaitLimit; ++it)
        if (tc_try_wait(bar, parity)) return true;
    return false;
}

// byte offset of element (row, k) in a K-major no-swizzle tile with KC columns
__device__ __forceinline__ int tc_off(int row, int k) {
    return (row >> 3) * (kTcKC / 8 * 128) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// bf16 hi/lo split of two values, packed (first value in the low half)
__device__ __forceinline__ void tc_split2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// 8-byte asynchronous global -> shared copy; src_bytes = 0 writes zeros
__device__ __forceinline__ void tc_cp8(void* dst, const void* src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(tc_smem(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}

// Prefetch the samples of chunk `ch` (region samples [32 ch, 32 ch + 32)) into zs.
__device__ __forceinline__ void tc_prefetch(const TcArgs& a, cfloat* zs, int ch, int rr0, int cc0, int tid) {
    const int n = a.n;
    const int k0 = ch * kTcKC;
    for (int e = tid; e < kTcKC * n; e += kTcThreads) {
        const int k = e / n, t = e - k * n;
        const int sidx = k0 + k;
        const int ry = sidx / a.region_c, cx = sidx - ry * a.region_c;
        const int r = rr0 + ry, c = cc0 + cx;
        const bool in = ry < a.region_r && r < a.rows && c < a.cols;
        const cfloat* src = in ? a.zt + ((int64_t)r * a.cols + c) * n + t : a.zt;
        tc_cp8(zs + e, src, in ? 8 : 0);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void tc_ld32(uint32_t addr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kTcThreads, 1) k_cov_tc(TcArgs a) {
    extern __shared__ unsigned char tc_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = a.n, nn = n * n, wy = 2 * a.hy + 1, wx = 2 * a.hx + 1;
    const int O = n * (n - 1) / 2;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + a.off_bar);  // [0], [1]: stage MMA done
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + a.off_bar + 64);
    cfloat* const zb0 = reinterpret_cast<cfloat*>(sm + a.off_z);
    cfloat* const zb1 = reinterpret_cast<cfloat*>(sm + a.off_z + a.z_bytes);
    float* rtab = reinterpret_cast<float*>(sm + a.off_r);           // [128][ld_r]: 1/sqrt(amp_i)
    uint32_t* pairs = reinterpret_cast<uint32_t*>(sm + a.off_pair); // [O]: i | j << 16
    uint32_t* mask = reinterpret_cast<uint32_t*>(sm + a.off_mask);  // [128][wy][2]
    int* win = reinterpret_cast<int*>(sm + a.off_win);              // [128][2]: window origin in region

    for (int o = tid; o < O; o += kTcThreads) {
        int i = (int)((sqrtf(8.f * o + 1.f) + 1.f) * 0.5f);  // o = i(i-1)/2 + j, 0 <= j < i
        while (i * (i - 1) / 2 > o) --i;
        while ((i + 1) * i / 2 <= o) ++i;
        pairs[o] = (uint32_t)i | ((uint32_t)(o - i * (i - 1) / 2) << 16);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&bars[0])), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&bars[1])), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    constexpr int kAlloc = kTcMaxPW;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                     "r"(kAlloc));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    uint32_t phase[2] = {0u, 0u};
    uint32_t uses[2] = {0u, 0u};  // commits issued per stage (to know what to wait for)
    bool failed = false;
    const int nchunks = a.kpad / kTcKC;

    const int ntiles = a.tiles_r * a.tiles_c;
    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int tr0 = (tile / a.tiles_c) * kTcTileR, tc0 = (tile % a.tiles_c) * kTcTileC;
        // region origin: clamped window start of the tile's first output pixel
        const int rr0 = min(max(a.sy / 2 + tr0 * a.sy - a.hy, 0), a.rows - wy);
        const int cc0 = min(max(a.sx / 2 + tc0 * a.sx - a.hx, 0), a.cols - wx);
        // per-pixel window origin (in region coordinates) and mask bits
        if (tid < kTcM) {
            const int pr = tr0 + tid / kTcTileC, pc = tc0 + tid % kTcTileC;
            const bool ok = pr < a.out_rows && pc < a.out_cols;
            int cnt = 0;
            if (ok) {
                const int r0 = min(max(a.sy / 2 + pr * a.sy - a.hy, 0), a.rows - wy);
                const int c0 = min(max(a.sx / 2 + pc * a.sx - a.hx, 0), a.cols - wx);
                win[2 * tid] = r0 - rr0;
                win[2 * tid + 1] = c0 - cc0;
                const int64_t p = (int64_t)pr * a.out_cols + pc;
                const uint64_t full = wx >= 64 ? ~0ull : ((1ull << wx) - 1ull);
                for (int r = 0; r < wy; ++r) {
                    uint64_t m = full;
                    if (a.bits) {
                        const uint32_t* w = a.bits + (p * wy + r) * a.wpr;
                        m = w[0] | (a.wpr > 1 ? (uint64_t)w[1] << 32 : 0ull);
                        m &= full;
                    } else if (a.nb_u8) {
                        const uint8_t* b = a.nb_u8 + (p * wy + r) * wx;
                        m = 0;
                        for (int q = 0; q < wx; ++q) m |= (uint64_t)(b[q] != 0) << q;
                    }
                    mask[(tid * wy + r) * 2] = (uint32_t)m;
                    mask[(tid * wy + r) * 2 + 1] = (uint32_t)(m >> 32);
                    cnt += __popcll(m);
                }
                if (a.counts) a.counts[p] = cnt;
            } else {
                win[2 * tid] = -100000;  // never inside
                win[2 * tid + 1] = -100000;
            }
        }
        for (int pass = 0; pass < a.npass && !failed; ++pass) {
            const int pp0 = a.pair0[pass], npairs = a.pair0[pass + 1] - pp0;
            const int ndiag = pass == 0 ? n : 0;
            const int pcols = a.pcols[pass];
            const int gbase = pass == 0 ? 0 : n + 2 * pp0;  // output column of TMEM column 0
            const int gend = ndiag + 2 * npairs;            // TMEM columns holding outputs
            tc_prefetch(a, zb0, 0, rr0, cc0, tid);
            for (int ch = 0; ch < nchunks; ++ch) {
                const int s = ch & 1;
                unsigned char* sA = sm + a.off_stage + s * a.stage_bytes;
                unsigned char* sBh = sA + a.stage_a_bytes;
                unsigned char* sBl = sBh + a.plane_bytes;
                // wait until the MMAs that last read this stage are done
                if (uses[s] > 0) {
                    if (!tc_wait(&bars[s], phase[s])) failed = true;
                    phase[s] ^= 1u;
                    uses[s] = 0;
                }
                asm volatile("cp.async.wait_group 0;" ::: "memory");
                if (__syncthreads_or(failed)) {
                    failed = true;
                    break;
                }
                if (ch + 1 < nchunks) tc_prefetch(a, (ch & 1) ? zb0 : zb1, ch + 1, rr0, cc0, tid);
                const cfloat* zs = (ch & 1) ? zb1 : zb0;
                const int k0 = ch * kTcKC;
                // A: thread -> (pixel row, 8 samples)
                {
                    const int row = tid >> 2, g = tid & 3;
                    const int wr = win[2 * row], wc = win[2 * row + 1];
                    const int s0 = k0 + 8 * g;
                    int ry = s0 / a.region_c, cx = s0 - ry * a.region_c;
                    uint32_t w4[4];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int dr = ry - wr, dc = cx - wc;
                        uint32_t bit = 0u;
                        if (dr >= 0 && dr < wy && dc >= 0 && dc < wx && ry < a.region_r)
                            bit = (mask[(row * wy + dr) * 2 + (dc >> 5)] >> (dc & 31)) & 1u;
                        const uint32_t hv = bit ? 0x3F80u : 0u;  // bf16 1.0 or 0
                        if (q & 1) w4[q >> 1] |= hv << 16;
                        else w4[q >> 1] = hv;
                        if (++cx == a.region_c) {
                            cx = 0;
                            ++ry;
                        }
                    }
                    *reinterpret_cast<uint4*>(sA + tc_off(row, 8 * g)) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                }
                // B: tasks (diagonal i or pair o) x (8 samples), sample group outermost so
                // that a warp reads one group of samples
                {
                    const int units = ndiag + npairs;
                    for (int t = tid; t < 4 * units; t += kTcThreads) {
                        const int g = t / units, u = t - g * units;
                        const int kb = 8 * g;
                        uint4 hw, lw;
                        if (u < ndiag) {
                            float x[8];
#pragma unroll
                            for (int q = 0; q < 8; ++q) x[q] = cabs2(zs[(kb + q) * n + u]);
                            tc_split2(x[0], x[1], hw.x, lw.x);
                            tc_split2(x[2], x[3], hw.y, lw.y);
                            tc_split2(x[4], x[5], hw.z, lw.z);
                            tc_split2(x[6], x[7], hw.w, lw.w);
                            *reinterpret_cast<uint4*>(sBh + tc_off(u, kb)) = hw;
                            *reinterpret_cast<uint4*>(sBl + tc_off(u, kb)) = lw;
                        } else {
                            const int o = u - ndiag;
                            const uint32_t ij = pairs[pp0 + o];
                            const int i = ij & 0xffff, j = ij >> 16;
                            float re[8], im[8];
#pragma unroll
                            for (int q = 0; q < 8; ++q) {
                                const cfloat zi = zs[(kb + q) * n + i], zj = zs[(kb + q) * n + j];
                                re[q] = fmaf(zi.re, zj.re, zi.im * zj.im);    // Re z_i conj(z_j)
                                im[q] = fmaf(zi.im, zj.re, -(zi.re * zj.im));  // Im z_i conj(z_j)
                            }
                            const int col = ndiag + 2 * o;
                            tc_split2(re[0], re[1], hw.x, lw.x);
                            tc_split2(re[2], re[3], hw.y, lw.y);
                            tc_split2(re[4], re[5], hw.z, lw.z);
                            tc_split2(re[6], re[7], hw.w, lw.w);
                            *reinterpret_cast<uint4*>(sBh + tc_off(col, kb)) = hw;
                            *reinterpret_cast<uint4*>(sBl + tc_off(col, kb)) = lw;
                            tc_split2(im[0], im[1], hw.x, lw.x);
                            tc_split2(im[2], im[3], hw.y, lw.y);
                            tc_split2(im[4], im[5], hw.z, lw.z);
                            tc_split2(im[6], im[7], hw.w, lw.w);
                            *reinterpret_cast<uint4*>(sBh + tc_off(col + 1, kb)) = hw;
                            *reinterpret_cast<uint4*>(sBl + tc_off(col + 1, kb)) = lw;
                        }
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncthreads();
                if (tid == 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a_base = tc_smem(sA), b_hi = tc_smem(sBh), b_lo = tc_smem(sBl);
                    constexpr uint32_t LBO = 128, SBO = kTcKC / 8 * 128;
                    for (int kk = 0; kk < kTcKC; kk += 16) {
                        const uint64_t ad = tc_desc(a_base + (kk / 8) * LBO, LBO, SBO);
                        for (int n0 = 0; n0 < pcols; n0 += 256) {
                            const int nw = min(256, pcols - n0);
                            const uint32_t idesc = tc_idesc_bf16(kTcM, nw);
                            const uint32_t boff = (uint32_t)(n0 / 8) * SBO + (kk / 8) * LBO;
                            const uint32_t dt = tmem + (uint32_t)n0;
                            const uint32_t acc0 = (ch > 0 || kk > 0) ? 1u : 0u;
                            const uint64_t bh = tc_desc(b_hi + boff, LBO, SBO);
                            const uint64_t bl = tc_desc(b_lo + boff, LBO, SBO);
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
                                "l"(ad), "l"(bh), "r"(idesc), "r"(acc0));
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
                                "l"(ad), "l"(bl), "r"(idesc), "r"(1u));
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     tc_smem(&bars[s]))
                                 : "memory");
                }
                uses[s] = 1;
            }
            if (failed) break;
            // drain: wait for both stages' last MMAs (the accumulator is then complete)
            for (int s2 = 0; s2 < 2; ++s2) {
                if (uses[s2] > 0) {
                    if (!tc_wait(&bars[s2], phase[s2])) failed = true;
                    phase[s2] ^= 1u;
                    uses[s2] = 0;
                }
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (__syncthreads_or(failed)) {
                failed = true;
                break;
            }
            // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (pixels) and every
            // fourth group of 32 columns starting at group w / 4
            const int quarter = warp & 3, part = warp >> 2;
            const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
            float* tbuf = reinterpret_cast<float*>(sm + a.off_stage) + warp * (32 * 33);
            if (pass == 0) {
                // the diagonal (|z_i|^2 sums) is columns 0..n-1 of pass 0: r_i = 1 / sqrt(amp_i)
                if (part == 0) {
                    for (int c0 = 0; c0 < n; c0 += 32) {
                        uint32_t r[32];
                        tc_ld32(tmem + lane_base + (uint32_t)c0, r);
                        float* rrow = rtab + (quarter * 32 + lane) * a.ld_r;
#pragma unroll
                        for (int q = 0; q < 32; ++q)
                            if (c0 + q < n) rrow[c0 + q] = 1.f / sqrtf(__uint_as_float(r[q]));
                    }
                }
                __syncthreads();
            }
            for (int c0 = 32 * part; c0 < gend; c0 += 32 * 4) {
                uint32_t r[32];
                tc_ld32(tmem + lane_base + (uint32_t)c0, r);
                __syncwarp();
#pragma unroll
                for (int q = 0; q < 32; ++q) tbuf[lane * 33 + q] = __uint_as_float(r[q]);
                __syncwarp();
                // lane -> column c0 + lane and its (i, j)
                const int c = c0 + lane;
                int ci = 0, cj = 0;
                if (c < gend) {
                    if (c < ndiag) {
                        ci = cj = c;
                    } else {
                        const uint32_t ij = pairs[pp0 + ((c - ndiag) >> 1)];
                        ci = ij & 0xffff;
                        cj = ij >> 16;
                    }
                }
                for (int rr = 0; rr < 32; ++rr) {
                    const int pl = quarter * 32 + rr;
                    const int pr = tr0 + pl / kTcTileC, pc = tc0 + pl % kTcTileC;
                    if (pr < a.out_rows && pc < a.out_cols && c < gend) {
                        const float* rrow = rtab + pl * a.ld_r;
                        const float f = rrow[ci] * rrow[cj];
                        const float x = tbuf[rr * 33 + lane];
                        const int64_t p = (int64_t)pr * a.out_cols + pc;
                        a.Cg[p * nn + gbase + c] = f < 1e6f ? x * f : 0.f;
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (failed && tid == 0) atomicExch(a.status, (int)DPL_ERR_TIMEOUT);
    // before releasing TMEM make sure no MMA is still in flight (bounded)
    for (int s2 = 0; s2 < 2; ++s2)
        if (uses[s2] > 0) tc_wait(&bars[s2], phase[s2]);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kAlloc));
}

}  // namespace dpl
