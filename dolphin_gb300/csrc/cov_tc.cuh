// SHP-masked coherence matrices on the 5th-generation tensor cores (tcgen05).
//
// For a tile of 128 output pixels the sample covariance is one GEMM:
//
//     D[p][e] = sum_s  A[p][s] * B[e][s]
//
//   A[p][s]  0/1: sample s of the tile's input region lies in pixel p's (clamped)
//            window and is an SHP of p (exact in bf16)
//   B[e][s]  the real output e of the per-sample outer product z(s) z(s)^H:
//            e <  N          Re z_i conj(z_i) = |z_i|^2            (diagonal)
//            e <  N + O      Re z_i conj(z_j)  for i > j            (O = N(N-1)/2)
//            e <  N + 2O     Im z_i conj(z_j)  for i > j
//
// B is split into bf16 hi + lo parts (x = hi + lo + O(2^-17 x)); both products
// accumulate into one fp32 accumulator in tensor memory.  The N^2 real outputs are
// computed in passes of at most 512 TMEM columns (2 passes for N <= 31); the
// diagonal is in the first pass, so every pass can be normalised on the fly
// (covariance.py:131-142: C = numer / sqrt(amp_i amp_j) where that is > 1e-6).
//
// Shared-memory operands use the canonical K-major, no-swizzle layout: 8-row x
// 16-byte core matrices, LBO = 128 B between core matrices along K, SBO = 512 B
// (KC = 32) between 8-row groups.  Two stages are double buffered: the CTA builds
// chunk k+1 while the MMAs of chunk k run; one thread issues the MMAs and commits
// them to the stage's mbarrier.  Every wait is bounded.
//
// Output: planar per pixel, Cg[p][0 .. N^2) in the column order above.
#pragma once

#include <cuda_bf16.h>

namespace dpl {

constexpr int kTcM = 128;        // pixels per tile (MMA M)
constexpr int kTcKC = 32;        // samples per K chunk
constexpr int kTcThreads = 256;  // 8 warps
constexpr int kTcMaxPW = 512;    // TMEM columns per pass
constexpr uint32_t kTcWaitLimit = 1u << 26;

struct TcArgs {
    int n, rows, cols, hy, hx, sy, sx, out_rows, out_cols;
    int tile_r, tile_c, tiles_r, tiles_c;
    int region_r, region_c;  // max region extent of a tile
    int kpad;                // region samples padded to a multiple of kTcKC
    int npass, pw;           // passes and columns per pass (multiple of 16)
    const cfloat* zt;        // (rows, cols, n) masked, pixel-major
    const uint32_t* bits;    // (out_rows, out_cols, wy, wpr) or null (rectangular window)
    const uint8_t* nb_u8;    // alternative mask input (out_rows, out_cols, wy, wx)
    int wpr;
    float* Cg;               // (out_rows * out_cols, n * n) planar output
    int32_t* counts;         // (out_rows * out_cols) or null
    int* status;
    // shared-memory carve (bytes from the aligned base)
    int off_stage0, off_stage1, stage_a_bytes, stage_b_bytes;
    int off_z, off_amp, off_col, off_mask, off_win, off_bar, smem_bytes;
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

__device__ __forceinline__ uint32_t bf16x2(float lo_elem, float hi_elem) {
    const uint32_t a = __bfloat16_as_ushort(__float2bfloat16_rn(lo_elem));
    const uint32_t b = __bfloat16_as_ushort(__float2bfloat16_rn(hi_elem));
    return a | (b << 16);
}

__global__ void __launch_bounds__(kTcThreads, 1) k_cov_tc(TcArgs a) {
    extern __shared__ unsigned char tc_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = a.n, nn = n * n, wy = 2 * a.hy + 1, wx = 2 * a.hx + 1;
    const int O = n * (n - 1) / 2;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + a.off_bar);  // [0], [1]: stage MMA done
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + a.off_bar + 64);
    cfloat* zs = reinterpret_cast<cfloat*>(sm + a.off_z);          // [kTcKC][n]
    float* amp = reinterpret_cast<float*>(sm + a.off_amp);          // [128][n+1]
    uint32_t* colmap = reinterpret_cast<uint32_t*>(sm + a.off_col); // [npass*pw]: i | j<<8 | kind<<16
    uint32_t* mask = reinterpret_cast<uint32_t*>(sm + a.off_mask);  // [128][wy][2]
    int* win = reinterpret_cast<int*>(sm + a.off_win);              // [128][2]: window origin in region

    // column map and barriers
    for (int c = tid; c < a.npass * a.pw; c += blockDim.x) {
        uint32_t v;
        if (c < n) {
            v = (uint32_t)c | ((uint32_t)c << 8) | (0u << 16);
        } else if (c < n + 2 * O) {
            const int o = (c - n) % (O > 0 ? O : 1);
            int i = (int)((sqrtf(8.f * o + 1.f) + 1.f) * 0.5f);  // o = i(i-1)/2 + j
            while (i * (i - 1) / 2 > o) --i;
            while ((i + 1) * i / 2 <= o) ++i;
            const int j = o - i * (i - 1) / 2;
            v = (uint32_t)i | ((uint32_t)j << 8) | ((c < n + O ? 1u : 2u) << 16);
        } else {
            v = 3u << 16;  // padding
        }
        colmap[c] = v;
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&bars[0])), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&bars[1])), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const int ncols_alloc = a.pw <= 256 ? 256 : 512;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                     "r"(ncols_alloc));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    uint32_t phase[2] = {0u, 0u};
    uint32_t uses[2] = {0u, 0u};  // commits issued per stage (to know what to wait for)
    bool failed = false;

    const int ntiles = a.tiles_r * a.tiles_c;
    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int tr0 = (tile / a.tiles_c) * a.tile_r, tc0 = (tile % a.tiles_c) * a.tile_c;
        // region origin: clamped window start of the tile's first output pixel
        const int rr0 = min(max(a.sy / 2 + tr0 * a.sy - a.hy, 0), a.rows - wy);
        const int cc0 = min(max(a.sx / 2 + tc0 * a.sx - a.hx, 0), a.cols - wx);
        // per-pixel window origin (in region coordinates) and mask bits
        if (tid < kTcM) {
            const int pr = tr0 + tid / a.tile_c, pc = tc0 + tid % a.tile_c;
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
        __syncthreads();
        const int nchunks = a.kpad / kTcKC;
        for (int pass = 0; pass < a.npass && !failed; ++pass) {
            for (int ch = 0; ch < nchunks; ++ch) {
                const int s = ch & 1;
                unsigned char* stage = sm + (s ? a.off_stage1 : a.off_stage0);
                unsigned char* sA = stage;
                unsigned char* sB = stage + a.stage_a_bytes;
                // wait until the MMAs that last read this stage are done
                if (uses[s] > 0) {
                    if (!tc_wait(&bars[s], phase[s])) failed = true;
                    phase[s] ^= 1u;
                    uses[s] = 0;
                }
                if (__syncthreads_or(failed)) {
                    failed = true;
                    break;
                }
                // stage the chunk's samples: zs[k][t]
                const int k0 = ch * kTcKC;
                for (int e = tid; e < kTcKC * n; e += blockDim.x) {
                    const int k = e / n, t = e - k * n;
                    const int sidx = k0 + k;
                    const int ry = sidx / a.region_c, cx = sidx - ry * a.region_c;
                    const int r = rr0 + ry, c = cc0 + cx;
                    cfloat z = cmake(0.f, 0.f);
                    if (ry < a.region_r && r < a.rows && c < a.cols) z = a.zt[((int64_t)r * a.cols + c) * n + t];
                    zs[k * n + t] = z;
                }
                __syncthreads();
                // A: mask rows (thread -> pixel row, half of the chunk)
                {
                    const int row = tid >> 1, half = tid & 1;
                    const int wr = win[2 * row], wc = win[2 * row + 1];
                    for (int g = 0; g < 2; ++g) {
                        const int kb = half * 16 + g * 8;
                        uint32_t w4[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            float v2[2];
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const int sidx = k0 + kb + 2 * q + h;
                                const int ry = sidx / a.region_c, cx = sidx - ry * a.region_c;
                                const int dr = ry - wr, dc = cx - wc;
                                float mv = 0.f;
                                if (dr >= 0 && dr < wy && dc >= 0 && dc < wx && ry < a.region_r) {
                                    const uint32_t wd = mask[(row * wy + dr) * 2 + (dc >> 5)];
                                    mv = ((wd >> (dc & 31)) & 1u) ? 1.f : 0.f;
                                }
                                v2[h] = mv;
                            }
                            w4[q] = bf16x2(v2[0], v2[1]);
                        }
                        *reinterpret_cast<uint4*>(sA + tc_off(row, kb)) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                    }
                }
                // B: hi and lo planes, rows = this pass's output columns
                for (int e = tid; e < a.pw; e += blockDim.x) {
                    const uint32_t cm = colmap[pass * a.pw + e];
                    const int i = cm & 0xff, j = (cm >> 8) & 0xff, kind = cm >> 16;
                    for (int kb = 0; kb < kTcKC; kb += 8) {
                        float hv[8], lv[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            float x = 0.f;
                            if (kind < 3) {
                                const cfloat zi = zs[(kb + q) * n + i], zj = zs[(kb + q) * n + j];
                                x = kind == 2 ? (zi.im * zj.re - zi.re * zj.im) : (zi.re * zj.re + zi.im * zj.im);
                            }
                            const __nv_bfloat16 hb = __float2bfloat16_rn(x);
                            hv[q] = __bfloat162float(hb);
                            lv[q] = x - hv[q];
                        }
                        uint4 hw = make_uint4(bf16x2(hv[0], hv[1]), bf16x2(hv[2], hv[3]), bf16x2(hv[4], hv[5]),
                                              bf16x2(hv[6], hv[7]));
                        uint4 lw = make_uint4(bf16x2(lv[0], lv[1]), bf16x2(lv[2], lv[3]), bf16x2(lv[4], lv[5]),
                                              bf16x2(lv[6], lv[7]));
                        *reinterpret_cast<uint4*>(sB + tc_off(e, kb)) = hw;
                        *reinterpret_cast<uint4*>(sB + a.stage_b_bytes / 2 + tc_off(e, kb)) = lw;
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncthreads();
                if (tid == 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a_base = tc_smem(sA), b_hi = tc_smem(sB), b_lo = b_hi + a.stage_b_bytes / 2;
                    constexpr uint32_t LBO = 128, SBO = kTcKC / 8 * 128;
                    for (int kk = 0; kk < kTcKC; kk += 16) {
                        const uint64_t ad = tc_desc(a_base + (kk / 8) * LBO, LBO, SBO);
                        for (int n0 = 0; n0 < a.pw; n0 += 256) {
                            const int nw = min(256, a.pw - n0);
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
            // epilogue: warps 0-3 own TMEM lanes 0-127 (one pixel each)
            float* stagef = reinterpret_cast<float*>(sm + a.off_stage0);  // [128][33]
            const int p_loc = tid & 127;
            const int pr = tr0 + p_loc / a.tile_c, pc = tc0 + p_loc % a.tile_c;
            const bool pix_ok = pr < a.out_rows && pc < a.out_cols;
            for (int c0 = 0; c0 < a.pw; c0 += 32) {
                if (warp < 4) {
                    uint32_t r[32];
                    const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                          "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                        : "r"(addr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (pass == 0 && c0 == 0) {
                        // the diagonal (|z_i|^2 sums) is columns 0..n-1 of pass 0 (n <= 64 <= pw)
                        for (int q = 0; q < 32; ++q)
                            if (q < n) amp[p_loc * (n + 1) + q] = __uint_as_float(r[q]);
                    }
                    if (pass == 0 && c0 == 32 && n > 32) {
                        for (int q = 0; q < 32; ++q)
                            if (32 + q < n) amp[p_loc * (n + 1) + 32 + q] = __uint_as_float(r[q]);
                    }
                    for (int q = 0; q < 32; ++q) stagef[p_loc * 33 + q] = __uint_as_float(r[q]);
                }
                __syncthreads();
                // normalise and store: each warp writes 16 pixel rows x 32 columns (coalesced)
                for (int rr = warp; rr < kTcM; rr += 8) {
                    const int pr2 = tr0 + rr / a.tile_c, pc2 = tc0 + rr % a.tile_c;
                    const int c = c0 + lane;
                    const int gc = pass * a.pw + c;
                    if (pr2 < a.out_rows && pc2 < a.out_cols && c < a.pw && gc < nn) {
                        const uint32_t cm = colmap[gc];
                        const int i = cm & 0xff, j = (cm >> 8) & 0xff;
                        const float ai = amp[rr * (n + 1) + i], aj = amp[rr * (n + 1) + j];
                        const float sq = fsqrt(fmul(ai, aj));
                        const float x = stagef[rr * 33 + lane];
                        const int64_t p = (int64_t)pr2 * a.out_cols + pc2;
                        a.Cg[p * nn + gc] = sq > 1e-6f ? fdiv(x, sq) : 0.f;
                    }
                }
                __syncthreads();
            }
            (void)pix_ok;
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
    }
    if (failed && tid == 0) atomicExch(a.status, (int)DPL_ERR_TIMEOUT);
    // before releasing TMEM make sure no MMA is still in flight (bounded)
    for (int s2 = 0; s2 < 2; ++s2)
        if (uses[s2] > 0) tc_wait(&bars[s2], phase[s2]);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_alloc));
}

}  // namespace dpl
