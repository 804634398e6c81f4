// SHP-masked coherence matrices on the 5th-generation tensor cores (tcgen05).
//
// For a tile of 16 x 16 output pixels the sample covariance is one GEMM:
//
//     D[e][p] = sum_s  KR[e][s] * M[p][s]
//
//   KR[e][s]  the real components of the per-sample outer product z(s) z(s)^H
//             (Khatri-Rao rows, the MMA's A operand, 128 rows per M tile):
//             |z_i|^2 (diagonal), Re and Im of z_i conj(z_j) for each lower pair i > j
//   M[p][s]   0/1: sample s of the tile's input region lies in pixel p's (clamped)
//             window and is an SHP of p (the B operand, N = 256 pixels; exact in bf16)
//
// KR is split into bf16 hi + lo parts (x = hi + lo + O(2^-17 x)); both products
// accumulate into one fp32 accumulator in tensor memory.  The TF32 form (kTf) stores KR
// once, rounded to tf32 (x (1 + O(2^-11))), with a tf32 mask, and issues kind::tf32
// MMAs (8 samples each); its stages are 64 KB, so two of them fit.  A pass fills two M tiles
// (2 x 256 TMEM columns) row by row: in pass 0 rows 0 .. N-1 of M tile 0 hold the
// diagonal; every other used row holds one lower pair, its real part in M tile 0 and
// its imaginary part in the same row of M tile 1, so one builder thread forms both
// from one pair of sample loads.  kTcRows = 128 rows per pass keep the Khatri-Rao work
// of a K chunk at one item per builder thread.  The kernel writes the sums unnormalised
// (its shared memory goes to a third operand stage); the readers of the planar matrices
// normalise them as covariance.py:131-142 does (C = numer / sqrt(amp_i amp_j) where that
// is > 1e-6, evaluated as numer * r_i * r_j with r = 1 / sqrt(amp), and 0 where
// r_i r_j >= 1e6).
//
// Per tile the masks are turned once into per-pixel bit arrays over the region's
// samples.  Per K chunk of 32 samples, warps 0-16 (builders) form the KR rows of the
// pass from the chunk's samples (prefetched into shared memory while the previous
// chunk was built), expand the chunk's mask bits to bf16 and signal the stage's
// `full` mbarrier (three operand stages where shared memory allows, else two); warp 17
// waits on it, issues the MMAs (canonical K-major no-swizzle
// layout: 8-row x 16-byte core matrices, LBO 128 B, SBO 512 B) and commits them to the
// stage's `empty` mbarrier, which the builders wait on before reusing the stage.
// Every wait is bounded.
// Epilogue: TMEM lane = row, column = pixel, so each pair of tcgen05.ld rows gives the
// (Re, Im) sums of one pair for 16 pixels, written as coalesced float2 stores.
//
// Output: planar per pixel, Cg[p][0 .. N^2): diagonal, then (Re, Im) per lower pair.
#pragma once

#include <cuda_bf16.h>

#include "tc_common.cuh"

namespace dpl {

constexpr int kTcM = 128;                    // rows per M tile
constexpr int kTcRows = 128;                 // rows of each M tile used per pass
constexpr int kTcN = 256;                    // pixels per tile (MMA N)
constexpr int kTcTileR = 16, kTcTileC = 16;  // tile of output pixels
constexpr int kTcKC = 32;                    // samples per K chunk
constexpr int kTcThreads = 576;              // 18 warps
constexpr int kTcBuilders = 544;             // warps 0-16; warp 17 issues the MMAs
static_assert(4 * kTcRows <= kTcBuilders, "one Khatri-Rao item per builder");
constexpr int kTcCols = 512;                 // TMEM columns: two M tiles x 256 pixels
constexpr int kTcStageBytes = 4 * 8192 + 16384;  // KR hi/lo of two M tiles + mask (bf16)
// TF32 form: one tf32 plane per M tile (16 KB) and a tf32 mask (32 KB)
constexpr int kTcStageBytesTf = 2 * 16384 + 32768;
template <bool kTf>
constexpr int tc_stage_bytes() {
    return kTf ? kTcStageBytesTf : kTcStageBytes;
}
constexpr int kTcMaxStages = 3;

struct TcArgs {
    int n, rows, cols, hy, hx, sy, sx, out_rows, out_cols;
    int tiles_r, tiles_c;
    int region_r, region_c;  // max region extent of a tile
    int kpad, kwords;        // region samples padded to a multiple of kTcKC; 32-bit words per pixel
    int npass;               // 1 + ceil((N(N-1)/2 - (kTcRows - N)) / kTcRows)
    int nst;                 // operand stages (2 or 3)
    const cfloat* zt;        // (rows, cols, n) masked, pixel-major
    const uint32_t* bits;    // (out_rows, out_cols, wy, wpr) or null (rectangular window)
    const uint8_t* nb_u8;    // alternative mask input (out_rows, out_cols, wy, wx)
    int wpr;
    float* Cg;               // (out_rows * out_cols, n * n) planar output
    int32_t* counts;         // (out_rows * out_cols) or null
    int* status;
    // shared-memory carve (bytes from the 1024-aligned base)
    int off_stage, off_z, z_bytes, off_pbits, off_soff, off_runs, off_rows, off_bar, smem_bytes;
};

// A batch of stacks for one work-queue launch (passed as a kernel parameter, 2.6 KB).
constexpr int kTcMaxItems = 16;
struct TcBatch {
    TcArgs items[kTcMaxItems];
    int tile_start[kTcMaxItems];
    int nitems, total;
};

constexpr int kTcRuns = 3;  // contiguous runs of image samples per K chunk (a chunk spans <= 3 region rows)
constexpr int kTcZBuf = 4;  // ring of chunk sample buffers (bulk prefetch distance)

// byte offset of element (row, k) in a K-major no-swizzle tile with KC columns
__device__ __forceinline__ int tc_off(int row, int k) {
    return (row >> 3) * (kTcKC / 8 * 128) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// byte offset of element (row, k) in a K-major no-swizzle tf32 tile with KC columns
// (core matrices of 8 rows x 4 elements)
__device__ __forceinline__ int tc_off32(int row, int k) {
    return (row >> 3) * (kTcKC / 4 * 128) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

// 8 values rounded to tf32 (nearest, ties away: cvt.rna.tf32.f32) into row `row`,
// samples kb..kb+7, of a tf32 KR M tile
__device__ __forceinline__ void tc_store8_tf32(unsigned char* plane, int row, int kb, const float (&x)[8]) {
    uint32_t t[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t[q]) : "f"(x[q]));
    *reinterpret_cast<uint4*>(plane + tc_off32(row, kb)) = make_uint4(t[0], t[1], t[2], t[3]);
    *reinterpret_cast<uint4*>(plane + tc_off32(row, kb + 4)) = make_uint4(t[4], t[5], t[6], t[7]);
}

// 4 mask bits -> 4 tf32 (1.0 or 0)
__device__ __forceinline__ uint4 tc_expand4_tf32(uint32_t b) {
    return make_uint4((b & 1u) * 0x3F800000u, ((b >> 1) & 1u) * 0x3F800000u, ((b >> 2) & 1u) * 0x3F800000u,
                      ((b >> 3) & 1u) * 0x3F800000u);
}

// bf16 hi/lo split of two values, packed (first value in the low half)
__device__ __forceinline__ void tc_split2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// hi/lo planes of 8 values into row `row`, samples kb..kb+7, of a KR M tile
__device__ __forceinline__ void tc_store8(unsigned char* hi_plane, unsigned char* lo_plane, int row, int kb,
                                          const float (&x)[8]) {
    uint4 hw, lw;
    tc_split2(x[0], x[1], hw.x, lw.x);
    tc_split2(x[2], x[3], hw.y, lw.y);
    tc_split2(x[4], x[5], hw.z, lw.z);
    tc_split2(x[6], x[7], hw.w, lw.w);
    *reinterpret_cast<uint4*>(hi_plane + tc_off(row, kb)) = hw;
    *reinterpret_cast<uint4*>(lo_plane + tc_off(row, kb)) = lw;
}

// 8 mask bits -> 8 bf16 (1.0 or 0), packed in pairs (bit 0 -> first element): with
// x = b | b << 15, bits 2k and 2k+1 of b sit at bits 0 and 16 of x >> 2k, and times
// 0x3F80 (bf16 1.0) each becomes its 16-bit half
__device__ __forceinline__ uint4 tc_expand8(uint32_t b) {
    const uint32_t x = (b & 0xffu) | ((b & 0xffu) << 15);
    uint4 r;
    r.x = (x & 0x10001u) * 0x3F80u;
    r.y = ((x >> 2) & 0x10001u) * 0x3F80u;
    r.z = ((x >> 4) & 0x10001u) * 0x3F80u;
    r.w = ((x >> 6) & 0x10001u) * 0x3F80u;
    return r;
}


// Prefetch the samples of chunk `ch` into zs[k][t] (builder threads; soff = element
// offset of each region sample in zt, or -1 outside the image: zero-filled).
__device__ __forceinline__ void tc_prefetch(const TcArgs& a, cfloat* zs, const int* soff, int ch, int btid) {
    const int n = a.n;
    for (int idx = btid; idx < kTcKC * 16; idx += kTcBuilders) {
        const int k = idx >> 4;
        const int off = soff[ch * kTcKC + k];
        for (int t = idx & 15; t < n; t += 16) {
            const cfloat* src = off >= 0 ? a.zt + off + t : a.zt;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(tc_smem(zs + k * n + t)), "l"(src),
                         "r"(off >= 0 ? 8 : 0)
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Even N: the chunk's image samples are <= 3 contiguous runs of zt (one per region
// row), copied by one thread with 1-D bulk copies that complete on zbar.  Samples
// outside the image are not copied: no pixel's window contains them, so whatever
// finite values their slots hold are multiplied by zero mask entries.
// runs[ch][r] = (k_start | len << 8, element offset), len = 0 for an unused slot.
__device__ __forceinline__ void tc_prefetch_bulk(const TcArgs& a, cfloat* zs, uint64_t* zbar, const int2* runs,
                                                 int ch) {
    const int n = a.n;
    const int2* rc = runs + ch * kTcRuns;
    uint32_t total = 0;
#pragma unroll
    for (int r = 0; r < kTcRuns; ++r) total += (uint32_t)((rc[r].x >> 8) * n * 8);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     tc_smem(zbar)),
                 "r"(total)
                 : "memory");
#pragma unroll
    for (int r = 0; r < kTcRuns; ++r) {
        const int len = rc[r].x >> 8;
        if (len > 0)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    tc_smem(zs + (rc[r].x & 0xff) * n)),
                "l"(a.zt + rc[r].y), "r"(len * n * 8), "r"(tc_smem(zbar))
                : "memory");
    }
}

// One launch serves one stack (kQueue false: the tiles of b.items[0], strided over the
// grid) or a batch of stacks (kQueue true): b.items[i] describes stack i, b.tile_start[i]
// its first tile in the batch's tile numbering (b.total tiles in all), and every CTA
// takes the next batch tile from `counter` (a work queue; the items are ordered largest
// first).  All items share one shared-memory carve (offsets, stage count, z_bytes).
template <bool kTf, bool kQueue>
__global__ void __launch_bounds__(kTcThreads, 1) k_cov_tc(const __grid_constant__ TcBatch b, int* counter) {
    constexpr int kStage = tc_stage_bytes<kTf>();
    extern __shared__ unsigned char tc_raw[];
    // 1024-byte aligned base, derived from the shared array itself so that every access
    // below stays a shared-memory access
    unsigned char* sm = tc_raw + ((1024u - (tc_smem(tc_raw) & 1023u)) & 1023u);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    TcArgs a = b.items[0];
    int cur = 0;  // the item `a` describes
    int n = a.n, nn = n * n, wy = 2 * a.hy + 1, wx = 2 * a.hx + 1;
    int O = n * (n - 1) / 2;
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + a.off_bar);  // [kTcMaxStages] builders -> issuer
    uint64_t* empty = full + kTcMaxStages;                           // [kTcMaxStages] MMAs done -> builders
    uint64_t* zbar = empty + kTcMaxStages;                           // [kTcZBuf] bulk sample copies landed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(zbar + kTcZBuf);
    int* sfail = reinterpret_cast<int*>(tmem_slot + 2);
    int* snext = sfail + 1;                                          // the next batch tile (kQueue)
    int2* runs = reinterpret_cast<int2*>(sm + a.off_runs);          // [nchunks][kTcRuns]
    bool bulk = (a.n & 1) == 0;
    auto zbuf = [&](int c) { return reinterpret_cast<cfloat*>(sm + a.off_z + (c & (kTcZBuf - 1)) * a.z_bytes); };
    uint32_t* pbits = reinterpret_cast<uint32_t*>(sm + a.off_pbits);  // [256][kwords]: pixel mask bits
    int* soff = reinterpret_cast<int*>(sm + a.off_soff);              // [kpad]: sample offsets in zt
    // row table [npass][kTcRows]: i | j << 16 of the row's (i, j), i == j for the diagonal
    uint32_t* rowtab = reinterpret_cast<uint32_t*>(sm + a.off_rows);

    for (int e = tid; e < kTcZBuf * a.z_bytes / 4; e += kTcThreads)  // no NaN patterns in unused slots
        reinterpret_cast<float*>(sm + a.off_z)[e] = 0.f;
    // the row table of the current item's N (rebuilt when a batch moves to another stack)
    auto fill_rowtab = [&]() {
        for (int idx = tid; idx < a.npass * kTcRows; idx += kTcThreads) {
            const int pass = idx / kTcRows, u = idx - pass * kTcRows;
            const int d0 = pass == 0 ? n : 0;
            const int o = (pass == 0 ? 0 : (kTcRows - n) + (pass - 1) * kTcRows) + u - d0;
            uint32_t ij = 0u;  // unused rows: (0, 0)
            if (u < d0) {
                ij = (uint32_t)u | ((uint32_t)u << 16);
            } else if (o < O) {
                int i = (int)((sqrtf(8.f * o + 1.f) + 1.f) * 0.5f);  // o = i(i-1)/2 + j, 0 <= j < i
                while (i * (i - 1) / 2 > o) --i;
                while ((i + 1) * i / 2 <= o) ++i;
                ij = (uint32_t)i | ((uint32_t)(o - i * (i - 1) / 2) << 16);
            }
            rowtab[idx] = ij;
        }
    };
    fill_rowtab();
    if (tid == 0) {
        for (int s = 0; s < a.nst; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&full[s])), "r"(kTcBuilders / 32));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&empty[s])), "r"(1));
        }
        for (int c = 0; c < kTcZBuf; ++c)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&zbar[c])), "r"(1));
        *sfail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                     "r"(kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const bool builder = warp < kTcBuilders / 32;
    // per-stage state as bit s: mbarrier phase parities, and (builders) an MMA commit on
    // empty[s] still to be consumed
    uint32_t ph_full = 0u, ph_empty = 0u, pend = 0u, ph_z = 0u;
    // issuer: per sample buffer, bit c of z_arm = parity of the next phase it arms, bit c
    // of z_used = armed at least once (to drain the copies in flight on a timeout)
    uint32_t z_arm = 0u, z_used = 0u;
    auto arm_bulk = [&](int c, int ch) {
        const int zi = c & (kTcZBuf - 1);
        tc_prefetch_bulk(a, zbuf(c), &zbar[zi], runs, ch);
        z_arm ^= 1u << zi;
        z_used |= 1u << zi;
    };
    int nchunks = a.kpad / kTcKC;

    const int ntiles = a.tiles_r * a.tiles_c;
    for (int it = 0;; ++it) {
        int tile;
        if (kQueue) {
            __syncthreads();  // the previous tile is done with every shared buffer and with snext
            if (tid == 0) *snext = atomicAdd(counter, 1);
            __syncthreads();
            const int t = *snext;
            if (t >= b.total) break;
            int i = cur;  // a CTA's tiles only increase, so its item only moves forward
            while (i + 1 < b.nitems && b.tile_start[i + 1] <= t) ++i;
            if (i != cur) {
                cur = i;
                a = b.items[i];
                n = a.n;
                nn = n * n;
                wy = 2 * a.hy + 1;
                wx = 2 * a.hx + 1;
                O = n * (n - 1) / 2;
                bulk = (n & 1) == 0;
                nchunks = a.kpad / kTcKC;
                fill_rowtab();
                __syncthreads();
            }
            tile = t - b.tile_start[i];
        } else {
            tile = blockIdx.x + it * gridDim.x;
            if (tile >= ntiles) break;
        }
        const int tr0 = (tile / a.tiles_c) * kTcTileR, tc0 = (tile % a.tiles_c) * kTcTileC;
        // region origin: clamped window start of the tile's first output pixel
        const int rr0 = min(max(a.sy / 2 + tr0 * a.sy - a.hy, 0), a.rows - wy);
        const int cc0 = min(max(a.sx / 2 + tc0 * a.sx - a.hx, 0), a.cols - wx);
        // sample offsets of the region
        for (int s = tid; s < a.kpad; s += kTcThreads) {
            const int ry = s / a.region_c, cx = s - ry * a.region_c;
            const int r = rr0 + ry, c = cc0 + cx;
            soff[s] = (ry < a.region_r && r < a.rows && c < a.cols) ? (r * a.cols + c) * n : -1;
        }
        __syncthreads();
        if (bulk) {
            for (int ch = tid; ch < nchunks; ch += kTcThreads) {
                int2* rc = runs + ch * kTcRuns;
                int nr = 0;
                for (int k = 0; k < kTcKC;) {
                    const int off = soff[ch * kTcKC + k];
                    if (off < 0) {
                        ++k;
                        continue;
                    }
                    int len = 1;
                    while (k + len < kTcKC && soff[ch * kTcKC + k + len] == off + len * n) ++len;
                    if (nr < kTcRuns) rc[nr++] = make_int2(k | (len << 8), off);
                    k += len;
                }
                for (; nr < kTcRuns; ++nr) rc[nr] = make_int2(0, 0);
            }
        }
        // per-pixel mask bits over the region's samples
        if (tid < kTcN) {
            uint32_t* pb = pbits + tid * a.kwords;
            for (int w = 0; w < a.kwords; ++w) pb[w] = 0u;
            const int pr = tr0 + tid / kTcTileC, pc = tc0 + tid % kTcTileC;
            if (pr < a.out_rows && pc < a.out_cols) {
                const int r0 = min(max(a.sy / 2 + pr * a.sy - a.hy, 0), a.rows - wy);
                const int c0 = min(max(a.sx / 2 + pc * a.sx - a.hx, 0), a.cols - wx);
                const int wr = r0 - rr0, wc = c0 - cc0;
                const int64_t p = (int64_t)pr * a.out_cols + pc;
                const uint64_t fullrow = wx >= 64 ? ~0ull : ((1ull << wx) - 1ull);
                int cnt = 0;
                for (int dr = 0; dr < wy; ++dr) {
                    uint64_t m = fullrow;
                    if (a.bits) {
                        const uint32_t* w = a.bits + (p * wy + dr) * a.wpr;
                        m = (w[0] | (a.wpr > 1 ? (uint64_t)w[1] << 32 : 0ull)) & fullrow;
                    } else if (a.nb_u8) {
                        const uint8_t* b = a.nb_u8 + (p * wy + dr) * wx;
                        m = 0;
                        for (int q = 0; q < wx; ++q) m |= (uint64_t)(b[q] != 0) << q;
                    }
                    cnt += __popcll(m);
                    const int s0 = (wr + dr) * a.region_c + wc;  // first sample of the window row
                    const int w0 = s0 >> 5, sh = s0 & 31;
                    const uint64_t lo = m << sh;
                    pb[w0] |= (uint32_t)lo;
                    if ((uint32_t)(lo >> 32)) pb[w0 + 1] |= (uint32_t)(lo >> 32);
                    const uint32_t hi = sh ? (uint32_t)(m >> (64 - sh)) : 0u;
                    if (hi) pb[w0 + 2] |= hi;
                }
                if (a.counts) a.counts[p] = cnt;
            }
        }
        __syncthreads();
        for (int pass = 0; pass < a.npass; ++pass) {
            // rows of the pass: d0 diagonal rows (pass 0), then np lower pairs from qb on
            const int d0 = pass == 0 ? n : 0;
            const int qb = pass == 0 ? 0 : (kTcRows - n) + (pass - 1) * kTcRows;
            const int np = max(min(O - qb, kTcRows - d0), 0);
            const int rows0 = d0 + np;
            const int mt = np > 0 ? 2 : 1;  // M tiles holding rows (tile 1: imaginary parts)
            const uint32_t* rows_p = rowtab + pass * kTcRows;
            if (builder) {
                const int btid = tid;
                if (!bulk) tc_prefetch(a, zbuf(0), soff, 0, btid);
                for (int ch = 0, s = 0; ch < nchunks; ++ch, s = s + 1 == a.nst ? 0 : s + 1) {
                    const int zi = ch & (kTcZBuf - 1);
                    unsigned char* stage = sm + a.off_stage + s * kStage;
                    unsigned char* msk = stage + 32768;  // after the two M tiles in both forms
                    // Before building, the MMAs that last read this stage must be done and
                    // the chunk's samples must have landed.  Even N (bulk copies): each
                    // warp's lane 0 waits on the mbarriers and the warp reconverges, so the
                    // warps run up to one chunk apart (a warp cannot wait on a phase more
                    // than one ahead: the next one needs its own arrival on `full`).  Odd N
                    // (cp.async by every builder): thread 0 waits, then the named barrier;
                    // bar.sync counts a warp as arrived when any of its lanes arrives, so
                    // warp 0 reconverges first.
                    const bool waiter = bulk ? lane == 0 : btid == 0;
                    if ((pend >> s) & 1u) {
                        if (waiter && !tc_wait(&empty[s], (ph_empty >> s) & 1u)) atomicExch(sfail, 1);
                        ph_empty ^= 1u << s;
                        pend &= ~(1u << s);
                    }
                    if (bulk) {
                        if (waiter && !tc_wait(&zbar[zi], (ph_z >> zi) & 1u)) atomicExch(sfail, 1);
                        ph_z ^= 1u << zi;
                        __syncwarp();
                    } else {
                        asm volatile("cp.async.wait_group 0;" ::: "memory");
                        __syncwarp();
                        asm volatile("bar.sync 1, %0;" ::"n"(kTcBuilders) : "memory");
                    }
                    if (*(volatile int*)sfail) break;
                    if (!bulk && ch + 1 < nchunks) tc_prefetch(a, zbuf(ch + 1), soff, ch + 1, btid);
                    const cfloat* zs = zbuf(ch);
                    // Khatri-Rao items (row x 8 samples, at most one per builder; consecutive
                    // lanes take consecutive rows), then mask items (pixel row x 16
                    // samples), the latter starting on the builders without a row item
                    const int nkr = 4 * rows0;
                    if (btid < nkr) {
                        const int g = (btid >= rows0) + (btid >= 2 * rows0) + (btid >= 3 * rows0);
                        const int u = btid - g * rows0, kb = 8 * g;
                        const uint32_t ij = rows_p[u];
                        const cfloat* zk = zs + kb * n;  // sample kb; + n per sample
                        const cfloat* pi = zk + (ij & 0xffff);
                        const cfloat* pj = zk + (ij >> 16);
                        // Re and Im of z_i conj(z_j); for a diagonal row (i == j) Re = |z_i|^2
                        // and the Im row (M tile 1) is not read back
                        float xr[8], xi[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const cfloat zi = pi[q * n], zj = pj[q * n];
                            xr[q] = fmaf(zi.re, zj.re, zi.im * zj.im);
                            xi[q] = fmaf(zi.im, zj.re, -(zi.re * zj.im));
                        }
                        if (kTf) {
                            tc_store8_tf32(stage, u, kb, xr);
                            tc_store8_tf32(stage + 16384, u, kb, xi);
                        } else {
                            tc_store8(stage, stage + 8192, u, kb, xr);
                            tc_store8(stage + 16384, stage + 24576, u, kb, xi);
                        }
                    }
                    int m = btid - nkr;
                    if (m < 0) m += kTcBuilders;
                    for (; m < 2 * kTcN; m += kTcBuilders) {
                        const int row = m >> 1, half = m & 1;
                        const uint32_t bw = pbits[row * a.kwords + ch] >> (16 * half);
                        if (kTf) {
#pragma unroll
                            for (int g4 = 0; g4 < 4; ++g4)
                                *reinterpret_cast<uint4*>(msk + tc_off32(row, 16 * half + 4 * g4)) =
                                    tc_expand4_tf32(bw >> (4 * g4));
                        } else {
                            *reinterpret_cast<uint4*>(msk + tc_off(row, 16 * half)) = tc_expand8(bw);
                            *reinterpret_cast<uint4*>(msk + tc_off(row, 16 * half + 8)) = tc_expand8(bw >> 8);
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0)
                        asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(
                                         tc_smem(&full[s]))
                                     : "memory");
                    pend |= 1u << s;
                }
                // drain: the last MMAs of the pass must be complete before the epilogue
                for (int s2 = 0; s2 < a.nst; ++s2) {
                    if ((pend >> s2) & 1u) {
                        if (btid == 0 && !tc_wait(&empty[s2], (ph_empty >> s2) & 1u)) atomicExch(sfail, 1);
                        ph_empty ^= 1u << s2;
                        pend &= ~(1u << s2);
                    }
                }
            } else if (lane == 0) {
                // MMA issuer
                // core matrices are 16 bytes wide: 8 bf16 or 4 tf32 samples
                constexpr int kCoreK = kTf ? 4 : 8;
                constexpr uint32_t LBO = 128, SBO = kTcKC / kCoreK * 128;
                const uint32_t idesc = kTf ? tc_idesc_tf32(kTcM, kTcN) : tc_idesc_bf16(kTcM, kTcN);
                // Descriptors of stage 0 (M tile 0, hi plane, k = 0) and of its mask.  Every
                // other operand of a chunk lies a fixed offset away, and bits 0-13 of a
                // descriptor hold the shared address >> 4: with every address below 256 KB,
                // adding offset >> 4 never carries into the other fields.
                const uint64_t dA = tc_desc(tc_smem(sm + a.off_stage), LBO, SBO);
                const uint64_t dB = dA + (uint64_t)(32768 >> 4);
                if (bulk)
                    for (int c = 0; c < kTcZBuf && c < nchunks; ++c) arm_bulk(c, c);
                for (int ch = 0, s = 0; ch < nchunks; ++ch, s = s + 1 == a.nst ? 0 : s + 1) {
                    if (!tc_wait(&full[s], (ph_full >> s) & 1u)) {
                        atomicExch(sfail, 1);
                        break;
                    }
                    ph_full ^= 1u << s;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint64_t so = (uint64_t)((s * kStage) >> 4);
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        if (t >= mt) break;
                        const uint32_t dt = tmem + (uint32_t)(t * kTcN);
                        // one MMA covers 32 bytes of K: 16 bf16 or 8 tf32 samples
#pragma unroll
                        for (int kk = 0; kk < kTcKC; kk += 2 * kCoreK) {
                            const uint64_t ko = (uint64_t)(((kk / kCoreK) * LBO) >> 4);
                            const uint64_t bd = dB + so + ko;
                            const uint64_t ah = dA + so + (uint64_t)((t * 16384) >> 4) + ko;
                            const uint64_t al = ah + (uint64_t)(8192 >> 4);
                            const uint32_t acc0 = (ch > 0 || kk > 0) ? 1u : 0u;
                            if (kTf) {  // tf32: one product
                                asm volatile(
                                    "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                                    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
                                    "l"(ah), "l"(bd), "r"(idesc), "r"(acc0));
                                continue;
                            }
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
                                "l"(ah), "l"(bd), "r"(idesc), "r"(acc0));
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
                                "l"(al), "l"(bd), "r"(idesc), "r"(1u));
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     tc_smem(&empty[s]))
                                 : "memory");
                    // the builders are done with this chunk's samples: refill its buffer
                    if (bulk && ch + kTcZBuf < nchunks) arm_bulk(ch, ch + kTcZBuf);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (*(volatile int*)sfail) break;
            // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows) for its share of
            // the 16-pixel groups of both M tiles
            const int quarter = warp & 3;
            const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
            const int u = quarter * 32 + lane;  // this lane's row
            // (Re, Im) pairs go out as float2 where the planar rows keep 8-byte alignment
            const bool v2 = (nn & 1) == 0 && (reinterpret_cast<uintptr_t>(a.Cg) & 7u) == 0;
            if (quarter * 32 < rows0) {
                // this lane's row: its place in the planar output
                const bool diag = u < d0;
                const int e = diag ? u : n + 2 * (qb + u - d0);
                // 16-pixel group g is row g of the 16 x 16 tile
                const int qn = min(kTcTileC, a.out_cols - tc0);
                // warps of this lane quarter: warp w takes groups w / 4, + nq, + 2 nq, ...
                const int nq = (kTcThreads / 32 - quarter + 3) / 4;
                for (int g = warp >> 2; g < kTcN / 16; g += nq) {
                    uint32_t re[16], im[16];
                    tc_ld16(tmem + lane_base + (uint32_t)(16 * g), re);
                    if (mt == 2) tc_ld16(tmem + lane_base + (uint32_t)(kTcN + 16 * g), im);
                    const int pr = tr0 + g;
                    if (u < rows0 && pr < a.out_rows) {
                        float* dst = a.Cg + ((int64_t)pr * a.out_cols + tc0) * nn + e;
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            if (q < qn) {
                                if (diag) {
                                    dst[(int64_t)q * nn] = __uint_as_float(re[q]);
                                } else if (v2) {
                                    *reinterpret_cast<float2*>(dst + (int64_t)q * nn) =
                                        make_float2(__uint_as_float(re[q]), __uint_as_float(im[q]));
                                } else {
                                    dst[(int64_t)q * nn] = __uint_as_float(re[q]);
                                    dst[(int64_t)q * nn + 1] = __uint_as_float(im[q]);
                                }
                            }
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        if (*(volatile int*)sfail) break;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (tid == 0 && *(volatile int*)sfail) atomicExch(a.status, (int)DPL_ERR_TIMEOUT);
    // before releasing TMEM make sure no MMA is still in flight (bounded)
    if (tid == 0)
        for (int s2 = 0; s2 < a.nst; ++s2)
            if ((pend >> s2) & 1u) tc_wait(&empty[s2], (ph_empty >> s2) & 1u);
    // and, after a timeout, that no bulk sample copy still writes into shared memory:
    // the issuer waits (bounded) on the last phase it armed on each buffer, which has
    // already completed where a builder consumed it
    if (tid == kTcBuilders && *(volatile int*)sfail)
        for (int c = 0; c < kTcZBuf; ++c)
            if ((z_used >> c) & 1u) tc_wait(&zbar[c], ((z_arm >> c) & 1u) ^ 1u);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols));
}

}  // namespace dpl
