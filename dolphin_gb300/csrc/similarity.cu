// Phase-similarity raster: median_similarity / max_similarity (similarity.py:31-173),
// the search circle (similarity.py:176-254) and the nearest-n phase differences
// (similarity.py:355-375) on the GPU.
//
// k_sim_prep  -- one thread per pixel, one pass over the stack: the invalid test (the
//                sum over the stack of nan_to_num(z) is exactly 0, summed layer by layer
//                in float32 as numpy reduces the first axis) and the comparison phasors
//                exp(i angle z) or exp(i phase), planar (m, rows, cols).  A pixel that is
//                invalid or masked gets NaN phasors: every similarity it takes part in is
//                then NaN, which the summaries skip, exactly as the reference skips masked
//                pixels (the count of usable neighbours only matters through "none").
// k_similarity<H> -- persistent; a CTA of 512 threads owns a tile of pixels.  Eight
//                layers at a time of the tile's neighbourhood (tile + H on every side,
//                edge pixels replicated: the reference clips each neighbour coordinate
//                to the image) are staged in shared memory with cp.async, double-
//                buffered across chunks and tiles.  A group of G >= 2H + 1 lanes owns P
//                vertically adjacent pixels of one column; lane dc + H loads the
//                2H + P staged values of column c + dc and accumulates, in registers and
//                over all layers, the similarities of its P pixels with their 2H + 1
//                neighbours in that column (each load serves P pixels).  The circle's
//                K similarities of a pixel thus sit in the registers of its group, and
//                the summary is taken there: the maximum by a group reduction, the
//                median by a selection on order-preserving keys, each step one
//                group-wide count (redux.sync) around an interpolated pivot.  The
//                pixel itself (which
//                a clipped offset reaches at the image edge) and NaN similarities are
//                left out.
#include <algorithm>
#include <cstdio>
#include <utility>
#include <vector>

#include "dpl_common.cuh"

namespace dpl {

constexpr int kSimHMax = 15;  // largest offset: search radius 16

// ----------------------------------------------------------------------------------
// search circle (host)
// ----------------------------------------------------------------------------------

// Concentric midpoint circles of radius 1 .. max_radius - 1; each one, walked over its
// first octant, is extended inward along its rows until it meets the area covered by
// the previous rings, then mirrored into all eight octants.  The offsets come out ring
// by ring in the reference's order (its set and its unsorted order depend on these
// steps), sorted lexicographically on request.
std::vector<std::pair<int, int>> circle_offsets(int max_radius, int min_radius, bool sorted_out) {
    std::vector<std::pair<int, int>> found;
    if (max_radius < 1) return found;
    std::vector<uint8_t> cover((size_t)max_radius * max_radius, 0);
    auto at = [&](int a, int b) -> uint8_t& { return cover[(size_t)a * max_radius + b]; };
    at(0, 0) = 1;
    for (int ring = 1; ring < max_radius; ++ring) {
        const bool emit = ring > min_radius;
        if (emit) {
            found.push_back({ring, 0});
            found.push_back({-ring, 0});
            found.push_back({0, ring});
            found.push_back({0, -ring});
        }
        at(ring, 0) = at(0, ring) = 1;
        int a = ring, b = 0, decision = 1 - ring, backlog = 0;
        while (a > b) {
            if (backlog > 0) {
                --backlog;
            } else {
                ++b;
                if (decision <= 0) {
                    decision += 2 * b + 1;
                } else {
                    --a;
                    decision += 2 * b - 2 * a + 1;
                }
            }
            if (a < b) break;
            while (!at(a - 1, b)) {
                --a;
                ++backlog;
            }
            at(a, b) = at(b, a) = 1;
            if (emit) {
                const int pts[4][2] = {{a, b}, {-a, -b}, {a, -b}, {-a, b}};
                for (auto& q : pts) found.push_back({q[0], q[1]});
                if (a != b) {
                    const int sw[4][2] = {{b, a}, {-b, -a}, {b, -a}, {-b, a}};
                    for (auto& q : sw) found.push_back({q[0], q[1]});
                }
            }
            if (backlog > 0) ++a;
        }
    }
    if (sorted_out) std::sort(found.begin(), found.end());
    return found;
}

// Column table of a full circle (min_radius 0): for dc = -H..H the half-height of the
// column (its row offsets are exactly -hc..hc, the centre excluded) and its first slot.
// Returns false if some column is not such a run (it is for every radius checked).
static bool circle_columns(int radius, int H, int* hc, int* base, int* K) {
    auto offs = circle_offsets(radius, 0, true);
    std::vector<int> lo(2 * H + 1, 1 << 20), hi(2 * H + 1, -(1 << 20)), cnt(2 * H + 1, 0);
    for (auto& o : offs) {
        const int dr = o.first, dc = o.second;
        if (dc < -H || dc > H || dr < -H || dr > H) return false;
        const int i = dc + H;
        lo[i] = std::min(lo[i], dr);
        hi[i] = std::max(hi[i], dr);
        ++cnt[i];
    }
    int slot = 0;
    for (int i = 0; i <= 2 * H; ++i) {
        if (cnt[i] == 0) {
            hc[i] = -1;
        } else {
            if (lo[i] != -hi[i]) return false;
            const int expect = 2 * hi[i] + 1 - (i == H ? 1 : 0);
            if (cnt[i] != expect) return false;
            hc[i] = hi[i];
        }
        base[i] = slot;
        slot += cnt[i];
    }
    *K = slot;
    return slot == (int)offs.size();
}

// ----------------------------------------------------------------------------------
// prep: validity and comparison phasors
// ----------------------------------------------------------------------------------
struct SimPrepArgs {
    int nin;         // layers of the input stack
    int m;           // comparison layers written
    int nearest;     // 0, or n of the nearest-n pairs
    int is_complex;  // complex64 input (else float32 phase)
    int64_t npix;
    const float* stack;   // (nin, npix) complex64 or float32
    const uint8_t* mask;  // (npix) or null
    uint8_t* valid;       // (npix) out
    float2* unit;         // (m, npix) out
};

__device__ __forceinline__ float nan_to_num_f(float x) {
    if (isnan(x)) return 0.f;
    if (isinf(x)) return x > 0.f ? 3.402823466e38f : -3.402823466e38f;
    return x;
}

__device__ __forceinline__ float sim_phase(const SimPrepArgs& a, int t, int64_t p) {
    if (a.is_complex) {
        const float2 z = reinterpret_cast<const float2*>(a.stack)[(int64_t)t * a.npix + p];
        return atan2f(z.y, z.x);
    }
    return a.stack[(int64_t)t * a.npix + p];
}

__global__ void __launch_bounds__(256) k_sim_prep(SimPrepArgs a) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.npix) return;
    const float qnan = __int_as_float(0x7fffffff);
    const bool masked = a.mask && a.mask[p] == 0;
    float sre = 0.f, sim = 0.f;
    if (!a.nearest) {
        // one pass: sums and phasors; a pixel found invalid is overwritten with NaN
        for (int t = 0; t < a.nin; ++t) {
            float ph;
            if (a.is_complex) {
                const float2 z = reinterpret_cast<const float2*>(a.stack)[(int64_t)t * a.npix + p];
                sre = fadd(sre, nan_to_num_f(z.x));
                sim = fadd(sim, nan_to_num_f(z.y));
                ph = atan2f(z.y, z.x);
            } else {
                ph = a.stack[(int64_t)t * a.npix + p];
                sre = fadd(sre, nan_to_num_f(ph));
            }
            float2 u = make_float2(qnan, qnan);
            if (!masked) sincosf(ph, &u.y, &u.x);
            a.unit[(int64_t)t * a.npix + p] = u;
        }
        const bool ok = !(sre == 0.f && sim == 0.f) && !masked;
        a.valid[p] = ok ? 1 : 0;
        if (!ok && !masked)
            for (int t = 0; t < a.m; ++t) a.unit[(int64_t)t * a.npix + p] = make_float2(qnan, qnan);
        return;
    }
    bool finite = true;
    for (int t = 0; t < a.nin; ++t) {
        if (a.is_complex) {
            const float2 z = reinterpret_cast<const float2*>(a.stack)[(int64_t)t * a.npix + p];
            sre = fadd(sre, nan_to_num_f(z.x));
            sim = fadd(sim, nan_to_num_f(z.y));
            finite = finite && !isnan(z.x) && !isnan(z.y);
        } else {
            const float x = a.stack[(int64_t)t * a.npix + p];
            sre = fadd(sre, nan_to_num_f(x));
            finite = finite && isfinite(x);
        }
    }
    // nearest-n: the pair phases come from a matrix product in which every layer takes
    // part, so one non-finite phase spoils all of them and the pixel becomes invalid
    const bool ok = !(sre == 0.f && sim == 0.f) && finite && !masked;
    a.valid[p] = ok ? 1 : 0;
    // pairs (i, j), i < j <= i + n, over the nin + 1 dates; date 0 is the reference
    int k = 0;
    for (int i = 0; i <= a.nin; ++i) {
        const float pi_ = (i == 0 || !ok) ? 0.f : sim_phase(a, i - 1, p);
        const int jmax = min(i + a.nearest, a.nin);
        for (int j = i + 1; j <= jmax; ++j, ++k) {
            float2 u = make_float2(qnan, qnan);
            if (ok) sincosf(sim_phase(a, j - 1, p) - pi_, &u.y, &u.x);
            a.unit[(int64_t)k * a.npix + p] = u;
        }
    }
}

// ----------------------------------------------------------------------------------
// similarity
// ----------------------------------------------------------------------------------
constexpr int kSimChunk = 8;  // layers per staged chunk

struct SimArgs {
    int m, rows, cols;
    int tiles_c, tiles;  // tile grid (row-major)
    int kind;            // 0 median, 1 max
    const float2* unit;  // (m, rows, cols)
    float* out;          // (rows, cols)
    int hc[2 * kSimHMax + 1];  // half-height of column dc (at index dc + H)
};

// Work layout for largest offset H.  A group of G lanes (G >= 2H + 1) owns P vertically
// adjacent pixels of one column; its lane dc + H accumulates their similarities with
// the 2H + 1 neighbours in column c + dc.  A CTA owns TC x TR pixels.
template <int H>
struct SimShape {
    static constexpr int D = 2 * H + 1;
    static constexpr int G = D <= 4 ? 4 : D <= 8 ? 8 : D <= 16 ? 16 : 32;
    static constexpr int P = H <= 10 ? 4 : 2;
    static constexpr int GPW = 32 / G;
    // 256 threads (two CTAs per SM, which drift apart so that one accumulates while the
    // other takes its summaries) except for the widest groups, whose tiles would be thin
    static constexpr int THREADS = G == 32 ? 512 : 256;
    static constexpr int UNITS = THREADS / 32 * GPW;
    static constexpr int TC = G == 4 ? 32 : 16;
    static constexpr int TR = UNITS / TC * P;
    static constexpr int TRH = TR + 2 * H, SW = TC + 2 * H;  // staged rows and columns
    static constexpr int LAYER = TRH * SW;                   // float2 per staged layer
    static constexpr int STAGE = kSimChunk * LAYER;
    static constexpr size_t SMEM = 2 * (size_t)STAGE * sizeof(float2);
    static_assert(UNITS % TC == 0, "tile rows");
};

__device__ __forceinline__ void sim_cp8(float2* dst, const float2* src, bool fill) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    const int n = fill ? 8 : 0;  // 0 source bytes: the 8 destination bytes are zeroed
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(src), "r"(n) : "memory");
}

// Order-preserving unsigned key of a float that is not NaN, and its inverse.
__device__ __forceinline__ uint32_t sim_key(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float sim_unkey(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Reductions over the G-lane groups of a warp, executed by all 32 lanes together so
// that no collective runs under divergence: sums through one warp-wide redux of
// per-group bit fields (a group's sum never exceeds its field), minima and maxima
// through xor butterflies that stay inside each group.
template <int G>
struct SimGroup {
    static constexpr int FW = G;  // bits of a group's field: 32 / (32 / G)
    int shift;
    __device__ __forceinline__ explicit SimGroup(int lane) : shift((lane / G) * G) {}
    __device__ __forceinline__ int sum(int v) const {
        const unsigned t = __reduce_add_sync(0xffffffffu, (unsigned)v << shift);
        if (FW == 32) return (int)t;
        return (int)((t >> shift) & ((1u << (FW & 31)) - 1u));
    }
    __device__ __forceinline__ uint32_t min(uint32_t v) const {
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1) v = ::min(v, __shfl_xor_sync(0xffffffffu, v, o));
        return v;
    }
    __device__ __forceinline__ uint32_t max(uint32_t v) const {
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1) v = ::max(v, __shfl_xor_sync(0xffffffffu, v, o));
        return v;
    }
};

// Number of keys below t, summed as a tree (no long chain of dependent adds).
template <int D>
__device__ __forceinline__ int sim_count_below(const uint32_t (&key)[D], uint32_t t) {
    int part[4] = {0, 0, 0, 0};
#pragma unroll
    for (int i = 0; i < D; ++i) part[i & 3] += key[i] < t ? 1 : 0;
    return (part[0] + part[1]) + (part[2] + part[3]);
}

// Key of rank k (0-based, among the group's n valid keys; a left-out entry has key 0,
// below every key of a number, and a lane holds `zeros` of them) given that it lies in
// [L, U], `below` valid keys are < L and `upto` are <= U.  Each step counts the valid
// keys below a pivot t with one group-wide reduction and keeps the side that holds rank
// k.  The pivot interpolates the rank linearly in value between L and U (a pixel's
// similarities are spread fairly evenly; about 7 steps for a median of 20 to 140), or
// bisects [L, U] in key order after a step that did not halve it, so the key range at
// least halves every two steps (at most 64 steps).  The warp steps until all its groups
// are done.
template <int D, int G>
__device__ __forceinline__ uint32_t sim_kth(const uint32_t (&key)[D], int zeros, const SimGroup<G>& grp, uint32_t L,
                                            uint32_t U, int below, int upto, int k) {
    bool bisect = false;
    for (int it = 0; it < 80; ++it) {
        const bool live = L < U && upto - below > 1;
        if (!__any_sync(0xffffffffu, live)) break;
        uint32_t t;
        if (bisect) {
            t = L + ((U - L) >> 1) + 1u;
        } else {
            const float lv = sim_unkey(L), uv = sim_unkey(U);
            // any pivot in [L + 1, U] is correct; the fraction only steers it
            const float f = __fdividef((float)(k - below) + 0.5f, (float)max(upto - below, 1));
            t = min(max(sim_key(fmaf(uv - lv, f, lv)), L + 1u), U);
        }
        const int c_lane = sim_count_below<D>(key, t) - zeros;
        const int c = grp.sum(live ? c_lane : 0);  // valid keys < t (a finished group adds nothing: its
                                    // pivot need not exceed its zeros)
        if (live) {
            const uint32_t span = U - L;
            if (k < c) {
                U = t - 1u;
                upto = c;
            } else {
                L = t;
                below = c;
            }
            bisect = !bisect && U - L > span / 2;
        }
    }
    uint32_t f = 0;
#pragma unroll
    for (int i = 0; i < D; ++i)
        if (key[i] >= L && key[i] <= U) f = ::max(f, key[i]);
    f = grp.max(f);
    return L == U ? L : f;
}

template <int H>
__global__ void __launch_bounds__(SimShape<H>::THREADS, 512 / SimShape<H>::THREADS) k_similarity(SimArgs a) {
    using S = SimShape<H>;
    constexpr int D = S::D, G = S::G, P = S::P;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* stages = reinterpret_cast<float2*>(smem);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gl = lane % G;  // column offset dc = gl - H
    const int unit = warp * S::GPW + lane / G;
    const int cu = unit % S::TC, rb = unit / S::TC;
    const bool active = gl < D;
    const int lc = active ? gl : D - 1;  // idle lanes read an in-bounds column
    const int dc = gl - H;
    const int hc = active ? a.hc[gl] : -1;
    uint32_t run = 0;  // bit i: row offset i - H belongs to this lane's column of the circle
#pragma unroll
    for (int i = 0; i < 2 * H + 1; ++i)
        if (i - H >= -hc && i - H <= hc && !(dc == 0 && i == H)) run |= 1u << i;
    const int64_t npix = (int64_t)a.rows * a.cols;
    const int nch = (a.m + kSimChunk - 1) / kSimChunk;
    const int my_tiles = a.tiles > (int)blockIdx.x ? (a.tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int steps = my_tiles * nch;

    // one warp copies whole staged rows, a lane per column: the clipped source column is
    // per lane, the clipped source row per warp
    auto issue = [&](int s) {
        const int tile = blockIdx.x + (s / nch) * gridDim.x, ch = s % nch;
        const int r0 = (tile / a.tiles_c) * S::TR, c0 = (tile % a.tiles_c) * S::TC;
        float2* dst = stages + (s & 1) * S::STAGE;
        const int ca = min(max(c0 - H + lane, 0), a.cols - 1);
        const int cb = min(max(c0 - H + lane + 32, 0), a.cols - 1);
        for (int row = warp; row < kSimChunk * S::TRH; row += S::THREADS / 32) {
            const int j = row / S::TRH, tr = row - j * S::TRH;
            const int layer = ch * kSimChunk + j;
            const bool inside = layer < a.m;
            const int r = min(max(r0 - H + tr, 0), a.rows - 1);
            const float2* src = a.unit + (inside ? (int64_t)layer * npix + (int64_t)r * a.cols : 0);
            float2* d = dst + row * S::SW;
            if (lane < S::SW) sim_cp8(d + lane, src + (inside ? ca : 0), inside);
            if (S::SW > 32 && lane + 32 < S::SW) sim_cp8(d + lane + 32, src + (inside ? cb : 0), inside);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    float acc[P][D];
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
        for (int i = 0; i < D; ++i) acc[p][i] = 0.f;
    if (steps > 0) issue(0);
    for (int s = 0; s < steps; ++s) {
        if (s + 1 < steps) {
            issue(s + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        const int ch = s % nch;
        const float2* T = stages + (s & 1) * S::STAGE;
        const int nl = min(kSimChunk, a.m - ch * kSimChunk);
        constexpr int kUnroll = H <= 7 ? 2 : 1;  // two layers in flight where registers allow
#pragma unroll(kUnroll)
        for (int j = 0; j < nl; ++j) {
            const float2* colp = T + j * S::LAYER + (rb * P) * S::SW + cu + lc;
            const float2* ownp = T + j * S::LAYER + (rb * P + H) * S::SW + cu + H;
            float2 own[P], v[D + P - 1];
#pragma unroll
            for (int p = 0; p < P; ++p) own[p] = ownp[p * S::SW];
#pragma unroll
            for (int t = 0; t < D + P - 1; ++t) v[t] = colp[t * S::SW];
            // all real-part products first, then the imaginary ones: the two multiply-adds
            // of an accumulator are far apart in the instruction stream
#pragma unroll
            for (int t = 0; t < D + P - 1; ++t)
#pragma unroll
                for (int p = 0; p < P; ++p)
                    if (t - p >= 0 && t - p < D) acc[p][t - p] = fmaf(own[p].x, v[t].x, acc[p][t - p]);
#pragma unroll
            for (int t = 0; t < D + P - 1; ++t)
#pragma unroll
                for (int p = 0; p < P; ++p)
                    if (t - p >= 0 && t - p < D) acc[p][t - p] = fmaf(own[p].y, v[t].y, acc[p][t - p]);
        }
        if (ch == nch - 1) {
            // the tile's sums are complete: summaries of the group's P pixels, all lanes
            // of the warp in step
            const int tile = blockIdx.x + (s / nch) * gridDim.x;
            const int r0 = (tile / a.tiles_c) * S::TR, c = (tile % a.tiles_c) * S::TC + cu;
            const float fm = (float)a.m;
            const bool col_self = dc == 0 || (dc < 0 && c == 0) || (dc > 0 && c == a.cols - 1);
            const SimGroup<G> grp(lane);
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const int r = r0 + rb * P + p;
                const bool inside = r < a.rows && c < a.cols;
                // the pixel itself, reached through a clipped offset at the image edge
                uint32_t self = 0;
                if (col_self) {
                    self = 1u << H;
                    if (r == 0) self |= (1u << H) - 1u;
                    if (r == a.rows - 1) self |= ((1u << D) - 1u) & ~((2u << H) - 1u);
                }
                const uint32_t vm = inside ? run & ~self : 0u;
                uint32_t key[D];  // 0: left out
                uint32_t kmin = 0xffffffffu, kmax = 0;
                int cnt = 0;
#pragma unroll
                for (int i = 0; i < D; ++i) {
                    const bool use = ((vm >> i) & 1u) && !isnan(acc[p][i]);
                    key[i] = use ? sim_key(acc[p][i]) : 0u;
                    cnt += use ? 1 : 0;
                    kmin = ::min(kmin, use ? key[i] : 0xffffffffu);
                    kmax = ::max(kmax, key[i]);
                }
                const int n = grp.sum(cnt);
                const uint32_t gmax = grp.max(kmax);
                float res = __int_as_float(0x7fffffff);
                if (a.kind == 1) {
                    if (n > 0) res = sim_unkey(gmax) / fm;
                } else {
                    const uint32_t gmin = grp.min(kmin);
                    const int k = n > 0 ? (n - 1) / 2 : 0;  // the median, or the lower one for even n
                    const uint32_t lo = sim_kth<D, G>(key, D - cnt, grp, gmin, gmax, 0, n, k);
                    // upper median: lo again if more than k + 1 keys are <= lo, else the
                    // smallest key above lo
                    int le = sim_count_below<D>(key, lo + 1u) + cnt - D;
                    uint32_t gt = 0xffffffffu;
#pragma unroll
                    for (int i = 0; i < D; ++i) gt = ::min(gt, key[i] > lo ? key[i] : 0xffffffffu);
                    le = grp.sum(le);
                    gt = grp.min(gt);
                    if (n > 0) {
                        res = sim_unkey(lo) / fm;
                        if (!(n & 1)) {
                            const float up = sim_unkey(le >= k + 2 ? lo : gt) / fm;
                            res = (float)(((double)res + (double)up) * 0.5);
                        }
                    }
                }
                if (gl == 0 && inside) a.out[(int64_t)r * a.cols + c] = res;
#pragma unroll
                for (int i = 0; i < D; ++i) acc[p][i] = 0.f;  // next tile
            }
        }
        __syncthreads();  // the buffer just read is refilled by the next issue
    }
}

template <int H>
static dpl_status sim_dispatch_h(SimArgs& a, cudaStream_t st) {
    using S = SimShape<H>;
    a.tiles_c = ceil_div(a.cols, S::TC);
    const int64_t tiles = (int64_t)a.tiles_c * ceil_div(a.rows, S::TR);
    if (tiles > INT32_MAX) return fail(DPL_ERR_UNSUPPORTED, "dpl_similarity: image too large");
    a.tiles = (int)tiles;
    DPL_CUDA_TRY(cudaFuncSetAttribute(k_similarity<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM));
    int dev = 0, sms = 0, per_sm = 0;
    DPL_CUDA_TRY(cudaGetDevice(&dev));
    DPL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DPL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_similarity<H>, S::THREADS, S::SMEM));
    if (per_sm < 1) return fail(DPL_ERR_UNSUPPORTED, "dpl_similarity: kernel does not fit on an SM");
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)sms * per_sm);
    k_similarity<H><<<grid, S::THREADS, S::SMEM, st>>>(a);
    return check_launch("k_similarity");
}

}  // namespace dpl

using namespace dpl;

extern "C" dpl_status dpl_circle_offsets(int max_radius, int min_radius, int sort_output, int32_t* offsets,
                                         int64_t capacity, int64_t* count) {
    if (max_radius < 1) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_circle_offsets: max_radius must be >= 1");
    auto offs = circle_offsets(max_radius, min_radius, sort_output != 0);
    if (count) *count = (int64_t)offs.size();
    if (offsets) {
        const int64_t n = std::min<int64_t>(capacity, (int64_t)offs.size());
        for (int64_t i = 0; i < n; ++i) {
            offsets[2 * i] = offs[i].first;
            offsets[2 * i + 1] = offs[i].second;
        }
    }
    return DPL_OK;
}

extern "C" int dpl_similarity_max_radius(void) { return kSimHMax + 1; }

extern "C" dpl_status dpl_similarity_prep(const float* stack, int is_complex, int64_t nlayers, int64_t rows,
                                          int64_t cols, const uint8_t* mask, int nearest_n, float* unit,
                                          int64_t unit_layers, uint8_t* valid, dpl_stream_t stream) {
    if (nlayers < 0 || rows < 0 || cols < 0 || nearest_n < 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity_prep: bad shape");
    if (nlayers > INT32_MAX) return fail(DPL_ERR_UNSUPPORTED, "dpl_similarity_prep: too many layers");
    int64_t m = nlayers;
    if (nearest_n > 0) {
        m = 0;
        for (int64_t i = 0; i <= nlayers; ++i) m += std::min<int64_t>(nearest_n, nlayers - i);
    }
    if (unit_layers != m)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity_prep: unit_layers must be " + std::to_string(m));
    const int64_t npix = rows * cols;
    if (npix == 0) return DPL_OK;
    if (!valid || (m > 0 && !unit) || (nlayers > 0 && !stack))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity_prep: null pointer");
    if ((is_complex && misaligned_c8(stack)) || misaligned_c8(unit))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity_prep: complex arrays must be 8-byte aligned");
    SimPrepArgs a{};
    a.nin = (int)nlayers;
    a.m = (int)m;
    a.nearest = nearest_n;
    a.is_complex = is_complex != 0;
    a.npix = npix;
    a.stack = stack;
    a.mask = mask;
    a.valid = valid;
    a.unit = reinterpret_cast<float2*>(unit);
    k_sim_prep<<<(unsigned)ceil_div(npix, 256), 256, 0, (cudaStream_t)stream>>>(a);
    return check_launch("k_sim_prep");
}

extern "C" dpl_status dpl_similarity(const float* unit, int64_t nlayers, int64_t rows, int64_t cols,
                                     int search_radius, int kind, float* out, dpl_stream_t stream) {
    if (nlayers < 0 || rows < 0 || cols < 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity: bad shape");
    if (kind != 0 && kind != 1) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity: kind must be 0 or 1");
    if (search_radius < 1) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity: search_radius must be >= 1");
    if (search_radius > kSimHMax + 1)
        return fail(DPL_ERR_UNSUPPORTED, "dpl_similarity: search_radius above " + std::to_string(kSimHMax + 1));
    if (rows > INT32_MAX || cols > INT32_MAX || nlayers > INT32_MAX)
        return fail(DPL_ERR_UNSUPPORTED, "dpl_similarity: image too large");
    const int64_t npix = rows * cols;
    if (npix == 0) return DPL_OK;
    if (!out || (nlayers > 0 && !unit)) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity: null pointer");
    if (misaligned_c8(unit))  // read with 8-byte cp.async copies
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_similarity: complex arrays must be 8-byte aligned");
    const int H = search_radius - 1;
    SimArgs a{};
    int K = 0, base[2 * kSimHMax + 1];
    if (H > 0 && !circle_columns(search_radius, H, a.hc, base, &K))
        return fail(DPL_ERR_UNSUPPORTED, "dpl_similarity: search circle has a non-contiguous column");
    if (K == 0 || nlayers == 0) {
        // no offsets, or no layers (every pixel invalid): all NaN
        DPL_CUDA_TRY(cudaMemsetAsync(out, 0xff, (size_t)npix * sizeof(float), (cudaStream_t)stream));
        return DPL_OK;
    }
    a.m = (int)nlayers;
    a.rows = (int)rows;
    a.cols = (int)cols;
    a.kind = kind;
    a.unit = reinterpret_cast<const float2*>(unit);
    a.out = out;
    cudaStream_t st = (cudaStream_t)stream;
    switch (H) {
        case 1: return sim_dispatch_h<1>(a, st);
        case 2: return sim_dispatch_h<2>(a, st);
        case 3: return sim_dispatch_h<3>(a, st);
        case 4: return sim_dispatch_h<4>(a, st);
        case 5: return sim_dispatch_h<5>(a, st);
        case 6: return sim_dispatch_h<6>(a, st);
        case 7: return sim_dispatch_h<7>(a, st);
        case 8: return sim_dispatch_h<8>(a, st);
        case 9: return sim_dispatch_h<9>(a, st);
        case 10: return sim_dispatch_h<10>(a, st);
        case 11: return sim_dispatch_h<11>(a, st);
        case 12: return sim_dispatch_h<12>(a, st);
        case 13: return sim_dispatch_h<13>(a, st);
        case 14: return sim_dispatch_h<14>(a, st);
        default: return sim_dispatch_h<15>(a, st);
    }
}
