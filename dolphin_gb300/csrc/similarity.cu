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
//                median by a radix selection on order-preserving keys with one
//                group-wide count per bit (redux.sync), from the highest bit in which
//                the group's smallest and largest key differ.  The pixel itself (which
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
constexpr int kSimThreads = 512;
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
// the 2H + 1 neighbours in column c + dc.  A CTA of 512 threads owns TC x TR pixels.
template <int H>
struct SimShape {
    static constexpr int D = 2 * H + 1;
    static constexpr int G = D <= 4 ? 4 : D <= 8 ? 8 : D <= 16 ? 16 : 32;
    static constexpr int P = H <= 10 ? 4 : 2;
    static constexpr int GPW = 32 / G;
    static constexpr int UNITS = kSimThreads / 32 * GPW;
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

// k-th smallest (0-based) of the n keys that the group holds (key[i] of every lane where
// bit i of vm is set; all in [lo, hi]): radix selection from the highest bit in which lo
// and hi differ, one group-wide count per bit, stopping as soon as one key is left.
template <int D>
__device__ __forceinline__ uint32_t sim_kth(const uint32_t (&key)[D], uint32_t vm, unsigned gmask, uint32_t lo,
                                            uint32_t hi, int n, int k) {
    if (lo == hi) return lo;
    int b = 31 - __clz(lo ^ hi);
    uint32_t prefix = lo & ~(0xffffffffu >> (31 - b));
    int cand = n;
    for (; b >= 0; --b) {
        const uint32_t want = prefix >> b;  // bit b of the prefix is 0
        int c0 = 0;
#pragma unroll
        for (int i = 0; i < D; ++i) c0 += (((vm >> i) & 1u) && (key[i] >> b) == want) ? 1 : 0;
        c0 = (int)__reduce_add_sync(gmask, (unsigned)c0);
        if (k < c0) {
            cand = c0;
        } else {
            k -= c0;
            prefix |= 1u << b;
            cand -= c0;
        }
        if (cand == 1) {
            const uint32_t w = prefix >> b;
            uint32_t f = 0;
#pragma unroll
            for (int i = 0; i < D; ++i)
                if (((vm >> i) & 1u) && (key[i] >> b) == w) f = key[i];
            return __reduce_max_sync(gmask, f);
        }
    }
    return prefix;
}

template <int H>
__global__ void __launch_bounds__(kSimThreads, 1) k_similarity(SimArgs a) {
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
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane / G * G));
    const int64_t npix = (int64_t)a.rows * a.cols;
    const int nch = (a.m + kSimChunk - 1) / kSimChunk;
    const int my_tiles = a.tiles > (int)blockIdx.x ? (a.tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int steps = my_tiles * nch;

    auto issue = [&](int s) {
        const int tile = blockIdx.x + (s / nch) * gridDim.x, ch = s % nch;
        const int r0 = (tile / a.tiles_c) * S::TR, c0 = (tile % a.tiles_c) * S::TC;
        float2* dst = stages + (s & 1) * S::STAGE;
        for (int e = threadIdx.x; e < S::STAGE; e += kSimThreads) {
            const int j = e / S::LAYER, rem = e - j * S::LAYER;
            const int tr = rem / S::SW, tc = rem - tr * S::SW;
            const int layer = ch * kSimChunk + j;
            const int r = min(max(r0 - H + tr, 0), a.rows - 1);
            const int c = min(max(c0 - H + tc, 0), a.cols - 1);
            const bool inside = layer < a.m;
            const float2* src = a.unit + (inside ? (int64_t)layer * npix + (int64_t)r * a.cols + c : 0);
            sim_cp8(dst + e, src, inside);
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
#pragma unroll 1
        for (int j = 0; j < nl; ++j) {
            const float2* colp = T + j * S::LAYER + (rb * P) * S::SW + cu + lc;
            const float2* ownp = T + j * S::LAYER + (rb * P + H) * S::SW + cu + H;
            float2 own[P];
#pragma unroll
            for (int p = 0; p < P; ++p) own[p] = ownp[p * S::SW];
#pragma unroll
            for (int t = 0; t < D + P - 1; ++t) {
                const float2 v = colp[t * S::SW];
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    const int i = t - p;
                    if (i >= 0 && i < D) acc[p][i] = fmaf(own[p].y, v.y, fmaf(own[p].x, v.x, acc[p][i]));
                }
            }
        }
        if (ch == nch - 1) {
            // the tile's sums are complete: summaries of the group's P pixels
            const int tile = blockIdx.x + (s / nch) * gridDim.x;
            const int r0 = (tile / a.tiles_c) * S::TR, c = (tile % a.tiles_c) * S::TC + cu;
            const float fm = (float)a.m;
            const bool col_self = dc == 0 || (dc < 0 && c == 0) || (dc > 0 && c == a.cols - 1);
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const int r = r0 + rb * P + p;
                if (r < a.rows && c < a.cols) {  // uniform over the group
                    uint32_t key[D];
                    uint32_t vm = 0, kmin = 0xffffffffu, kmax = 0;
                    int cnt = 0;
#pragma unroll
                    for (int i = 0; i < D; ++i) {
                        const int dr = i - H;
                        const bool row_self = dr == 0 || (dr < 0 && r == 0) || (dr > 0 && r == a.rows - 1);
                        const bool use = dr >= -hc && dr <= hc && !(dc == 0 && dr == 0) && !(row_self && col_self) &&
                                         !isnan(acc[p][i]);
                        key[i] = sim_key(acc[p][i]);
                        if (use) {
                            vm |= 1u << i;
                            ++cnt;
                            kmin = min(kmin, key[i]);
                            kmax = max(kmax, key[i]);
                        }
                    }
                    const int n = (int)__reduce_add_sync(gmask, (unsigned)cnt);
                    float res = __int_as_float(0x7fffffff);
                    if (n > 0) {
                        const uint32_t gmax = __reduce_max_sync(gmask, kmax);
                        if (a.kind == 1) {
                            res = sim_unkey(gmax) / fm;
                        } else {
                            const uint32_t gmin = __reduce_min_sync(gmask, kmin);
                            const int k = (n - 1) / 2;  // the median, or the lower one for even n
                            const uint32_t lo = sim_kth<D>(key, vm, gmask, gmin, gmax, n, k);
                            res = sim_unkey(lo) / fm;
                            if (!(n & 1)) {
                                // upper median: lo again if more than k + 1 keys are <= lo,
                                // else the smallest key above lo
                                int le = 0;
                                uint32_t gt = 0xffffffffu;
#pragma unroll
                                for (int i = 0; i < D; ++i) {
                                    if ((vm >> i) & 1u) {
                                        le += key[i] <= lo ? 1 : 0;
                                        if (key[i] > lo) gt = min(gt, key[i]);
                                    }
                                }
                                le = (int)__reduce_add_sync(gmask, (unsigned)le);
                                gt = __reduce_min_sync(gmask, gt);
                                const float up = sim_unkey(le >= k + 2 ? lo : gt) / fm;
                                res = (float)(((double)res + (double)up) * 0.5);
                            }
                        }
                    }
                    if (gl == 0) a.out[(int64_t)r * a.cols + c] = res;
                }
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
    DPL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_similarity<H>, kSimThreads, S::SMEM));
    if (per_sm < 1) return fail(DPL_ERR_UNSUPPORTED, "dpl_similarity: kernel does not fit on an SM");
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)sms * per_sm);
    k_similarity<H><<<grid, kSimThreads, S::SMEM, st>>>(a);
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
