// Phase linking: run_phase_linking (phase_link/_core.py:67-249) on one GPU.
//
// Pipeline (one stream, no host round trip until the final status check):
//   k_prep   -- per input pixel: nodata |= any NaN, ps &= !nodata, the masked stack
//               (NaN and ignored pixels -> 0, the reference's `where(mask, z, 0)`)
//               transposed to pixel-major (rows, cols, N), nanmean|z| if needed, and a
//               per-SLC "has a non-NaN sample" bitmask for the all-NaN check.
//   k_pixel  -- one warp per output pixel, matrices in the warp's shared memory:
//               SHP-masked sample coherence (covariance.py:110-142), baseline lag
//               (_core.py:333-337), closure phases (_closure_phase.py:6-40),
//               |Gamma| regularisation and Cholesky inverse (_core.py:452-472),
//               EMI by LU + inverse iteration (_eigenvalues.py:139-205) or EVD by
//               power iteration (:93-136) with the reference's per-pixel fallback,
//               referencing (_core.py:530-534), temporal coherence (metrics.py:74-97)
//               and CRLB (crlb.py:132-189).  Written pixel-major.
//   k_post   -- per output pixel: unit phasors, PS filling (_ps_filling.py:16-97),
//               use_slc_amp, nodata NaNs (_core.py:207-238), transposed to the
//               reference's (N, rows, cols) output layout.
//
// Precision: float32 throughout, as in the reference (jax with x64 disabled).
// Iteration caps and tolerances are the reference's (<= 49 iterations, 1e-5).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <sstream>
#include <vector>

#include "dpl_common.cuh"
#include "pix_args.cuh"

namespace dpl {

__device__ __forceinline__ int clamp_start_i(int center, int half, int size, int dim) {
    int s = center - half;
    s = s < 0 ? 0 : s;
    return s > dim - size ? dim - size : s;
}

// ---------------------------------------------------------------------------------
// k_prep
// ---------------------------------------------------------------------------------
constexpr int kPrepPix = 64;

__global__ void __launch_bounds__(256) k_prep(const cfloat* __restrict__ slc, int n, int64_t npix,
                                              const uint8_t* __restrict__ nodata_in,
                                              const uint8_t* __restrict__ ps_in, int mask_input_ps,
                                              int nan_is_nodata, uint8_t* __restrict__ flags,
                                              cfloat* __restrict__ zt,
                                              float* __restrict__ avgmag, unsigned int* __restrict__ valid_bits) {
    extern __shared__ cfloat prep_s[];  // [kPrepPix][n + 1]
    __shared__ uint8_t ign[kPrepPix];
    __shared__ unsigned long long vbits;
    const int ld = n + 1;
    const int64_t p0 = (int64_t)blockIdx.x * kPrepPix;
    if (threadIdx.x == 0) vbits = 0ull;
    for (int i = threadIdx.x; i < n * kPrepPix; i += blockDim.x) {
        const int t = i / kPrepPix, px = i - t * kPrepPix;
        const int64_t p = p0 + px;
        prep_s[px * ld + t] = p < npix ? slc[(int64_t)t * npix + p] : cmake(0.f, 0.f);
    }
    __syncthreads();
    if (threadIdx.x < kPrepPix) {
        const int px = threadIdx.x;
        const int64_t p = p0 + px;
        if (p < npix) {
            bool anynan = false;
            unsigned long long vb = 0ull;
            float msum = 0.f;
            int mcnt = 0;
            for (int t = 0; t < n; ++t) {
                cfloat z = prep_s[px * ld + t];
                bool nan = cisnan(z);
                anynan |= nan;
                if (!nan) {
                    vb |= 1ull << t;
                    float m = hypotf(z.re, z.im);
                    msum = mcnt == 0 ? m : fadd(msum, m);
                    ++mcnt;
                }
            }
            // run_phase_linking marks a pixel with any NaN as nodata (_core.py:181);
            // the bare covariance masks NaN samples one by one (covariance.py:122-123)
            const bool nodata = (nodata_in && nodata_in[p]) || (nan_is_nodata && anynan);
            const bool ps = ps_in && ps_in[p] && !nodata;
            const bool ignore = nodata || (mask_input_ps && ps);
            flags[p] = (nodata ? kNodata : 0) | (ps ? kPs : 0) | (ignore ? kIgnore : 0);
            ign[px] = ignore;
            if (avgmag) avgmag[p] = fdiv(msum, (float)mcnt);
            if (vb) atomicOr(&vbits, vb);
        } else {
            ign[px] = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && vbits) {
        atomicOr(valid_bits, (unsigned int)(vbits & 0xffffffffull));
        atomicOr(valid_bits + 1, (unsigned int)(vbits >> 32));
    }
    for (int i = threadIdx.x; i < kPrepPix * n; i += blockDim.x) {
        const int px = i / n, t = i - px * n;
        const int64_t p = p0 + px;
        if (p < npix) {
            cfloat z = prep_s[px * ld + t];
            if (ign[px] || cisnan(z)) z = cmake(0.f, 0.f);
            zt[p * n + t] = z;
        }
    }
}

}  // namespace dpl

#include "solver.cuh"
#include "eigh.cuh"

namespace dpl {

// ---------------------------------------------------------------------------------
// covariance (covariance.py:110-170): raw sums into packed C, then normalisation
// ---------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t row_mask(const PixArgs& a, int64_t p, int wa, int wx, int lane) {
    const uint64_t full = wx >= 64 ? ~0ull : ((1ull << wx) - 1ull);
    if (a.nb_bits) {
        const uint32_t* w = a.nb_bits + ((p * (2 * a.hy + 1) + wa) * a.wpr);
        uint64_t m = w[0];
        if (a.wpr > 1) m |= (uint64_t)w[1] << 32;
        return m & full;
    }
    if (a.nb_u8) {
        const uint8_t* b = a.nb_u8 + (p * (2 * a.hy + 1) + wa) * wx;
        uint32_t lo = __ballot_sync(0xffffffffu, lane < wx && b[lane] != 0);
        uint32_t hi = __ballot_sync(0xffffffffu, lane + 32 < wx && b[lane + 32] != 0);
        return ((uint64_t)hi << 32) | lo;
    }
    return full;
}

template <int NB>
__device__ void warp_covariance(const PixArgs& a, int64_t p, cfloat* C, cfloat* stg, float* amp, int lane,
                                int* count_out) {
    const int n = a.n, wy = 2 * a.hy + 1, wx = 2 * a.hx + 1, np = a.np;
    const int out_r = (int)(p / a.out_cols), out_c = (int)(p - (int64_t)out_r * a.out_cols);
    const int in_r = a.sy / 2 + out_r * a.sy, in_c = a.sx / 2 + out_c * a.sx;
    const int r0 = clamp_start_i(in_r, a.hy, wy, a.rows), c0 = clamp_start_i(in_c, a.hx, wx, a.cols);
    int count = 0;
    for (int rb = 0; rb < NB; ++rb) {
        for (int cb = rb; cb < NB; ++cb) {
            float are[32], aim[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) are[j] = aim[j] = 0.f;
            for (int wa = 0; wa < wy; ++wa) {
                const uint64_t rm = row_mask(a, p, wa, wx, lane);
                if (rb == 0 && cb == 0) count += __popcll(rm);
                if (rm == 0ull) continue;
                const cfloat* src = a.zt + ((int64_t)(r0 + wa) * a.cols + c0) * n;
                __syncwarp();
                for (int idx = lane; idx < a.stg; idx += 32) {
                    const int b = idx / np, t = idx - b * np;
                    stg[idx] = (b < wx && t < n) ? src[b * n + t] : cmake(0.f, 0.f);
                }
                __syncwarp();
                for (int wb = 0; wb < wx; ++wb) {
                    if (!((rm >> wb) & 1ull)) continue;
                    const cfloat* s = stg + wb * np;
                    const cfloat zi = s[rb * 32 + lane];
                    const float4* sj = reinterpret_cast<const float4*>(s + cb * 32);
#pragma unroll
                    for (int j2 = 0; j2 < 16; ++j2) {
                        const float4 q = sj[j2];
                        are[2 * j2] += zi.re * q.x + zi.im * q.y;
                        aim[2 * j2] += zi.im * q.x - zi.re * q.y;
                        are[2 * j2 + 1] += zi.re * q.z + zi.im * q.w;
                        aim[2 * j2 + 1] += zi.im * q.z - zi.re * q.w;
                    }
                }
            }
            const int row = rb * 32 + lane;
            if (row < n) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int col = cb * 32 + j;
                    if (col <= row) C[pk(row, col)] = cmake(are[j], aim[j]);
                    else if (rb != cb && col < n) C[pk(col, row)] = cmake(are[j], -aim[j]);
                }
            }
        }
    }
    __syncwarp();
    // C = numer / sqrt(amp_i amp_j) where that root > 1e-6, else 0
    for (int i = lane; i < n; i += 32) amp[i] = C[pk(i, i)].re;
    __syncwarp();
    for (int i = 0; i < n; ++i) {
        const float ai = amp[i];
        for (int j = lane; j <= i; j += 32) {
            const float s = fsqrt(fmul(ai, amp[j]));
            const cfloat c = C[pk(i, j)];
            C[pk(i, j)] = s > 1e-6f ? cmake(fdiv(c.re, s), fdiv(c.im, s)) : cmake(0.f, 0.f);
        }
    }
    __syncwarp();
    if (count_out) *count_out = count;
}

template <int NB, int MODE, bool kLU>
__global__ void __launch_bounds__(256) k_pixel(PixArgs a) {
    extern __shared__ __align__(16) unsigned char pix_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    unsigned char* base = pix_smem + warp * a.warp_bytes;
    SolveMats m;
    m.C = reinterpret_cast<cfloat*>(base + a.off_C);
    m.G = reinterpret_cast<float*>(base + a.off_G);
    m.ldg = a.ldg;
    m.R = reinterpret_cast<cfloat*>(base + a.off_S);
    m.v = reinterpret_cast<cfloat*>(base + a.off_v);
    m.d = reinterpret_cast<float*>(base + a.off_d);
    m.piv = reinterpret_cast<int*>(base + a.off_piv);
    const int n = a.n;
    const int64_t total = kLU ? (int64_t)*a.list_count : a.npix;
    for (int64_t idx = (int64_t)blockIdx.x * nwarps + warp; idx < total; idx += (int64_t)gridDim.x * nwarps) {
        const int64_t p = kLU ? (int64_t)a.list[idx] : idx;
        if (MODE == kSolveOnly) {
            __syncwarp();
            if (a.Cplanar) {
                // unnormalised planar sums: C_ij = numer_ij r_i r_j, r = 1 / sqrt(amp), 0 where
                // r_i r_j >= 1e6 (covariance.py:131-142)
                const float* src = a.Cplanar + p * n * n;
                for (int i = 0; i < n; ++i) {
                    const float ri = __frsqrt_rn(src[i]);
                    for (int j = lane; j <= i; j += 32) {
                        const float f = ri * __frsqrt_rn(src[j]);
                        const bool ok = f < 1e6f;
                        const int o = i * (i - 1) / 2 + j;  // pair (i, j), i > j
                        m.C[pk(i, j)] = i == j ? cmake(ok ? src[i] * f : 0.f, 0.f)
                                               : (ok ? cmake(src[n + 2 * o] * f, src[n + 2 * o + 1] * f)
                                                     : cmake(0.f, 0.f));
                    }
                }
            } else {
                const cfloat* src = a.Cin + p * n * n;
                for (int i = 0; i < n; ++i)
                    for (int j = lane; j <= i; j += 32) m.C[pk(i, j)] = src[i * n + j];
            }
            __syncwarp();
        } else {
            int count = 0;
            warp_covariance<NB>(a, p, m.C, m.R, m.d, lane, &count);
            if (a.counts && lane == 0) a.counts[p] = count;
        }
        if (MODE == kCovOnly) {
            cfloat* dst = a.Cout + p * n * n;
            for (int i = 0; i < n; ++i)
                for (int j = lane; j < n; j += 32) dst[i * n + j] = cget(m.C, i, j);
            __syncwarp();
        } else {
            solve_pixel<NB, kLU>(a, p, m, lane);
        }
    }
}

// ---------------------------------------------------------------------------------
// k_eigh: the dense eigensolver for the listed non-converged pixels (eigh.cuh), one
// warp per pixel, a persistent grid over the list
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(32) k_eigh(PixArgs a, EighLayout L) {
    extern __shared__ __align__(16) unsigned char eigh_smem[];
    const int lane = threadIdx.x;
    cfloat* C = reinterpret_cast<cfloat*>(eigh_smem + L.off_C);
    cfloat* A = reinterpret_cast<cfloat*>(eigh_smem + L.off_A);
    double* G = reinterpret_cast<double*>(eigh_smem + L.off_A);  // |Gamma| work matrix, until A is formed
    double* col = reinterpret_cast<double*>(eigh_smem + L.off_col);
    const EighVec V = eigh_vectors(eigh_smem, L);
    cfloat* w = V.w;
    const int n = a.n, ld = L.ld, lag = a.baseline_lag;
    const int count = *a.nc_count;
    for (int idx = blockIdx.x; idx < count; idx += gridDim.x) {
        const int64_t p = a.nc_list[idx];
        __syncwarp();
        // the coherence, normalised as the solvers read it
        if (a.Cplanar) {
            const float* src = a.Cplanar + p * n * n;
            float* rv = reinterpret_cast<float*>(w);
            for (int i = lane; i < n; i += 32) rv[i] = __frsqrt_rn(src[i]);
            __syncwarp();
            for (int i = lane; i < n; i += 32) {
                const float f = rv[i] * rv[i];
                C[i * ld + i] = cmake(f < 1e6f ? src[i] * f : 0.f, 0.f);
            }
            // lower pairs (r, c), c < r, at e = r(r-1)/2 + c: every lane walks the pairs
            // e = lane, lane + 32, ..., so its loads do not wait on one another
            const int npairs = n * (n - 1) / 2;
            int r = 1, c = lane;
            while (c >= r) c -= r++;
            for (int e = lane; e < npairs; e += 32) {
                const float f = rv[r] * rv[c];
                cfloat v = f < 1e6f ? cmake(src[n + 2 * e] * f, src[n + 2 * e + 1] * f) : cmake(0.f, 0.f);
                if (lag > 0 && r - c >= lag) v = cmake(0.f, 0.f);
                C[r * ld + c] = v;
                C[c * ld + r] = cconj(v);
                c += 32;
                while (c >= r) c -= r++;
            }
        } else {
            const cfloat* src = a.Cin + p * n * n;
            for (int r = 0; r < n; ++r)
                for (int c = lane; c <= r; c += 32) {
                    cfloat v = src[r * n + c];
                    if (lag > 0 && r - c >= lag) v = cmake(0.f, 0.f);
                    C[r * ld + c] = v;
                    C[c * ld + r] = cconj(v);
                }
        }
        __syncwarp();
        const bool evd = a.est[p] == 0;  // the estimator the solver chose
        bool ok = true;
        if (!evd) {
            // |Gamma| + 1e-6 I inverted in double; A = |Gamma|^{-1} o C (lower triangles)
            for (int i = 0; i < n; ++i)
                for (int j = lane; j <= i; j += 32)
                    G[i * ld + j] = (double)s_gamma(a, C[i * ld + j], i == j) + (i == j ? 1e-6 : 0.0);
            ok = e_inverse_spd(G, ld, col, col + kEighMaxN, n, lane);
            if (ok)  // in place: each element of G is read, then A written over it, by one lane
                for (int i = 0; i < n; ++i)
                    for (int j = lane; j <= i; j += 32) {
                        const float gi = (float)G[i * ld + j];
                        A[i * ld + j] = cscale(C[i * ld + j], gi);
                    }
        } else {
            for (int i = 0; i < n; ++i)
                for (int j = lane; j <= i; j += 32) {
                    const cfloat c = C[i * ld + j];
                    A[i * ld + j] = cscale(c, sqrtf(c.re * c.re + c.im * c.im));
                }
        }
        __syncwarp();
        if (ok) {
            // EMI: the eigenvalue nearest the shift 0.99; EVD: the largest in magnitude
            cfloat* x = V.pw;
            const float lambda = e_eigpair(A, n, ld, evd, V, x, lane);
            {
                float s2 = 0.f;
                for (int i = lane; i < n; i += 32) s2 += cabs2(x[i]);
                s2 = warp_sum(s2);
                const float scale = (evd ? 1.f : sqrtf((float)n)) / sqrtf(s2);
                const cfloat rot = cconj(fphasor(x[a.ref_idx]));
                __syncwarp();
                for (int i = lane; i < n; i += 32) {
                    const cfloat v = cmul(cscale(x[i], scale), rot);
                    a.vout[p * n + i] = v;
                    w[i] = fphasor(v);
                }
                __syncwarp();
                // temporal coherence over pairs c < r, as the solvers compute it
                float sre = 0.f, sim = 0.f;
                int cnt = 0;
                for (int r = 1; r < n; ++r)
                    for (int c = lane; c < r; c += 32) {
                        const cfloat u = fphasor(C[r * ld + c]);
                        const cfloat t = cconj(cmulc(cmul(u, w[c]), w[r]));
                        if (!cisnan(t)) {
                            sre += t.re;
                            sim += t.im;
                            ++cnt;
                        }
                    }
                sre = warp_sum(sre);
                sim = warp_sum(sim);
                cnt = warp_sum_int(cnt);
                if (lane == 0) {
                    const float fc = (float)cnt;
                    const float tc = hypotf(sre / fc, sim / fc);
                    a.tcoh[p] = isfinite(tc) ? tc : 0.f;
                    a.eig[p] = lambda;
                }
            }
        }
        if (lane == 0 && a.nc_flag) a.nc_flag[p] = 1;
        __syncwarp();
    }
}

}  // namespace dpl

#include "solver64.cuh"
#include "cov_tc.cuh"

namespace dpl {

// planar sums (tensor-core layout) -> normalised full (npix, n, n) complex: C_ij =
// numer_ij r_i r_j with r = 1 / sqrt(amp), 0 where r_i r_j >= 1e6 (covariance.py:131-142)
__global__ void k_unpack_planar(const float* __restrict__ Cg, int n, int64_t npix, cfloat* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nn = (int64_t)n * n;
    if (e >= npix * nn) return;
    const int64_t p = e / nn;
    const int r = (int)(e - p * nn), i = r / n, j = r - i * n;
    const float* src = Cg + p * nn;
    const int hi = i > j ? i : j, lo = i > j ? j : i;  // the stored pair (hi, lo)
    const float f = __frsqrt_rn(src[hi]) * __frsqrt_rn(src[lo]);
    const bool ok = f < 1e6f;
    cfloat v;
    if (i == j) {
        v = cmake(ok ? src[i] * f : 0.f, 0.f);
    } else {
        const int o = n + 2 * (hi * (hi - 1) / 2 + lo);
        v = ok ? cmake(src[o] * f, i > j ? src[o + 1] * f : -(src[o + 1] * f)) : cmake(0.f, 0.f);
    }
    out[e] = v;
}

// ---------------------------------------------------------------------------------
// k_post: phasors, PS fill, use_slc_amp, nodata, transposition to (N, rows, cols)
// ---------------------------------------------------------------------------------
struct PostArgs {
    int n, rows, cols, sy, sx, out_rows, out_cols;
    const cfloat* slc;  // original stack (N, rows, cols)
    const uint8_t* flags;
    const float* mag;   // brightness for the PS argmax (avg_mag or nanmean |slc|)
    const cfloat* V;    // (P, n) referenced eigenvectors
    const float* CR;    // (P, n)
    int use_max_ps, use_slc_amp, ref_idx;
    cfloat* cpx;        // (n, P)
    float* tcoh;        // (P), in/out
    float* crlb;        // (n, P)
    int* status;
};

__global__ void __launch_bounds__(256) k_post(PostArgs a) {
    const int64_t P = (int64_t)a.out_rows * a.out_cols;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int orow = (int)(p / a.out_cols), ocol = (int)(p - (int64_t)orow * a.out_cols);
    const int64_t npix_in = (int64_t)a.rows * a.cols;
    bool all_nodata = true, any_ps = false;
    float best = -INFINITY;
    int br = -1, bc = -1, nps = 0;
    for (int dr = 0; dr < a.sy; ++dr) {
        for (int dc = 0; dc < a.sx; ++dc) {
            const int r = orow * a.sy + dr, c = ocol * a.sx + dc;
            const uint8_t f = a.flags[(int64_t)r * a.cols + c];
            all_nodata &= (f & kNodata) != 0;
            if (f & kPs) {
                any_ps = true;
                ++nps;
                const float mg = a.mag[(int64_t)r * a.cols + c];
                if (!isnan(mg) && mg > best) {
                    best = mg;
                    br = r;
                    bc = c;
                }
            }
        }
    }
    if (any_ps && a.use_max_ps && br < 0) atomicExch(a.status, (int)DPL_ERR_INVALID_ARGUMENT);
    const int in_r = a.sy / 2 + orow * a.sy, in_c = a.sx / 2 + ocol * a.sx;
    for (int t = 0; t < a.n; ++t) {
        cfloat out = cphasor(a.V[p * a.n + t]);
        if (any_ps) {
            const float amp = cabs(out);
            if (a.use_max_ps) {
                if (br >= 0) {
                    const cfloat zt = a.slc[(int64_t)t * npix_in + (int64_t)br * a.cols + bc];
                    const cfloat zr = a.slc[(int64_t)a.ref_idx * npix_in + (int64_t)br * a.cols + bc];
                    out = cscale(cmul(cphasor(zt), cconj(cphasor(zr))), amp);
                }
            } else {
                float sre = 0.f, sim = 0.f;
                int cnt = 0;
                for (int dr = 0; dr < a.sy; ++dr) {
                    for (int dc = 0; dc < a.sx; ++dc) {
                        const int r = orow * a.sy + dr, c = ocol * a.sx + dc;
                        if (!(a.flags[(int64_t)r * a.cols + c] & kPs)) continue;
                        const int64_t q = (int64_t)r * a.cols + c;
                        const cfloat z = cmul(a.slc[(int64_t)t * npix_in + q], cconj(cphasor(a.slc[q])));
                        if (cisnan(z)) continue;
                        sre += z.re;
                        sim += z.im;
                        ++cnt;
                    }
                }
                const cfloat avg = cmake(fdiv(sre, (float)cnt), fdiv(sim, (float)cnt));
                out = cscale(cphasor(avg), amp);
            }
        }
        if (a.use_slc_amp) {
            const cfloat z = a.slc[(int64_t)t * npix_in + (int64_t)in_r * a.cols + in_c];
            out = cscale(cphasor(out), cabs(z));
        }
        if (all_nodata) out = cmake(nanf(""), 0.f);
        a.cpx[(int64_t)t * P + p] = out;
        a.crlb[(int64_t)t * P + p] = a.CR[p * a.n + t];
    }
    float tc = a.tcoh[p];
    if (any_ps) tc = 1.f;
    if (all_nodata) tc = nanf("");
    a.tcoh[p] = tc;
}

// ---------------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------------
static void fill_pix_layout(PixArgs& a, int n, int wx, bool lu = false) {
    PixLayout L = make_layout(n, wx, lu);
    a.n = n;
    a.np = L.np;
    a.stg = L.stg;
    a.ldg = L.ldg;
    a.off_C = L.off_C;
    a.off_G = L.off_G;
    a.off_S = L.off_S;
    a.off_v = L.off_v;
    a.off_d = L.off_d;
    a.off_piv = L.off_piv;
    a.warp_bytes = L.bytes;
}

// Optional timing of the per-pixel kernel: CUDA events recorded on the launch
// stream around each k_pixel launch while enabled (used by the benchmark).
struct PixTimer {
    std::mutex mu;
    bool on = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[2];  // [0] covariance, [1] solver
};
static PixTimer g_timer;


template <class F>
static dpl_status timed(cudaStream_t s, int slot, F&& launch) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    {
        std::lock_guard<std::mutex> g(g_timer.mu);
        if (g_timer.on) {
            DPL_CUDA_TRY(cudaEventCreate(&e0));
            DPL_CUDA_TRY(cudaEventCreate(&e1));
            g_timer.ev[slot].emplace_back(e0, e1);
        }
    }
    if (e0) DPL_CUDA_TRY(cudaEventRecord(e0, s));
    dpl_status st = launch();
    if (e1) DPL_CUDA_TRY(cudaEventRecord(e1, s));
    return st;
}

template <int MODE, bool kLU>
static dpl_status launch_pixel_pass(const PixArgs& a, cudaStream_t s) {
    // as many warps per CTA as fit ~100 KB (two CTAs per SM), at most 8
    int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (size_t)(100 * 1024) / a.warp_bytes));
    size_t smem = (size_t)warps * a.warp_bytes;
    if (smem > 220 * 1024) return fail(DPL_ERR_UNSUPPORTED, "per-pixel shared memory exceeds the SM limit");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto go = [&](auto kernel) -> dpl_status {
        DPL_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        DPL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, warps * 32, smem));
        const int64_t resident = (int64_t)std::max(1, per_sm) * std::max(1, sms);
        int64_t grid = kLU ? resident : std::min<int64_t>((a.npix + warps - 1) / warps, resident * 8);
        kernel<<<(unsigned)std::max<int64_t>(grid, 1), warps * 32, smem, s>>>(a);
        return check_launch(kLU ? "k_pixel (LU pass)" : "k_pixel");
    };
    if (a.n <= 32) return go(k_pixel<1, MODE, kLU>);
    return go(k_pixel<2, MODE, kLU>);
}

// ---------------------------------------------------------------------------------
// register-solver dispatch: K = n rounded up to even (at least 4), or a.slots when
// that is larger (a tuned choice); G threads per pixel from solver_lanes
// ---------------------------------------------------------------------------------
dpl_status launch_solve_reg_a(int K, int G, const PixArgs& a, cudaStream_t s);
dpl_status launch_solve_reg_b(int K, int G, const PixArgs& a, cudaStream_t s);
dpl_status launch_solve_reg_c(int K, int G, const PixArgs& a, cudaStream_t s);
dpl_status launch_solve_reg_d(int K, int G, const PixArgs& a, cudaStream_t s);
dpl_status launch_solve_reg_e(int K, int G, const PixArgs& a, cudaStream_t s);

dpl_status launch_solve_reg(const PixArgs& a, cudaStream_t s) {
    int K = std::max(4, (a.n + 1) & ~1);
    if (a.slots > K && a.slots <= 64 && (a.slots & 1) == 0 && (K > 32) == (a.slots > 32)) K = a.slots;
    const int G = solver_lanes(K, a.lanes);
    if (K <= 16) return launch_solve_reg_a(K, G, a, s);
    if (K <= 32) return launch_solve_reg_b(K, G, a, s);
    if (K <= 44) return launch_solve_reg_c(K, G, a, s);
    if (K <= 54) return launch_solve_reg_d(K, G, a, s);
    return launch_solve_reg_e(K, G, a, s);
}

// Main pass (Cholesky inverse iteration) and, for the pixels it lists, the LU pass.
// `fb` holds a counter followed by room for every pixel index.
// FP64 form: covariance and solver in double, one warp per pixel
static dpl_status launch_pixel64(const PixArgs& a, cudaStream_t s) {
    const Pix64Layout L = make_layout64(a.n, a.stg);
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(4, (size_t)(200 * 1024) / L.bytes));
    const size_t smem = (size_t)warps * L.bytes;
    if (smem > (size_t)227 * 1024) return fail(DPL_ERR_UNSUPPORTED, "fp64 form: window or nslc too large");
    int dev = 0, sms = 0;
    DPL_CUDA_TRY(cudaGetDevice(&dev));
    DPL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t want = (a.npix + warps - 1) / warps;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 8));
    if (a.n <= 32) {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_pixel64<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_pixel64<1><<<grid, 32 * warps, smem, s>>>(a, L);
    } else {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_pixel64<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_pixel64<2><<<grid, 32 * warps, smem, s>>>(a, L);
    }
    return check_launch("k_pixel64");
}

// Dense eigensolver over the listed non-converged pixels: one-warp CTAs, a persistent
// grid of up to 8 per SM (the list length is known only on the device).
static dpl_status launch_eigh(const PixArgs& a, cudaStream_t s) {
    const EighLayout L = make_eigh_layout(a.n);
    if (a.n > kEighMaxN || L.bytes > 227 * 1024)
        return fail(DPL_ERR_UNSUPPORTED, "eigensolver: N above 64 or shared memory above the SM limit");
    int dev = 0, sms = 0, per_sm = 0;
    DPL_CUDA_TRY(cudaGetDevice(&dev));
    DPL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DPL_CUDA_TRY(cudaFuncSetAttribute(k_eigh, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.bytes));
    DPL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eigh, 32, L.bytes));
    // one resident wave: each warp strides over the listed pixels
    k_eigh<<<(unsigned)std::max(1, sms * std::max(1, per_sm)), 32, L.bytes, s>>>(a, L);
    return check_launch("k_eigh");
}

// Solve pass, then the LU pass over the pixels it lists (`fb`: a counter, then room
// for every pixel index) and, with `nc` (the same shape), the dense eigensolver over
// the pixels whose iteration missed its stopping rule.
template <int MODE>
static dpl_status launch_pixel(PixArgs& a, cudaStream_t s, int* fb = nullptr, int* nc = nullptr) {
    if (a.npix == 0) return DPL_OK;
    if (MODE == kCovOnly) return launch_pixel_pass<MODE, false>(a, s);
    if (!fb) return fail(DPL_ERR_WORKSPACE, "solver: missing fallback list");
    DPL_CUDA_TRY(cudaMemsetAsync(fb, 0, sizeof(int), s));
    a.fb_count = fb;
    a.fb_list = fb + 64;
    // non-converged pixels are listed (and solved again) only where the coherence is stored
    a.nc_count = MODE == kSolveOnly && nc ? nc : nullptr;
    a.nc_list = a.nc_count ? nc + 64 : nullptr;
    if (!a.nc_count) a.nc_flag = nullptr;
    if (a.nc_count) DPL_CUDA_TRY(cudaMemsetAsync(nc, 0, sizeof(int), s));
    dpl_status st = MODE == kSolveOnly && a.n <= 64 ? launch_solve_reg(a, s) : launch_pixel_pass<MODE, false>(a, s);
    if (st != DPL_OK) return st;
    PixArgs b = a;
    fill_pix_layout(b, a.n, 2 * a.hx + 1, true);
    b.list = a.fb_list;
    b.list_count = a.fb_count;
    st = launch_pixel_pass<MODE, true>(b, s);
    if (st != DPL_OK || !a.nc_count) return st;
    return launch_eigh(a, s);
}

// Tensor-core covariance: fills `Cg` (npix x n*n planar floats).
// Tile, pass and shared-memory plan of the tensor-core covariance.  False if the
// shape does not fit (then the plain SIMT form is used).
// Shared-memory carve of the covariance kernel for nst operand stages, sized for up to
// n SLCs, kpad region samples and npass passes (a batch carves once for all its items).
static void tc_carve(TcArgs& a, int nst, int n, int kpad, int npass, bool tf32) {
    size_t o = 0;
    auto take = [&](size_t bytes, size_t al) {
        o = align_up(o, al);
        size_t at = o;
        o += bytes;
        return (int)at;
    };
    a.nst = nst;
    a.off_stage = take((size_t)nst * (tf32 ? kTcStageBytesTf : kTcStageBytes), 1024);
    a.z_bytes = (int)align_up((size_t)kTcKC * n * sizeof(cfloat), 16);
    a.off_z = take(kTcZBuf * (size_t)a.z_bytes, 16);
    a.off_pbits = take((size_t)kTcN * (kpad / 32) * sizeof(uint32_t), 16);
    a.off_soff = take((size_t)kpad * sizeof(int), 16);
    a.off_runs = take((size_t)(kpad / kTcKC) * kTcRuns * sizeof(int2), 16);
    a.off_rows = take((size_t)npass * kTcRows * sizeof(uint32_t), 16);
    a.off_bar = take(128, 64);
    a.smem_bytes = (int)align_up(o, 128) + 1024;  // + alignment slack
}

static bool tc_configure(TcArgs& a, int n, int rows, int cols, int hy, int hx, int sy, int sx, bool tf32 = false) {
    a.n = n;
    a.rows = rows;
    a.cols = cols;
    a.hy = hy;
    a.hx = hx;
    a.sy = sy;
    a.sx = sx;
    a.out_rows = rows / sy;
    a.out_cols = cols / sx;
    const int wy = 2 * hy + 1, wx = 2 * hx + 1;
    if (wx > 64 || n < 1 || n > 64) return false;
    if ((int64_t)rows * cols * n >= (int64_t)1 << 31) return false;  // 32-bit sample offsets
    a.tiles_r = ceil_div(std::max(a.out_rows, 1), kTcTileR);
    a.tiles_c = ceil_div(std::max(a.out_cols, 1), kTcTileC);
    a.region_r = (kTcTileR - 1) * sy + wy;
    a.region_c = (kTcTileC - 1) * sx + wx;
    a.kpad = (int)(ceil_div((int64_t)a.region_r * a.region_c, kTcKC) * kTcKC);
    a.kwords = a.kpad / 32;
    const int O = n * (n - 1) / 2;
    // pass 0: the diagonal and kTcRows - n pairs; then kTcRows pairs per pass
    a.npass = 1 + ceil_div(std::max(0, O - (kTcRows - n)), kTcRows);
    // three operand stages where they fit in shared memory, else two
    for (a.nst = kTcMaxStages; a.nst >= 2; --a.nst) {
        tc_carve(a, a.nst, n, a.kpad, a.npass, tf32);
        if (a.smem_bytes <= 227 * 1024) break;
    }
    return a.nst >= 2 && a.smem_bytes <= 227 * 1024;
}

static dpl_status launch_cov_tc(int n, int rows, int cols, int hy, int hx, int sy, int sx, const cfloat* zt,
                                const uint32_t* bits, int wpr, const uint8_t* nb_u8, float* Cg, int32_t* counts,
                                int* status, cudaStream_t s, bool tf32 = false) {
    TcArgs a{};
    if (!tc_configure(a, n, rows, cols, hy, hx, sy, sx, tf32))
        return fail(DPL_ERR_UNSUPPORTED, "tensor-core covariance: unsupported shape");
    if (a.out_rows == 0 || a.out_cols == 0) return DPL_OK;
    a.zt = zt;
    a.bits = bits;
    a.wpr = wpr;
    a.nb_u8 = nb_u8;
    a.Cg = Cg;
    a.counts = counts;
    a.status = status;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int ntiles = a.tiles_r * a.tiles_c;
    const int grid = std::max(1, std::min(ntiles, sms));
    TcBatch b{};
    b.items[0] = a;
    b.nitems = 1;
    b.total = ntiles;
    if (tf32) {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_cov_tc<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          a.smem_bytes));
        k_cov_tc<true, false><<<grid, kTcThreads, a.smem_bytes, s>>>(b, nullptr);
    } else {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_cov_tc<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          a.smem_bytes));
        k_cov_tc<false, false><<<grid, kTcThreads, a.smem_bytes, s>>>(b, nullptr);
    }
    return check_launch("k_cov_tc");
}

// One work-queue launch of the covariance over the tiles of several stacks (items, each
// configured by tc_configure with its pointers set, all of one operand type).  The items
// go largest N first, and share one carve: the fewest stages any needs, the largest
// sizes.  `counter` (device int) is zeroed on the stream first.
static dpl_status launch_cov_tc_batch(std::vector<TcArgs> items, bool tf32, int* counter, cudaStream_t s) {
    if (items.empty()) return DPL_OK;
    if (items.size() > (size_t)kTcMaxItems) return fail(DPL_ERR_UNSUPPORTED, "batch: more than 16 stacks");
    std::stable_sort(items.begin(), items.end(), [](const TcArgs& x, const TcArgs& y) { return x.n > y.n; });
    int nst = kTcMaxStages, nmax = 0, kpad = 0, npass = 0;
    for (const TcArgs& t : items) {
        nst = std::min(nst, t.nst);
        nmax = std::max(nmax, t.n);
        kpad = std::max(kpad, t.kpad);
        npass = std::max(npass, t.npass);
    }
    TcArgs carve{};
    tc_carve(carve, nst, nmax, kpad, npass, tf32);
    if (carve.smem_bytes > 227 * 1024) return fail(DPL_ERR_UNSUPPORTED, "batch: covariance shared memory exceeds the SM limit");
    TcBatch b{};
    b.nitems = (int)items.size();
    int total = 0;
    for (int i = 0; i < b.nitems; ++i) {
        TcArgs t = items[i];
        t.nst = carve.nst;
        t.off_stage = carve.off_stage;
        t.z_bytes = carve.z_bytes;
        t.off_z = carve.off_z;
        t.off_pbits = carve.off_pbits;
        t.off_soff = carve.off_soff;
        t.off_runs = carve.off_runs;
        t.off_rows = carve.off_rows;
        t.off_bar = carve.off_bar;
        t.smem_bytes = carve.smem_bytes;
        t.status = items[0].status;
        b.items[i] = t;
        b.tile_start[i] = total;
        total += t.tiles_r * t.tiles_c;
    }
    b.total = total;
    if (total == 0) return DPL_OK;
    int dev = 0, sms = 0;
    DPL_CUDA_TRY(cudaGetDevice(&dev));
    DPL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DPL_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), s));
    const int grid = std::max(1, std::min(total, sms));
    if (tf32) {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_cov_tc<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          carve.smem_bytes));
        k_cov_tc<true, true><<<grid, kTcThreads, carve.smem_bytes, s>>>(b, counter);
    } else {
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_cov_tc<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          carve.smem_bytes));
        k_cov_tc<false, true><<<grid, kTcThreads, carve.smem_bytes, s>>>(b, counter);
    }
    return check_launch("k_cov_tc (batch)");
}

static int norm_ref(int ref, int n) { return ref < 0 ? n + ref : ref; }

static void set_solver_params(PixArgs& a, int use_evd, double beta, double zct, int ref_idx, double num_looks,
                              int first_real, int compute_crlb) {
    a.use_evd = use_evd;
    a.beta_on = beta > 0.0;
    a.one_minus_beta = (float)(1.0 - beta);
    a.beta = (float)beta;
    a.zct = (float)zct;
    a.ref_idx = ref_idx;
    a.compute_crlb = compute_crlb;
    a.crlb_ref = std::max(first_real - 1, 0);
    a.crlb_factor = (float)(2.0 * num_looks);
    a.beta_d = beta;
    a.zct_d = zct;
    a.crlb_factor_d = 2.0 * num_looks;
}

struct PlWorkspace {
    int* status;
    unsigned int* valid_bits;
    float* Cg;
    int* fb;
    int* nc;
    uint8_t* flags;
    float* avgmag;
    cfloat* zt;
    cfloat* V;
    float* CR;
};

static size_t pl_workspace_layout(int64_t n, int64_t rows, int64_t cols, int sy, int sx, int cov_form, char* base,
                                  PlWorkspace* w) {
    Workspace ws{base, ~size_t(0)};
    const int64_t npix = rows * cols, P = (rows / sy) * (cols / sx);
    PlWorkspace t{};
    t.status = ws.take<int>(16);
    t.valid_bits = ws.take<unsigned int>(16);
    t.Cg = cov_form == 0 || cov_form == 3 ? ws.take<float>(P * n * n) : nullptr;
    t.fb = ws.take<int>(P + 64);
    t.nc = ws.take<int>(P + 64);
    t.flags = ws.take<uint8_t>(npix);
    t.avgmag = ws.take<float>(npix);
    t.zt = ws.take<cfloat>(npix * n);
    t.V = ws.take<cfloat>(P * n);
    t.CR = ws.take<float>(P * n);
    if (w) *w = t;
    return align_up(ws.used, 256);
}

static dpl_status validate_common(int64_t n, int64_t rows, int64_t cols, int hy, int hx, int sy, int sx) {
    if (n <= 0 || rows <= 0 || cols <= 0 || hy < 0 || hx < 0 || sy <= 0 || sx <= 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "bad shape or window");
    if (n > kMaxNslc) return fail(DPL_ERR_UNSUPPORTED, "at most 64 SLCs per call are supported");
    if (2 * hx + 1 > 64) return fail(DPL_ERR_UNSUPPORTED, "window width 2*hx+1 must be <= 64");
    if (rows > INT32_MAX / 2 || cols > INT32_MAX / 2) return fail(DPL_ERR_UNSUPPORTED, "image too large");
    if (2 * hy + 1 > rows || 2 * hx + 1 > cols)
        return fail(DPL_ERR_INVALID_ARGUMENT, "half_window is larger than the SLC stack");
    return DPL_OK;
}

}  // namespace dpl

using namespace dpl;

extern "C" size_t dpl_phase_link_workspace_size(const dpl_pl_params* p) {
    if (!p) return 0;
    return pl_workspace_layout(p->nslc, p->rows, p->cols, std::max(1, p->sy), std::max(1, p->sx), p->cov_form, nullptr,
                               nullptr);
}

// Per-call state between the pipeline's stages (pl_begin, then the covariance, then
// pl_finish), so that a batch can run one covariance launch for several calls.
struct PlState {
    dpl_pl_params P;
    const dpl_pl_inputs* in;
    const dpl_pl_outputs* out;
    PlWorkspace w;
    PixArgs a;
    int n, ref, out_rows, out_cols;
    int64_t Pout;
    bool tc_fits, tf32;
    TcArgs tc;  // configured, pointers set, when tc_fits
};

// Validation, status words, k_prep and the per-pixel arguments of one call.
static dpl_status pl_begin(const dpl_pl_params* prm, const dpl_pl_inputs* in, const dpl_pl_outputs* out,
                           void* workspace, size_t workspace_bytes, cudaStream_t s, PlState& S) {
    if (!prm || !in || !out) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link: null argument");
    const dpl_pl_params& P = *prm;
    dpl_status st = validate_common(P.nslc, P.rows, P.cols, P.hy, P.hx, P.sy, P.sx);
    if (st != DPL_OK) return st;
    if (!in->slc || !out->cpx_phase || !out->temp_coh || !out->eigenvalues || !out->estimator || !out->crlb_std_dev)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link: null array");
    if (misaligned_c8(in->slc) || misaligned_c8(out->cpx_phase))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link: complex arrays must be 8-byte aligned");
    if (reinterpret_cast<uintptr_t>(workspace) & 15u)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link: workspace must be 16-byte aligned");
    const int n = (int)P.nslc;
    const int ref = norm_ref(P.reference_idx, n);
    if (ref < 0 || ref >= n) return fail(DPL_ERR_INVALID_ARGUMENT, "reference_idx out of range");
    if (P.cov_form < 0 || P.cov_form > 3) return fail(DPL_ERR_INVALID_ARGUMENT, "cov_form must be 0, 1, 2 or 3");
    if (P.nonconverged_mode < 0 || P.nonconverged_mode > 1)
        return fail(DPL_ERR_INVALID_ARGUMENT, "nonconverged_mode must be 0 or 1");
    if (workspace_bytes < dpl_phase_link_workspace_size(prm)) return fail(DPL_ERR_WORKSPACE, "workspace too small");
    S.P = P;
    S.in = in;
    S.out = out;
    S.n = n;
    S.ref = ref;
    PlWorkspace& w = S.w;
    pl_workspace_layout(P.nslc, P.rows, P.cols, P.sy, P.sx, P.cov_form, (char*)workspace, &w);
    const int64_t npix = P.rows * P.cols;
    S.out_rows = (int)(P.rows / P.sy);
    S.out_cols = (int)(P.cols / P.sx);
    S.Pout = (int64_t)S.out_rows * S.out_cols;
    DPL_CUDA_TRY(cudaMemsetAsync(w.status, 0, 64, s));
    DPL_CUDA_TRY(cudaMemsetAsync(w.valid_bits, 0, 64, s));
    {
        size_t smem = (size_t)kPrepPix * (n + 1) * sizeof(cfloat);
        DPL_CUDA_TRY(cudaFuncSetAttribute(k_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_prep<<<ceil_div(npix, kPrepPix), 256, smem, s>>>(
            reinterpret_cast<const cfloat*>(in->slc), n, npix, in->nodata_mask, in->ps_mask, P.mask_input_ps, 1, w.flags,
            w.zt, in->avg_mag ? nullptr : w.avgmag, w.valid_bits);
        st = check_launch("k_prep");
        if (st != DPL_OK) return st;
    }
    S.tc_fits = false;
    S.tf32 = P.cov_form == 3;
    if (S.Pout == 0) return DPL_OK;
    PixArgs& a = S.a;
    a = PixArgs{};
    fill_pix_layout(a, n, 2 * P.hx + 1);
    a.rows = (int)P.rows;
    a.cols = (int)P.cols;
    a.hy = P.hy;
    a.hx = P.hx;
    a.sy = P.sy;
    a.sx = P.sx;
    a.out_rows = S.out_rows;
    a.out_cols = S.out_cols;
    a.npix = S.Pout;
    a.zt = w.zt;
    a.nb_u8 = in->neighbors;
    set_solver_params(a, P.use_evd, P.beta, P.zero_correlation_threshold, ref, std::sqrt((double)P.hy * P.hx),
                      P.first_real_slc_idx, P.compute_crlb);
    a.baseline_lag = P.baseline_lag > 0 ? P.baseline_lag : 0;
    a.slots = P.solver_slots;
    a.lanes = P.solver_lanes;
    a.nc_flag = P.nonconverged_mode == 0 ? out->nonconverged : nullptr;
    a.eigh = P.nonconverged_mode == 0;
    if (out->nonconverged) DPL_CUDA_TRY(cudaMemsetAsync(out->nonconverged, 0, (size_t)S.Pout, s));
    a.vout = w.V;
    a.eig = out->eigenvalues;
    a.est = out->estimator;
    a.crlb = w.CR;
    a.tcoh = out->temp_coh;
    a.closure = n > 2 ? out->closure_phases : nullptr;
    a.counts = in->neighbors ? out->shp_counts : nullptr;
    S.tc = TcArgs{};
    S.tc_fits = (P.cov_form == 0 || S.tf32) &&
                tc_configure(S.tc, n, (int)P.rows, (int)P.cols, P.hy, P.hx, P.sy, P.sx, S.tf32);
    if (S.tc_fits) {
        S.tc.zt = w.zt;
        S.tc.bits = nullptr;
        S.tc.wpr = 0;
        S.tc.nb_u8 = in->neighbors;
        S.tc.Cg = w.Cg;
        S.tc.counts = a.counts;
        S.tc.status = w.status;
    }
    return DPL_OK;
}

// The covariance (unless `cov_done`: a batch launched it), the solver and the post pass
// of one call begun by pl_begin.
static dpl_status pl_finish(PlState& S, cudaStream_t s, bool cov_done) {
    if (S.Pout == 0) return DPL_OK;
    const dpl_pl_params& P = S.P;
    PlWorkspace& w = S.w;
    PixArgs& a = S.a;
    const int n = S.n;
    dpl_status st;
    if (P.cov_form == 2) {
        // FP64 form: covariance and solver in double precision
        st = timed(s, 0, [&] { return launch_pixel64(a, s); });
    } else if (S.tc_fits) {
        // chosen form: tensor-core covariance, then the solver on the planar matrices
        if (!cov_done) {
            st = timed(s, 0, [&] {
                return launch_cov_tc(n, (int)P.rows, (int)P.cols, P.hy, P.hx, P.sy, P.sx, w.zt, nullptr, 0,
                                     S.in->neighbors, w.Cg, a.counts, w.status, s, S.tf32);
            });
            if (st != DPL_OK) return st;
        }
        a.Cplanar = w.Cg;
        st = timed(s, 1, [&] {
            return launch_pixel<kSolveOnly>(a, s, w.fb, P.nonconverged_mode == 0 ? w.nc : nullptr);
        });
    } else {
        // plain form (or a window too large for the tensor-core tiles): SIMT covariance
        // fused with the solver
        st = timed(s, 0, [&] { return launch_pixel<kFused>(a, s, w.fb); });
    }
    if (st != DPL_OK) return st;

    PostArgs q{};
    q.n = n;
    q.rows = (int)P.rows;
    q.cols = (int)P.cols;
    q.sy = P.sy;
    q.sx = P.sx;
    q.out_rows = S.out_rows;
    q.out_cols = S.out_cols;
    q.slc = reinterpret_cast<const cfloat*>(S.in->slc);
    q.flags = w.flags;
    q.mag = S.in->avg_mag ? S.in->avg_mag : w.avgmag;
    q.V = w.V;
    q.CR = w.CR;
    q.use_max_ps = P.use_max_ps;
    q.use_slc_amp = P.use_slc_amp;
    q.ref_idx = S.ref;
    q.cpx = reinterpret_cast<cfloat*>(S.out->cpx_phase);
    q.tcoh = S.out->temp_coh;
    q.crlb = S.out->crlb_std_dev;
    q.status = w.status;
    k_post<<<ceil_div(S.Pout, 256), 256, 0, s>>>(q);
    return check_launch("k_post");
}

// Enqueues the whole pipeline on `stream` without synchronising.
static dpl_status pl_enqueue(const dpl_pl_params* prm, const dpl_pl_inputs* in, const dpl_pl_outputs* out,
                             void* workspace, size_t workspace_bytes, dpl_stream_t stream) {
    cudaStream_t s = (cudaStream_t)stream;
    PlState S;
    dpl_status st = pl_begin(prm, in, out, workspace, workspace_bytes, s, S);
    if (st != DPL_OK) return st;
    return pl_finish(S, s, false);
}

// Maps the status words the pipeline left (status, then the 64 per-SLC "has a finite
// sample" bits) to the reference's errors: an all-NaN SLC (its message), an undefined
// PS brightness, a device timeout.
static dpl_status pl_decode(int n, const int* status, const unsigned int* valid) {
    const unsigned long long vb = valid[0] | ((unsigned long long)valid[1] << 32);
    std::vector<int> bad;
    for (int t = 0; t < n; ++t)
        if (!((vb >> t) & 1ull)) bad.push_back(t);
    if (!bad.empty()) {
        std::ostringstream os;
        os << "slc_stack[[";
        for (size_t i = 0; i < bad.size(); ++i) os << (i ? " " : "") << bad[i];
        os << "]] out of " << n << " are all NaNs.";
        return fail(DPL_ERR_ALL_NAN_SLC, os.str());
    }
    if (status[0] == DPL_ERR_INVALID_ARGUMENT)
        return fail(DPL_ERR_INVALID_ARGUMENT, "a PS look window has no finite brightness (avg_mag is NaN at its PS pixels)");
    if (status[0] != 0) return fail((dpl_status)status[0], "device-side error");
    return DPL_OK;
}

// Waits for `stream`, then reports what the enqueued pipeline left in the workspace.
static dpl_status pl_check(int n, const PlWorkspace& w, cudaStream_t s) {
    int host_status[2] = {0, 0};
    unsigned int host_valid[2] = {0, 0};
    DPL_CUDA_TRY(cudaMemcpyAsync(host_status, w.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    DPL_CUDA_TRY(cudaMemcpyAsync(host_valid, w.valid_bits, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    DPL_CUDA_TRY(cudaStreamSynchronize(s));
    return pl_decode(n, host_status, host_valid);
}

extern "C" dpl_status dpl_phase_link(const dpl_pl_params* prm, const dpl_pl_inputs* in, const dpl_pl_outputs* out,
                                     void* workspace, size_t workspace_bytes, dpl_stream_t stream) {
    dpl_status st = pl_enqueue(prm, in, out, workspace, workspace_bytes, stream);
    if (st != DPL_OK) return st;
    return dpl_phase_link_status(prm, workspace, workspace_bytes, stream);
}

extern "C" dpl_status dpl_phase_link_async(const dpl_pl_params* prm, const dpl_pl_inputs* in,
                                           const dpl_pl_outputs* out, void* workspace, size_t workspace_bytes,
                                           dpl_stream_t stream) {
    return pl_enqueue(prm, in, out, workspace, workspace_bytes, stream);
}

extern "C" dpl_status dpl_phase_link_status(const dpl_pl_params* prm, void* workspace, size_t workspace_bytes,
                                            dpl_stream_t stream) {
    if (!prm || !workspace) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link_status: null argument");
    if (workspace_bytes < dpl_phase_link_workspace_size(prm)) return fail(DPL_ERR_WORKSPACE, "workspace too small");
    PlWorkspace w;
    pl_workspace_layout(prm->nslc, prm->rows, prm->cols, std::max(1, prm->sy), std::max(1, prm->sx), prm->cov_form,
                        (char*)workspace, &w);
    return pl_check((int)prm->nslc, w, (cudaStream_t)stream);
}

extern "C" dpl_status dpl_phase_link_status_copy(const dpl_pl_params* prm, void* workspace, size_t workspace_bytes,
                                                 void* words, dpl_stream_t stream) {
    if (!prm || !workspace || !words) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link_status_copy: null argument");
    if (workspace_bytes < dpl_phase_link_workspace_size(prm)) return fail(DPL_ERR_WORKSPACE, "workspace too small");
    PlWorkspace w;
    pl_workspace_layout(prm->nslc, prm->rows, prm->cols, std::max(1, prm->sy), std::max(1, prm->sx), prm->cov_form,
                        (char*)workspace, &w);
    cudaStream_t s = (cudaStream_t)stream;
    int* dst = static_cast<int*>(words);
    DPL_CUDA_TRY(cudaMemcpyAsync(dst, w.status, sizeof(int), cudaMemcpyDefault, s));
    DPL_CUDA_TRY(cudaMemcpyAsync(dst + 1, w.valid_bits, 2 * sizeof(unsigned int), cudaMemcpyDefault, s));
    return DPL_OK;
}

extern "C" dpl_status dpl_phase_link_status_words(int64_t nslc, const void* words) {
    if (!words) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link_status_words: null argument");
    const int* w = static_cast<const int*>(words);
    return pl_decode((int)nslc, w, reinterpret_cast<const unsigned int*>(w + 1));
}

// ---------------------------------------------------------------------------------
// batches: several stacks (ministacks of uneven N) with one work-queue covariance launch
// ---------------------------------------------------------------------------------
static size_t batch_item_offset(const dpl_pl_params* prms, int i) {
    size_t o = 256;  // two work-queue counters
    for (int k = 0; k < i; ++k) o += align_up(dpl_phase_link_workspace_size(&prms[k]), 256);
    return o;
}

extern "C" size_t dpl_phase_link_batch_workspace_size(const dpl_pl_params* prms, int count) {
    if (!prms || count < 0) return 0;
    return batch_item_offset(prms, count);
}

extern "C" dpl_status dpl_phase_link_batch(const dpl_pl_params* prms, const dpl_pl_inputs* ins,
                                           const dpl_pl_outputs* outs, int count, void* workspace,
                                           size_t workspace_bytes, dpl_stream_t stream) {
    if (!prms || !ins || !outs || !workspace || count < 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link_batch: null argument");
    if (count > kTcMaxItems) return fail(DPL_ERR_UNSUPPORTED, "dpl_phase_link_batch: at most 16 stacks per batch");
    if (reinterpret_cast<uintptr_t>(workspace) & 255u)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link_batch: workspace must be 256-byte aligned");
    if (workspace_bytes < dpl_phase_link_batch_workspace_size(prms, count))
        return fail(DPL_ERR_WORKSPACE, "dpl_phase_link_batch: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    char* base = static_cast<char*>(workspace);
    std::vector<PlState> S(count);
    dpl_status st;
    for (int i = 0; i < count; ++i) {
        const size_t off = batch_item_offset(prms, i);
        st = pl_begin(&prms[i], &ins[i], &outs[i], base + off, dpl_phase_link_workspace_size(&prms[i]), s, S[i]);
        if (st != DPL_OK) return st;
    }
    // the tensor-core covariance of every stack that takes it: one work-queue launch per
    // operand type
    int* counters = reinterpret_cast<int*>(base);
    for (int kind = 0; kind < 2; ++kind) {
        std::vector<TcArgs> items;
        for (int i = 0; i < count; ++i)
            if (S[i].tc_fits && S[i].tf32 == (kind == 1)) items.push_back(S[i].tc);
        if (items.empty()) continue;
        st = timed(s, 0, [&] { return launch_cov_tc_batch(items, kind == 1, counters + kind, s); });
        if (st != DPL_OK) return st;
    }
    for (int i = 0; i < count; ++i) {
        st = pl_finish(S[i], s, S[i].tc_fits);
        if (st != DPL_OK) return st;
    }
    return DPL_OK;
}

extern "C" dpl_status dpl_phase_link_batch_status(const dpl_pl_params* prms, int count, void* workspace,
                                                  size_t workspace_bytes, dpl_stream_t stream) {
    if (!prms || !workspace || count < 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_phase_link_batch_status: null argument");
    if (workspace_bytes < dpl_phase_link_batch_workspace_size(prms, count))
        return fail(DPL_ERR_WORKSPACE, "dpl_phase_link_batch_status: workspace too small");
    for (int i = 0; i < count; ++i) {
        const size_t off = batch_item_offset(prms, i);
        dpl_status st = dpl_phase_link_status(&prms[i], static_cast<char*>(workspace) + off,
                                              dpl_phase_link_workspace_size(&prms[i]), stream);
        if (st != DPL_OK) return st;
    }
    return DPL_OK;
}

extern "C" size_t dpl_covariance_workspace_size(int64_t nslc, int64_t rows, int64_t cols) {
    Workspace ws{nullptr, ~size_t(0)};
    ws.take<int>(16);
    ws.take<unsigned int>(16);
    ws.take<uint8_t>(rows * cols);
    ws.take<cfloat>(rows * cols * nslc);
    ws.take<float>(rows * cols * nslc * nslc);  // planar matrices of the tensor-core form (strides >= 1)
    return align_up(ws.used, 256);
}

extern "C" dpl_status dpl_covariance(const float* slc, int64_t nslc, int64_t rows, int64_t cols, int hy, int hx,
                                     int sy, int sx, const uint8_t* neighbors, int cov_form, float* C,
                                     void* workspace, size_t workspace_bytes, dpl_stream_t stream) {
    dpl_status st = validate_common(nslc, rows, cols, hy, hx, sy, sx);
    if (st != DPL_OK) return st;
    if (cov_form != 0 && cov_form != 1 && cov_form != 3)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_covariance: cov_form must be 0, 1 or 3 (2, fp64, is a phase-linking form)");
    if (!slc || !C || !workspace) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_covariance: null pointer");
    if (misaligned_c8(slc) || misaligned_c8(C) || (reinterpret_cast<uintptr_t>(workspace) & 15u))
        return fail(DPL_ERR_INVALID_ARGUMENT,
                    "dpl_covariance: complex arrays must be 8-byte and the workspace 16-byte aligned");
    if (workspace_bytes < dpl_covariance_workspace_size(nslc, rows, cols))
        return fail(DPL_ERR_WORKSPACE, "dpl_covariance: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)nslc;
    Workspace ws{(char*)workspace, workspace_bytes};
    int* status = ws.take<int>(16);
    unsigned int* vb = ws.take<unsigned int>(16);
    uint8_t* flags = ws.take<uint8_t>(rows * cols);
    cfloat* zt = ws.take<cfloat>(rows * cols * nslc);
    float* Cg = ws.take<float>(rows * cols * nslc * nslc);
    const int64_t npix = rows * cols;
    size_t smem = (size_t)kPrepPix * (n + 1) * sizeof(cfloat);
    DPL_CUDA_TRY(cudaFuncSetAttribute(k_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_prep<<<ceil_div(npix, kPrepPix), 256, smem, s>>>(reinterpret_cast<const cfloat*>(slc), n, npix, nullptr, nullptr,
                                                       0, 0, flags, zt, nullptr, vb);
    st = check_launch("k_prep");
    if (st != DPL_OK) return st;
    PixArgs a{};
    fill_pix_layout(a, n, 2 * hx + 1);
    a.rows = (int)rows;
    a.cols = (int)cols;
    a.hy = hy;
    a.hx = hx;
    a.sy = sy;
    a.sx = sx;
    a.out_rows = (int)(rows / sy);
    a.out_cols = (int)(cols / sx);
    a.npix = (int64_t)a.out_rows * a.out_cols;
    a.zt = zt;
    a.nb_u8 = neighbors;
    a.Cout = reinterpret_cast<cfloat*>(C);
    TcArgs tcfit{};
    if (cov_form == 1 || !tc_configure(tcfit, n, (int)rows, (int)cols, hy, hx, sy, sx, cov_form == 3))
        return launch_pixel<kCovOnly>(a, s);
    DPL_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
    st = launch_cov_tc(n, (int)rows, (int)cols, hy, hx, sy, sx, zt, nullptr, 0, neighbors, Cg, nullptr, status, s,
                       cov_form == 3);
    if (st != DPL_OK) return st;
    const int64_t tot = a.npix * n * n;
    k_unpack_planar<<<ceil_div(tot, 256), 256, 0, s>>>(Cg, n, a.npix, reinterpret_cast<cfloat*>(C));
    return check_launch("k_unpack_planar");
}

extern "C" size_t dpl_process_coherence_workspace_size(int64_t npix) {
    return align_up((size_t)(std::max<int64_t>(npix, 0) + 64) * sizeof(int), 256);
}

extern "C" dpl_status dpl_process_coherence(const float* C, int64_t npix, int nslc, int use_evd, double beta,
                                            double zero_correlation_threshold, int reference_idx, double num_looks,
                                            int first_real_slc_idx, int compute_crlb, float* eig_vecs,
                                            float* eig_vals, uint8_t* estimator, float* crlb_std_dev,
                                            float* temp_coh, float* closure_phases, void* workspace,
                                            size_t workspace_bytes, dpl_stream_t stream) {
    if (npix < 0 || nslc <= 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence: bad shape");
    if (nslc > kMaxNslc) return fail(DPL_ERR_UNSUPPORTED, "at most 64 SLCs per call are supported");
    if (npix == 0) return DPL_OK;
    if (!C || !eig_vecs || !eig_vals || !estimator || !crlb_std_dev || !temp_coh)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence: null pointer");
    if (misaligned_c8(C) || misaligned_c8(eig_vecs))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence: complex arrays must be 8-byte aligned");
    const int ref = norm_ref(reference_idx, nslc);
    if (ref < 0 || ref >= nslc) return fail(DPL_ERR_INVALID_ARGUMENT, "reference_idx out of range");
    PixArgs a{};
    fill_pix_layout(a, nslc, 1);
    a.npix = npix;
    a.Cin = reinterpret_cast<const cfloat*>(C);
    set_solver_params(a, use_evd, beta, zero_correlation_threshold, ref, num_looks, first_real_slc_idx, compute_crlb);
    a.vout = reinterpret_cast<cfloat*>(eig_vecs);
    a.eig = eig_vals;
    a.est = estimator;
    a.crlb = crlb_std_dev;
    a.tcoh = temp_coh;
    a.closure = nslc > 2 ? closure_phases : nullptr;
    if (!workspace || workspace_bytes < dpl_process_coherence_workspace_size(npix))
        return fail(DPL_ERR_WORKSPACE, "dpl_process_coherence: workspace too small");
    return launch_pixel<kSolveOnly>(a, (cudaStream_t)stream, reinterpret_cast<int*>(workspace));
}

extern "C" dpl_status dpl_process_coherence_warm(const float* C, int64_t npix, int nslc, int use_evd, double beta,
                                                 double zero_correlation_threshold, int reference_idx,
                                                 double num_looks, int first_real_slc_idx, int compute_crlb,
                                                 const float* vstart, float* eig_vecs, float* eig_vals,
                                                 uint8_t* estimator, float* crlb_std_dev, float* temp_coh,
                                                 float* closure_phases, int16_t* iterations, void* workspace,
                                                 size_t workspace_bytes, dpl_stream_t stream) {
    if (npix < 0 || nslc <= 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence_warm: bad shape");
    if (nslc > kMaxNslc) return fail(DPL_ERR_UNSUPPORTED, "at most 64 SLCs per call are supported");
    if (npix == 0) return DPL_OK;
    if (!C || !eig_vecs || !eig_vals || !estimator || !crlb_std_dev || !temp_coh)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence_warm: null pointer");
    if (misaligned_c8(C) || misaligned_c8(eig_vecs))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence_warm: complex arrays must be 8-byte aligned");
    const int ref = norm_ref(reference_idx, nslc);
    if (ref < 0 || ref >= nslc) return fail(DPL_ERR_INVALID_ARGUMENT, "reference_idx out of range");
    if (!workspace || workspace_bytes < dpl_process_coherence_workspace_size(npix))
        return fail(DPL_ERR_WORKSPACE, "dpl_process_coherence_warm: workspace too small");
    if (vstart && misaligned_c8(vstart))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence_warm: complex arrays must be 8-byte aligned");
    PixArgs a{};
    fill_pix_layout(a, nslc, 1);
    a.npix = npix;
    a.Cin = reinterpret_cast<const cfloat*>(C);
    set_solver_params(a, use_evd, beta, zero_correlation_threshold, ref, num_looks, first_real_slc_idx, compute_crlb);
    a.vstart = reinterpret_cast<const cfloat*>(vstart);
    a.iters = iterations;
    a.vout = reinterpret_cast<cfloat*>(eig_vecs);
    a.eig = eig_vals;
    a.est = estimator;
    a.crlb = crlb_std_dev;
    a.tcoh = temp_coh;
    a.closure = nslc > 2 ? closure_phases : nullptr;
    return launch_pixel<kSolveOnly>(a, (cudaStream_t)stream, reinterpret_cast<int*>(workspace));
}

// Scratch of dpl_process_coherence_noalloc: the fallback-pixel counter (word 0) and
// list (from word 64) of launch_pixel, sized for kNoAllocMaxPix pixels (4 MiB).  One
// copy per device, shared by every call on that device.
constexpr int64_t kNoAllocMaxPix = int64_t(1) << 20;
static __device__ __align__(256) int g_noalloc_scratch[64 + kNoAllocMaxPix];

static std::mutex g_noalloc_mu;
static int* g_noalloc_ptr[64];  // per device ordinal, resolved on the first call there

extern "C" int64_t dpl_process_coherence_noalloc_max_pixels(void) { return kNoAllocMaxPix; }

extern "C" dpl_status dpl_process_coherence_noalloc(const float* C, int64_t npix, int nslc, int use_evd,
                                                    double beta, double zero_correlation_threshold,
                                                    int reference_idx, double num_looks, int first_real_slc_idx,
                                                    int compute_crlb, float* eig_vecs, float* eig_vals,
                                                    uint8_t* estimator, float* crlb_std_dev, float* temp_coh,
                                                    float* closure_phases, dpl_stream_t stream) {
    if (npix < 0 || nslc <= 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence_noalloc: bad shape");
    if (npix > kNoAllocMaxPix) {
        char msg[160];
        snprintf(msg, sizeof msg,
                 "dpl_process_coherence_noalloc: npix=%lld exceeds the static scratch limit of %lld pixels",
                 (long long)npix, (long long)kNoAllocMaxPix);
        return fail(DPL_ERR_UNSUPPORTED, msg);
    }
    if (nslc > kMaxNslc) return fail(DPL_ERR_UNSUPPORTED, "at most 64 SLCs per call are supported");
    if (npix == 0) return DPL_OK;
    if (!C || !eig_vecs || !eig_vals || !estimator || !crlb_std_dev || !temp_coh)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence_noalloc: null pointer");
    if (misaligned_c8(C) || misaligned_c8(eig_vecs))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_process_coherence_noalloc: complex arrays must be 8-byte aligned");
    const int ref = norm_ref(reference_idx, nslc);
    if (ref < 0 || ref >= nslc) return fail(DPL_ERR_INVALID_ARGUMENT, "reference_idx out of range");
    int dev = 0;
    DPL_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(DPL_ERR_UNSUPPORTED, "dpl_process_coherence_noalloc: device ordinal >= 64");
    int* scratch = nullptr;
    {
        // set-up on the first call on this device (the current one): the symbol's address
        std::lock_guard<std::mutex> g(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            DPL_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            g_noalloc_ptr[dev] = static_cast<int*>(p);
        }
        scratch = g_noalloc_ptr[dev];
    }
    PixArgs a{};
    fill_pix_layout(a, nslc, 1);
    a.npix = npix;
    a.Cin = reinterpret_cast<const cfloat*>(C);
    set_solver_params(a, use_evd, beta, zero_correlation_threshold, ref, num_looks, first_real_slc_idx, compute_crlb);
    a.vout = reinterpret_cast<cfloat*>(eig_vecs);
    a.eig = eig_vals;
    a.est = estimator;
    a.crlb = crlb_std_dev;
    a.tcoh = temp_coh;
    a.closure = nslc > 2 ? closure_phases : nullptr;
    // launch_pixel zeroes the counter on the stream before the solve; the list needs no clearing
    return launch_pixel<kSolveOnly>(a, (cudaStream_t)stream, scratch);
}

extern "C" dpl_status dpl_kernel_timing(int enable, double* total_ms, int64_t* launches) {
    std::lock_guard<std::mutex> g(g_timer.mu);
    for (int slot = 0; slot < 2; ++slot) {
        double tot = 0.0;
        int64_t cnt = 0;
        for (auto& pr : g_timer.ev[slot]) {
            float ms = 0.f;
            if (cudaEventSynchronize(pr.second) == cudaSuccess &&
                cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) {
                tot += ms;
                ++cnt;
            }
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
        g_timer.ev[slot].clear();
        if (total_ms) total_ms[slot] = tot;
        if (launches) launches[slot] = cnt;
    }
    g_timer.on = enable != 0;
    return DPL_OK;
}
