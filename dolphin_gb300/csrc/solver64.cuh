// FP64 form of the per-pixel pipeline: covariance and solver in double precision.
//
// The same steps as the FP32 SIMT form (covariance.py:110-170, _core.py:379-534,
// _eigenvalues.py:25-205, crlb.py:132-189, metrics.py:10-97), one warp per pixel with
// the matrices in the warp's shared memory, every quantity in double:
//   covariance  sums of z_i conj(z_j) over the window's SHP samples, normalised by
//               sqrt(amp_i amp_j) where that root exceeds 1e-6
//   |Gamma|     (+ beta I, zero threshold) + 1e-6 I, inverted by Gauss-Jordan (a
//               non-positive pivot is the reference's Cholesky failure: EVD fallback)
//   EMI         LU with partial pivoting of Gamma^-1 o C - 0.99 I (the reference's
//               algorithm, for every pixel) and inverse iteration, <= 49 steps, stop
//               at |v_new - v| <= 1e-5; lambda = v^H (Gamma^-1 o C) v
//   EVD         power iteration on C o |C|
//   CRLB        FIM = 2L (Gamma o Gamma^-1 - I), row/column `ref` -> identity,
//               + 1e-6 I, Gauss-Jordan; sigma = sqrt(diag)
//   then referencing, temporal coherence and closure phases; the outputs are written
//   in float32 like every other form.
// It is the double-precision reference of the library (the arithmetic of a float64
// run of the reference's algorithm) and the FP64 variant of the precision study;
// GB300's FP64 rate makes it a reference form, not a production one.
#pragma once

namespace dpl {

struct cdbl {
    double re, im;
};
__device__ __forceinline__ cdbl dmk(double r, double i) { return cdbl{r, i}; }
__device__ __forceinline__ cdbl dadd(cdbl a, cdbl b) { return dmk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cdbl dsub(cdbl a, cdbl b) { return dmk(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ cdbl dmul(cdbl a, cdbl b) { return dmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ cdbl dmulc(cdbl a, cdbl b) { return dmk(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im); }
__device__ __forceinline__ cdbl dconj(cdbl a) { return dmk(a.re, -a.im); }
__device__ __forceinline__ cdbl dscale(cdbl a, double s) { return dmk(a.re * s, a.im * s); }
__device__ __forceinline__ double dabs2(cdbl a) { return a.re * a.re + a.im * a.im; }
__device__ __forceinline__ cdbl ddiv(cdbl a, cdbl b) {
    const double d = b.re * b.re + b.im * b.im;
    return dmk((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
__device__ __forceinline__ bool disnan(cdbl a) { return isnan(a.re) || isnan(a.im); }
__device__ __forceinline__ cdbl dshfl(cdbl a, int src) {
    return dmk(__shfl_sync(0xffffffffu, a.re, src), __shfl_sync(0xffffffffu, a.im, src));
}
__device__ __forceinline__ double dwarp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ cdbl dget(const cdbl* C, int i, int j) { return j <= i ? C[pk(i, j)] : dconj(C[pk(j, i)]); }
__device__ __forceinline__ cdbl dphasor(cdbl c) {
    const double m2 = dabs2(c);
    if (m2 == 0.0) return dmk(signbit(c.re) ? -1.0 : 1.0, 0.0);
    if (!(m2 <= INFINITY)) return dmk(nan(""), nan(""));
    const double r = 1.0 / sqrt(m2);
    return dmk(c.re * r, c.im * r);
}

struct Pix64Layout {
    int ldg;
    size_t off_C, off_G, off_A, off_V, off_v, off_piv, bytes;
};

inline Pix64Layout make_layout64(int n, int stg) {
    Pix64Layout L{};
    L.ldg = n | 1;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align_up(o + bytes, 16);
        return at;
    };
    L.off_C = take((size_t)n * (n + 1) / 2 * sizeof(cdbl));
    L.off_G = take((size_t)n * L.ldg * sizeof(double));
    L.off_A = take(std::max((size_t)n * n * sizeof(cdbl), (size_t)stg * sizeof(cfloat)));
    L.off_V = take((size_t)n * n * sizeof(cdbl));
    L.off_v = take(64 * sizeof(cdbl));
    L.off_piv = take(128 * sizeof(int));
    L.bytes = align_up(o, 128);
    return L;
}

template <int NB>
__device__ __forceinline__ cdbl d_bcast(const cdbl (&x)[NB], int k) {
    cdbl r = dshfl(x[0], k & 31);
    if (NB > 1) {
        const cdbl r1 = dshfl(x[NB - 1], k & 31);
        if (k >= 32) r = r1;
    }
    return r;
}
template <int NB>
__device__ __forceinline__ double d_norm2(const cdbl (&x)[NB]) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < NB; ++q) s += dabs2(x[q]);
    return dwarp_sum(s);
}

// covariance of output pixel p into packed C (double); `stg` stages one window row
template <int NB>
__device__ void cov64(const PixArgs& a, int64_t p, cdbl* C, cfloat* stg, double* amp, int lane, int* count_out) {
    const int n = a.n, wy = 2 * a.hy + 1, wx = 2 * a.hx + 1, np = a.np;
    const int out_r = (int)(p / a.out_cols), out_c = (int)(p - (int64_t)out_r * a.out_cols);
    const int in_r = a.sy / 2 + out_r * a.sy, in_c = a.sx / 2 + out_c * a.sx;
    const int r0 = clamp_start_i(in_r, a.hy, wy, a.rows), c0 = clamp_start_i(in_c, a.hx, wx, a.cols);
    int count = 0;
    for (int rb = 0; rb < NB; ++rb) {
        for (int cb = rb; cb < NB; ++cb) {
            double are[32], aim[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) are[j] = aim[j] = 0.0;
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
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const cfloat zj = s[cb * 32 + j];
                        are[j] += (double)zi.re * zj.re + (double)zi.im * zj.im;
                        aim[j] += (double)zi.im * zj.re - (double)zi.re * zj.im;
                    }
                }
            }
            const int row = rb * 32 + lane;
            if (row < n) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int col = cb * 32 + j;
                    if (col <= row) C[pk(row, col)] = dmk(are[j], aim[j]);
                    else if (rb != cb && col < n) C[pk(col, row)] = dmk(are[j], -aim[j]);
                }
            }
        }
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) amp[i] = C[pk(i, i)].re;
    __syncwarp();
    for (int i = 0; i < n; ++i) {
        const double ai = amp[i];
        for (int j = lane; j <= i; j += 32) {
            const double s = sqrt(ai * amp[j]);
            const cdbl c = C[pk(i, j)];
            C[pk(i, j)] = s > 1e-6 ? dmk(c.re / s, c.im / s) : dmk(0.0, 0.0);
        }
    }
    __syncwarp();
    if (count_out) *count_out = count;
}

// in-place inverse of a symmetric positive definite matrix (false on a non-positive pivot)
template <int NB>
__device__ bool gj64(double* A, int n, int ld, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        const double piv = A[k * ld + k];
        if (!(piv > 0.0)) return false;
        const double inv = 1.0 / piv;
        double rk[NB], rm[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int j = lane + 32 * q;
            rk[q] = j < n ? (j == k ? inv : A[k * ld + j] * inv) : 0.0;
            rm[q] = j == k ? 0.0 : rk[q];
        }
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            const double f = A[i * ld + k];
#pragma unroll
            for (int q = 0; q < NB; ++q)
                if (lane + 32 * q < n) A[i * ld + lane + 32 * q] -= f * rm[q];
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i < n && i != k) A[i * ld + k] = -A[i * ld + k] * inv;
            if (i < n) A[k * ld + i] = rk[q];
        }
    }
    __syncwarp();
    return true;
}

// LU with partial pivoting (first maximum of |re| + |im|) on a full n x n matrix
__device__ void lu64(cdbl* A, int n, int* piv, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        double best = -1.0;
        int bi = n;
        for (int i = k + lane; i < n; i += 32) {
            const cdbl x = A[i * n + k];
            const double v = fabs(x.re) + fabs(x.im);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (bi >= n) bi = k;
        if (lane == 0) piv[k] = bi;
        if (bi != k)
            for (int j = lane; j < n; j += 32) {
                const cdbl t = A[k * n + j];
                A[k * n + j] = A[bi * n + j];
                A[bi * n + j] = t;
            }
        __syncwarp();
        const cdbl pv = A[k * n + k];
        if (pv.re != 0.0 || pv.im != 0.0) {
            const cdbl r = ddiv(dmk(1.0, 0.0), pv);
            for (int i = k + 1 + lane; i < n; i += 32) A[i * n + k] = dmul(A[i * n + k], r);
        }
        __syncwarp();
        for (int i = k + 1; i < n; ++i) {
            const cdbl lik = A[i * n + k];
            for (int j = k + 1 + lane; j < n; j += 32) A[i * n + j] = dsub(A[i * n + j], dmul(lik, A[k * n + j]));
        }
    }
    __syncwarp();
}

// x <- (LU)^{-1} P x; src[i] is the original row that pivoting moved to row i
template <int NB>
__device__ void lusolve64(const cdbl* A, int n, const int* src, cdbl (&x)[NB], int lane) {
    cdbl w[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        const int s = i < n ? src[i] : 0;
        const cdbl t0 = dshfl(x[0], s & 31);
        const cdbl t1 = NB > 1 ? dshfl(x[NB - 1], s & 31) : t0;
        w[q] = i < n ? (s >= 32 ? t1 : t0) : dmk(0.0, 0.0);
    }
    for (int k = 0; k < n - 1; ++k) {
        const cdbl xk = d_bcast<NB>(w, k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i > k && i < n) w[q] = dsub(w[q], dmul(A[i * n + k], xk));
        }
    }
    for (int k = n - 1; k >= 0; --k) {
#pragma unroll
        for (int q = 0; q < NB; ++q)
            if (lane + 32 * q == k) w[q] = ddiv(w[q], A[k * n + k]);
        const cdbl xk = d_bcast<NB>(w, k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i < k) w[q] = dsub(w[q], dmul(A[i * n + k], xk));
        }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) x[q] = w[q];
}

template <int NB>
__device__ void publish64(cdbl* vpub, const cdbl (&x)[NB], int n, int lane) {
    __syncwarp();
#pragma unroll
    for (int q = 0; q < NB; ++q)
        if (lane + 32 * q < n) vpub[lane + 32 * q] = x[q];
    __syncwarp();
}

// y = H x for Hermitian packed-lower H, x published in vpub
template <int NB>
__device__ void hermv64(const cdbl* H, int n, const cdbl* vpub, cdbl (&y)[NB], int lane) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        cdbl acc = dmk(0.0, 0.0);
        if (i < n) {
            for (int j = 0; j < n; ++j) acc = dadd(acc, dmul(dget(H, i, j), vpub[j]));
        }
        y[q] = acc;
    }
}

template <int NB, class Op>
__device__ bool iterate64(cdbl (&v)[NB], Op&& op) {
    double diff = 1.0;
    for (int it = 1; diff > 1e-5 && it < 50; ++it) {
        cdbl x[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) x[q] = v[q];
        op(x);
        const double inv = 1.0 / sqrt(d_norm2<NB>(x));
        double dd = 0.0;
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            x[q] = dscale(x[q], inv);
            dd += dabs2(dsub(x[q], v[q]));
            v[q] = x[q];
        }
        diff = sqrt(dwarp_sum(dd));
    }
    return !(diff > 1e-5);  // a NaN difference ends the loop too, as in the reference
}

// The dense eigensolver of the non-convergence fallback in double (the FP64 form is a
// reference form, so the whole spectrum is computed): cyclic Jacobi for Hermitian
// matrices (Golub & Van Loan, Matrix Computations, section 8.5; each rotation removes
// the pivot's phase with a diagonal unitary, then applies the real rotation) on A (n x n,
// both triangles), eigenvectors in the columns of V, eigenvalues on the diagonal of A.
constexpr int kJacobiMaxSweeps = 30;

__device__ inline void e_jacobi64(cdbl* A, cdbl* V, int n, int lane) {
    for (int i = 0; i < n; ++i)
        for (int j = lane; j < n; j += 32) V[i * n + j] = dmk(i == j ? 1.0 : 0.0, 0.0);
    __syncwarp();
    for (int sweep = 0; sweep < kJacobiMaxSweeps; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) {
                const double m2 = dabs2(A[i * n + j]);
                tot += m2;
                if (j != i) off += m2;
            }
        off = dwarp_sum(off);
        tot = dwarp_sum(tot);
        if (!(off > 1e-30 * tot)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const cdbl b = A[p * n + q];
                const double e = sqrt(dabs2(b));
                if (!(e > 0.0)) continue;
                const double a = A[p * n + p].re, d = A[q * n + q].re;
                const double zeta = (d - a) / (2.0 * e);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
                const cdbl ph = dmk(b.re / e, b.im / e);
                const cdbl sm = dmk(s * ph.re, -s * ph.im);
                const cdbl cm = dmk(c * ph.re, -c * ph.im);
                __syncwarp();
                for (int k = lane; k < n; k += 32) {
                    const cdbl xp = A[k * n + p], xq = A[k * n + q];
                    A[k * n + p] = dsub(dscale(xp, c), dmul(sm, xq));
                    A[k * n + q] = dadd(dscale(xp, s), dmul(cm, xq));
                    const cdbl vp = V[k * n + p], vq = V[k * n + q];
                    V[k * n + p] = dsub(dscale(vp, c), dmul(sm, vq));
                    V[k * n + q] = dadd(dscale(vp, s), dmul(cm, vq));
                }
                __syncwarp();
                for (int k = lane; k < n; k += 32) {
                    const cdbl xp = A[p * n + k], xq = A[q * n + k];
                    A[p * n + k] = dsub(dscale(xp, c), dmul(dconj(sm), xq));
                    A[q * n + k] = dadd(dscale(xp, s), dmul(dconj(cm), xq));
                }
                __syncwarp();
                if (lane == 0) {
                    A[p * n + q] = dmk(0.0, 0.0);
                    A[q * n + p] = dmk(0.0, 0.0);
                    A[p * n + p] = dmk(a - t * e, 0.0);
                    A[q * n + q] = dmk(d + t * e, 0.0);
                }
                __syncwarp();
            }
    }
    __syncwarp();
}

// The fallback's choice on diag(A) after e_jacobi64: EMI the eigenvalue nearest 0.99,
// EVD the largest in magnitude; v (lane i + 32 q holds entry i) gets that column of V
// at unit norm, and the eigenvalue is returned.
template <int NB>
__device__ double pick64(const cdbl* A, const cdbl* V, int n, bool evd, cdbl (&v)[NB], int lane) {
    double best = INFINITY;
    int bi = n;
    for (int i = lane; i < n; i += 32) {
        const double lam = A[i * n + i].re;
        const double score = evd ? -fabs(lam) : fabs(lam - 0.99);
        if (score < best) {
            best = score;
            bi = i;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob < best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    if (bi >= n) bi = 0;
    double s2 = 0.0;
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        v[q] = i < n ? V[i * n + bi] : dmk(0.0, 0.0);
        s2 += dabs2(v[q]);
    }
    const double inv = 1.0 / sqrt(dwarp_sum(s2));
#pragma unroll
    for (int q = 0; q < NB; ++q) v[q] = dscale(v[q], inv);
    return A[bi * n + bi].re;
}

__device__ __forceinline__ double gamma64(const PixArgs& a, cdbl c, bool diag) {
    double g = sqrt(dabs2(c));
    if (a.beta_on) g = (1.0 - a.beta_d) * g + (diag ? a.beta_d : 0.0);
    return g < a.zct_d ? 0.0 : g;
}

template <int NB>
__device__ void solve64(const PixArgs& a, int64_t p, cdbl* C, double* G, int ld, cdbl* A, cdbl* V, cdbl* vp,
                        int* piv, int lane) {
    const int n = a.n;
    if (a.baseline_lag > 0) {
        for (int i = a.baseline_lag; i < n; ++i)
            for (int j = lane; j <= i - a.baseline_lag; j += 32) C[pk(i, j)] = dmk(0.0, 0.0);
        __syncwarp();
    }
    if (a.closure) {
        for (int i = lane; i < n - 2; i += 32) {
            const cdbl c = dmulc(dmul(dget(C, i, i + 1), dget(C, i + 1, i + 2)), dget(C, i, i + 2));
            a.closure[p * (n - 2) + i] = (float)atan2(c.im, c.re);
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = lane; j < n; j += 32) G[i * ld + j] = gamma64(a, dget(C, i, j), i == j) + (i == j ? 1e-6 : 0.0);
    bool inv_nan;
    if (gj64<NB>(G, n, ld, lane)) {
        bool bad = false;
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) bad |= isnan(G[i * ld + j]);
        inv_nan = warp_any(bad);
    } else {
        __syncwarp();
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) G[i * ld + j] = nan("");
        inv_nan = true;
    }
    __syncwarp();
    const bool evd = a.use_evd || inv_nan;
    cdbl v[NB];
    const double inv_sqrt_n = 1.0 / sqrt((double)n);
#pragma unroll
    for (int q = 0; q < NB; ++q) v[q] = lane + 32 * q < n ? dmk(inv_sqrt_n, 0.0) : dmk(0.0, 0.0);
    double lambda;
    bool converged;
    if (!evd) {
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) {
                cdbl x = dscale(dget(C, i, j), G[i * ld + j]);
                if (i == j) x.re -= 0.99;
                A[i * n + j] = x;
            }
        __syncwarp();
        lu64(A, n, piv, lane);
        int* src = piv + 64;
        if (lane == 0) {
            for (int i = 0; i < n; ++i) src[i] = i;
            for (int k = 0; k < n; ++k) {
                const int t = src[k];
                src[k] = src[piv[k]];
                src[piv[k]] = t;
            }
        }
        __syncwarp();
        converged = iterate64<NB>(v, [&](cdbl(&x)[NB]) { lusolve64<NB>(A, n, src, x, lane); });
        publish64<NB>(vp, v, n, lane);
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i < n) {
                cdbl acc = dmk(0.0, 0.0);
                for (int j = 0; j < n; ++j) acc = dadd(acc, dmul(dscale(dget(C, i, j), G[i * ld + j]), vp[j]));
                s += v[q].re * acc.re + v[q].im * acc.im;
            }
        }
        lambda = dwarp_sum(s);
        if (!converged && a.eigh) {
            // the dense eigensolver on A = |Gamma|^{-1} o C (the LU factors are no longer needed)
            __syncwarp();
            for (int i = 0; i < n; ++i)
                for (int j = lane; j < n; j += 32) A[i * n + j] = dscale(dget(C, i, j), G[i * ld + j]);
            e_jacobi64(A, V, n, lane);
            lambda = pick64<NB>(A, V, n, false, v, lane);
        }
        const double scale = sqrt((double)n) / sqrt(d_norm2<NB>(v));
#pragma unroll
        for (int q = 0; q < NB; ++q) v[q] = dscale(v[q], scale);
    } else {
        const int T = tri(n);
        for (int e = lane; e < T; e += 32) A[e] = dscale(C[e], sqrt(dabs2(C[e])));
        __syncwarp();
        converged = iterate64<NB>(v, [&](cdbl(&x)[NB]) {
            publish64<NB>(vp, x, n, lane);
            hermv64<NB>(A, n, vp, x, lane);
        });
        publish64<NB>(vp, v, n, lane);
        cdbl y[NB];
        hermv64<NB>(A, n, vp, y, lane);
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < NB; ++q) s += v[q].re * y[q].re + v[q].im * y[q].im;
        lambda = dwarp_sum(s);
        if (!converged && a.eigh) {
            // the dense eigensolver on the full C o |C|
            __syncwarp();
            for (int i = 0; i < n; ++i)
                for (int j = lane; j < n; j += 32) {
                    const cdbl c = dget(C, i, j);
                    V[i * n + j] = dscale(c, sqrt(dabs2(c)));
                }
            __syncwarp();
            for (int i = 0; i < n; ++i)
                for (int j = lane; j < n; j += 32) A[i * n + j] = V[i * n + j];
            e_jacobi64(A, V, n, lane);
            lambda = pick64<NB>(A, V, n, true, v, lane);
        }
    }
    __syncwarp();
    if (a.compute_crlb) {
        const int ref = a.crlb_ref;
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) {
                double f;
                if (i == ref || j == ref) {
                    f = i == j ? 1.0 : 0.0;
                } else {
                    const double x = a.crlb_factor_d * (gamma64(a, dget(C, i, j), i == j) * G[i * ld + j] -
                                                        (i == j ? 1.0 : 0.0));
                    f = i == j ? x + 1e-6 : x;
                }
                G[i * ld + j] = f;
            }
        const bool ok = gj64<NB>(G, n, ld, lane);
        for (int t = lane; t < n; t += 32)
            a.crlb[p * n + t] = t == ref ? 0.f : (ok ? (float)sqrt(G[t * ld + t]) : nanf(""));
        __syncwarp();
    } else {
        for (int t = lane; t < n; t += 32) a.crlb[p * n + t] = 0.f;
    }
    const cdbl rot = dconj(dphasor(d_bcast<NB>(v, a.ref_idx)));
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        v[q] = dmul(v[q], rot);
        if (i < n) a.vout[p * n + i] = cmake((float)v[q].re, (float)v[q].im);
    }
    if (lane == 0) {
        a.eig[p] = (float)lambda;
        a.est[p] = evd ? 0 : 1;
        if (a.nc_flag) a.nc_flag[p] = !converged && a.eigh ? 1 : 0;
    }
    cdbl w[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) w[q] = dphasor(v[q]);
    publish64<NB>(vp, w, n, lane);
    double sre = 0.0, sim = 0.0;
    int cnt = 0;
    for (int r = 1; r < n; ++r) {
        const cdbl wr = vp[r];
        for (int c = lane; c < r; c += 32) {
            const cdbl u = dphasor(C[pk(r, c)]);
            const cdbl t = dconj(dmulc(dmul(u, vp[c]), wr));
            if (!disnan(t)) {
                sre += t.re;
                sim += t.im;
                ++cnt;
            }
        }
    }
    sre = dwarp_sum(sre);
    sim = dwarp_sum(sim);
    cnt = warp_sum_int(cnt);
    if (lane == 0) {
        const double tc = hypot(sre / cnt, sim / cnt);
        a.tcoh[p] = isfinite(tc) ? (float)tc : 0.f;
    }
    __syncwarp();
}

template <int NB>
__global__ void __launch_bounds__(128) k_pixel64(PixArgs a, Pix64Layout L) {
    extern __shared__ __align__(16) unsigned char smem64[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    unsigned char* base = smem64 + warp * L.bytes;
    cdbl* C = reinterpret_cast<cdbl*>(base + L.off_C);
    double* G = reinterpret_cast<double*>(base + L.off_G);
    cdbl* A = reinterpret_cast<cdbl*>(base + L.off_A);
    cdbl* V = reinterpret_cast<cdbl*>(base + L.off_V);
    cdbl* vp = reinterpret_cast<cdbl*>(base + L.off_v);
    int* piv = reinterpret_cast<int*>(base + L.off_piv);
    for (int64_t p = (int64_t)blockIdx.x * nwarps + warp; p < a.npix; p += (int64_t)gridDim.x * nwarps) {
        int count = 0;
        cov64<NB>(a, p, C, reinterpret_cast<cfloat*>(A), reinterpret_cast<double*>(vp), lane, &count);
        if (a.counts && lane == 0) a.counts[p] = count;
        solve64<NB>(a, p, C, G, L.ldg, A, V, vp, piv, lane);
    }
}

}  // namespace dpl
