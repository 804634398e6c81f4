// Per-pixel solver: one warp per pixel, matrices in the warp's shared memory.
//
// Storage is packed lower-triangular (element (i, j), j <= i, at i(i+1)/2 + j): the
// coherence matrix C and every matrix derived from it is Hermitian or symmetric,
// so this halves shared memory per warp and lets more warps share an SM.  Loops
// run over rows with the lanes over columns (no index division, short divergent
// tails); triangular solves keep the iterate in registers (lane i owns entry i,
// entry i + 32 for N > 32) and broadcast pivots with shuffles.
//
// Algorithms (all float32, as the reference):
//   |Gamma| (+ beta I, zero threshold) + 1e-6 I = L L^T     (_core.py:452-467)
//   Y = L^{-1} (row by row), |Gamma|^{-1} = Y^T Y            (cho_solve(I), :472)
//   EMI: A - 0.99 I = R R^H (complex Cholesky of the Hermitian shifted matrix) and
//        inverse iteration v <- (R R^H)^{-1} v / |.|, <= 49 steps, stop at
//        |v_new - v| <= 1e-5 (_eigenvalues.py:139-205).  These are the iterates of
//        the reference's LU solve; where A - 0.99 I is not positive definite the
//        same iteration runs on an LU factorisation with partial pivoting.
//        lambda = v^H A v = |R^H v|^2 + 0.99 |v|^2.
//   EVD: power iteration on C o |C| (_eigenvalues.py:93-136) for use_evd and for
//        pixels whose |Gamma|^{-1} has NaNs (_core.py:496-515).
//   CRLB: FIM = 2L (Gamma o Gamma^{-1} - I) without row/column `ref`, + 1e-6 I,
//        sigma = sqrt(diag FIM^{-1}) with 0 at `ref` (crlb.py:132-189).
#pragma once

namespace dpl {

__host__ __device__ __forceinline__ int tri(int i) { return i * (i + 1) / 2; }
__host__ __device__ __forceinline__ int pk(int i, int j) { return tri(i) + j; }  // j <= i

// C_ij for any (i, j) from packed-lower storage
__device__ __forceinline__ cfloat cget(const cfloat* C, int i, int j) {
    return j <= i ? C[pk(i, j)] : cconj(C[pk(j, i)]);
}

struct SolveMats {
    cfloat* C;   // packed coherence
    float* W1;   // packed real
    float* W2;   // packed real
    cfloat* R;   // packed complex factor / B for EVD; LU (full, ld = n) on the fallback
    cfloat* v;   // 64 published vector entries
    float* d;    // 64 floats
    int* piv;    // 64 pivots (LU fallback)
};

// Real Cholesky in place on packed W (n x n).  Uniform result.
__device__ bool s_chol_real(float* W, int n, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        const float d = W[pk(k, k)];
        if (!(d > 0.f)) return false;
        const float lkk = fsqrt(d);
        __syncwarp();
        for (int i = k + 1 + lane; i < n; i += 32) W[pk(i, k)] = fdiv(W[pk(i, k)], lkk);
        if (lane == 0) W[pk(k, k)] = lkk;
        __syncwarp();
        for (int i = k + 1; i < n; ++i) {
            const float lik = W[pk(i, k)];
            for (int j = k + 1 + lane; j <= i; j += 32) W[pk(i, j)] -= lik * W[pk(j, k)];
        }
    }
    __syncwarp();
    return true;
}

// Y = L^{-1} (packed, lower) from packed L: row i = (e_i - sum_{k<i} l_ik y_k) / l_ii.
// If sumsq != nullptr, also the column sums of squares sum_k Y_kj^2 (lane-owned j).
__device__ void s_tri_inverse(const float* L, float* Y, int n, int lane, float* sumsq) {
    for (int i = 0; i < n; ++i) {
        __syncwarp();
        const float lii = L[pk(i, i)];
        for (int j = lane; j <= i; j += 32) {
            float s = i == j ? 1.f : 0.f;
            for (int k = j; k < i; ++k) s -= L[pk(i, k)] * Y[pk(k, j)];
            Y[pk(i, j)] = fdiv(s, lii);
        }
    }
    __syncwarp();
    if (sumsq) {
        for (int j = lane; j < n; j += 32) {
            float ss = 0.f;
            for (int k = j; k < n; ++k) {
                const float y = Y[pk(k, j)];
                ss += y * y;
            }
            sumsq[j] = ss;
        }
        __syncwarp();
    }
}

// Complex Cholesky in place on packed R (Hermitian, lower stored).  Uniform result.
__device__ bool s_chol_complex(cfloat* R, int n, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        const float d = R[pk(k, k)].re;
        if (!(d > 0.f)) return false;
        const float lkk = fsqrt(d);
        __syncwarp();
        for (int i = k + 1 + lane; i < n; i += 32) {
            const cfloat x = R[pk(i, k)];
            R[pk(i, k)] = cmake(fdiv(x.re, lkk), fdiv(x.im, lkk));
        }
        if (lane == 0) R[pk(k, k)] = cmake(lkk, 0.f);
        __syncwarp();
        for (int i = k + 1; i < n; ++i) {
            const cfloat lik = R[pk(i, k)];
            for (int j = k + 1 + lane; j <= i; j += 32) R[pk(i, j)] = csub(R[pk(i, j)], cmulc(lik, R[pk(j, k)]));
        }
    }
    __syncwarp();
    return true;
}

template <int NB>
__device__ __forceinline__ cfloat s_bcast(const cfloat (&x)[NB], int k) {
    cfloat r = shfl_c(x[0], k & 31);
    if (NB > 1) {
        const cfloat r1 = shfl_c(x[NB - 1], k & 31);
        if (k >= 32) r = r1;
    }
    return r;
}

template <int NB>
__device__ __forceinline__ float s_norm2(const cfloat (&x)[NB]) {
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < NB; ++q) s += cabs2(x[q]);
    return warp_sum(s);
}

// x <- (R R^H)^{-1} x with packed lower R (real positive diagonal)
template <int NB>
__device__ void s_chol_solve(const cfloat* R, int n, cfloat (&x)[NB], int lane) {
    for (int k = 0; k < n; ++k) {
        const float rkk = R[pk(k, k)].re;
#pragma unroll
        for (int q = 0; q < NB; ++q)
            if (lane + 32 * q == k) x[q] = cmake(fdiv(x[q].re, rkk), fdiv(x[q].im, rkk));
        const cfloat yk = s_bcast<NB>(x, k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i > k && i < n) x[q] = csub(x[q], cmul(R[pk(i, k)], yk));
        }
    }
    for (int k = n - 1; k >= 0; --k) {
        const float rkk = R[pk(k, k)].re;
#pragma unroll
        for (int q = 0; q < NB; ++q)
            if (lane + 32 * q == k) x[q] = cmake(fdiv(x[q].re, rkk), fdiv(x[q].im, rkk));
        const cfloat xk = s_bcast<NB>(x, k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i < k) x[q] = csub(x[q], cmul(cconj(R[pk(k, i)]), xk));
        }
    }
}

// LU with partial pivoting (getrf: first maximum of |re| + |im|) on a full n x n
// matrix (ld = n); piv[k] = pivot row of step k.
__device__ void s_lu(cfloat* A, int n, int* piv, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        float best = -1.f;
        int bi = n;
        for (int i = k + lane; i < n; i += 32) {
            const cfloat x = A[i * n + k];
            const float v = fabsf(x.re) + fabsf(x.im);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
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
                const cfloat t = A[k * n + j];
                A[k * n + j] = A[bi * n + j];
                A[bi * n + j] = t;
            }
        __syncwarp();
        const cfloat pv = A[k * n + k];
        if (pv.re != 0.f || pv.im != 0.f) {
            const cfloat r = cdiv(cmake(1.f, 0.f), pv);
            for (int i = k + 1 + lane; i < n; i += 32) A[i * n + k] = cmul(A[i * n + k], r);
        }
        __syncwarp();
        for (int i = k + 1; i < n; ++i) {
            const cfloat lik = A[i * n + k];
            for (int j = k + 1 + lane; j < n; j += 32) A[i * n + j] = csub(A[i * n + j], cmul(lik, A[k * n + j]));
        }
    }
    __syncwarp();
}

// x <- (LU)^{-1} P x; `src[i]` is the original row that pivoting moved to row i
template <int NB>
__device__ void s_lu_solve(const cfloat* A, int n, const int* src, cfloat (&x)[NB], int lane) {
    cfloat w[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        const int s = i < n ? src[i] : 0;
        const cfloat t0 = shfl_c(x[0], s & 31);
        const cfloat t1 = NB > 1 ? shfl_c(x[NB - 1], s & 31) : t0;
        w[q] = i < n ? (s >= 32 ? t1 : t0) : cmake(0.f, 0.f);
    }
    for (int k = 0; k < n - 1; ++k) {
        const cfloat xk = s_bcast<NB>(w, k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i > k && i < n) w[q] = csub(w[q], cmul(A[i * n + k], xk));
        }
    }
    for (int k = n - 1; k >= 0; --k) {
#pragma unroll
        for (int q = 0; q < NB; ++q)
            if (lane + 32 * q == k) w[q] = cdiv(w[q], A[k * n + k]);
        const cfloat xk = s_bcast<NB>(w, k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i < k) w[q] = csub(w[q], cmul(A[i * n + k], xk));
        }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) x[q] = w[q];
}

__device__ __forceinline__ float s_gamma(const PixArgs& a, cfloat c, bool diag) {
    float g = hypotf(c.re, c.im);
    if (a.beta_on) g = fadd(fmul(a.one_minus_beta, g), diag ? a.beta : 0.f);
    return g < a.zct ? 0.f : g;
}

// y_i = sum_j H_ij x_j for Hermitian H in packed lower storage; x published in vpub
template <int NB>
__device__ void s_hermv(const cfloat* H, int n, const cfloat* vpub, cfloat (&y)[NB], int lane) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        cfloat acc = cmake(0.f, 0.f);
        if (i < n) {
            for (int j = 0; j < n; ++j) acc = cadd(acc, cmul(cget(H, i, j), vpub[j]));
        }
        y[q] = acc;
    }
}

template <int NB>
__device__ void s_publish(cfloat* vpub, const cfloat (&x)[NB], int n, int lane) {
    __syncwarp();
#pragma unroll
    for (int q = 0; q < NB; ++q)
        if (lane + 32 * q < n) vpub[lane + 32 * q] = x[q];
    __syncwarp();
}

// Full solve for one pixel whose packed coherence matrix is in m.C.
template <int NB>
__device__ void solve_pixel(const PixArgs& a, int64_t p, const SolveMats& m, int lane) {
    const int n = a.n, T = tri(n);
    cfloat* C = m.C;
    if (a.baseline_lag > 0) {
        for (int i = a.baseline_lag; i < n; ++i)
            for (int j = lane; j <= i - a.baseline_lag; j += 32) C[pk(i, j)] = cmake(0.f, 0.f);
        __syncwarp();
    }
    if (a.closure) {
        for (int i = lane; i < n - 2; i += 32) {
            const cfloat c = cmulc(cmul(cget(C, i, i + 1), cget(C, i + 1, i + 2)), cget(C, i, i + 2));
            a.closure[p * (n - 2) + i] = atan2f(c.im, c.re);
        }
    }
    // |Gamma| + 1e-6 I -> L (W1) -> Y (W2) -> |Gamma|^{-1} (W1)
    for (int i = 0; i < n; ++i)
        for (int j = lane; j <= i; j += 32) m.W1[pk(i, j)] = fadd(s_gamma(a, C[pk(i, j)], i == j), i == j ? 1e-6f : 0.f);
    bool inv_nan;
    if (s_chol_real(m.W1, n, lane)) {
        s_tri_inverse(m.W1, m.W2, n, lane, nullptr);
        bool bad = false;
        for (int i = 0; i < n; ++i) {
            for (int j = lane; j <= i; j += 32) {
                float s = 0.f;
                for (int k = i; k < n; ++k) s += m.W2[pk(k, i)] * m.W2[pk(k, j)];
                m.W1[pk(i, j)] = s;
                bad |= isnan(s);
            }
        }
        inv_nan = warp_any(bad);
    } else {
        for (int e = lane; e < T; e += 32) m.W1[e] = nanf("");
        inv_nan = true;
    }
    __syncwarp();
    const bool evd = a.use_evd || inv_nan;
    // A - 0.99 I (EMI) or C o |C| (EVD) into R
    if (!evd) {
        for (int i = 0; i < n; ++i)
            for (int j = lane; j <= i; j += 32) {
                cfloat x = cscale(C[pk(i, j)], m.W1[pk(i, j)]);
                if (i == j) x.re = fsub(x.re, 0.99f);
                m.R[pk(i, j)] = x;
            }
    } else {
        for (int e = lane; e < T; e += 32) {
            const cfloat c = C[e];
            m.R[e] = cscale(c, hypotf(c.re, c.im));
        }
    }
    __syncwarp();
    cfloat v[NB];
    const float inv_sqrt_n = fdiv(1.f, fsqrt((float)n));
#pragma unroll
    for (int q = 0; q < NB; ++q) v[q] = lane + 32 * q < n ? cmake(inv_sqrt_n, 0.f) : cmake(0.f, 0.f);
    float lambda;
    if (!evd) {
        // keep A - 0.99 I (full) for the LU fallback before factorising in place
        const bool chol_ok = s_chol_complex(m.R, n, lane);
        if (chol_ok) {
            float diff = 1.f;
            for (int it = 1; diff > 1e-5f && it < 50; ++it) {
                cfloat x[NB];
#pragma unroll
                for (int q = 0; q < NB; ++q) x[q] = v[q];
                s_chol_solve<NB>(m.R, n, x, lane);
                const float nrm = fsqrt(s_norm2<NB>(x));
                float dd = 0.f;
#pragma unroll
                for (int q = 0; q < NB; ++q) {
                    x[q] = cmake(fdiv(x[q].re, nrm), fdiv(x[q].im, nrm));
                    dd += cabs2(csub(x[q], v[q]));
                    v[q] = x[q];
                }
                diff = fsqrt(warp_sum(dd));
            }
            // lambda = |R^H v|^2 + 0.99 |v|^2
            s_publish<NB>(m.v, v, n, lane);
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                const int i = lane + 32 * q;
                if (i < n) {
                    cfloat acc = cmake(0.f, 0.f);
                    for (int k = i; k < n; ++k) acc = cadd(acc, cmulc(m.v[k], m.R[pk(k, i)]));
                    s += cabs2(acc);
                }
            }
            lambda = fadd(warp_sum(s), fmul(0.99f, s_norm2<NB>(v)));
        } else {
            // LU fallback on the full shifted matrix (rebuilt from C and |Gamma|^{-1})
            cfloat* A = m.R;  // the scratch region holds n*n complex (see the layout)
            __syncwarp();
            for (int i = 0; i < n; ++i)
                for (int j = lane; j < n; j += 32) {
                    const cfloat c = cget(C, i, j);
                    cfloat x = cscale(c, j <= i ? m.W1[pk(i, j)] : m.W1[pk(j, i)]);
                    if (i == j) x.re = fsub(x.re, 0.99f);
                    A[i * n + j] = x;
                }
            __syncwarp();
            s_lu(A, n, m.piv, lane);
            int* src = m.piv + 64;
            if (lane == 0) {
                for (int i = 0; i < n; ++i) src[i] = i;
                for (int k = 0; k < n; ++k) {
                    const int pk_ = m.piv[k];
                    const int t = src[k];
                    src[k] = src[pk_];
                    src[pk_] = t;
                }
            }
            __syncwarp();
            float diff = 1.f;
            for (int it = 1; diff > 1e-5f && it < 50; ++it) {
                cfloat x[NB];
#pragma unroll
                for (int q = 0; q < NB; ++q) x[q] = v[q];
                s_lu_solve<NB>(A, n, src, x, lane);
                const float nrm = fsqrt(s_norm2<NB>(x));
                float dd = 0.f;
#pragma unroll
                for (int q = 0; q < NB; ++q) {
                    x[q] = cmake(fdiv(x[q].re, nrm), fdiv(x[q].im, nrm));
                    dd += cabs2(csub(x[q], v[q]));
                    v[q] = x[q];
                }
                diff = fsqrt(warp_sum(dd));
            }
            // lambda = Re(v^H (|Gamma|^{-1} o C) v)
            s_publish<NB>(m.v, v, n, lane);
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                const int i = lane + 32 * q;
                if (i < n) {
                    cfloat acc = cmake(0.f, 0.f);
                    for (int j = 0; j < n; ++j) {
                        const float w = j <= i ? m.W1[pk(i, j)] : m.W1[pk(j, i)];
                        acc = cadd(acc, cmul(cscale(cget(C, i, j), w), m.v[j]));
                    }
                    s += v[q].re * acc.re + v[q].im * acc.im;
                }
            }
            lambda = warp_sum(s);
        }
        const float scale = fdiv(fsqrt((float)n), fsqrt(s_norm2<NB>(v)));
#pragma unroll
        for (int q = 0; q < NB; ++q) v[q] = cscale(v[q], scale);
    } else {
        float diff = 1.f;
        for (int it = 1; diff > 1e-5f && it < 50; ++it) {
            s_publish<NB>(m.v, v, n, lane);
            cfloat y[NB];
            s_hermv<NB>(m.R, n, m.v, y, lane);
            const float nrm = fsqrt(s_norm2<NB>(y));
            float dd = 0.f;
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                y[q] = cmake(fdiv(y[q].re, nrm), fdiv(y[q].im, nrm));
                dd += cabs2(csub(y[q], v[q]));
                v[q] = y[q];
            }
            diff = fsqrt(warp_sum(dd));
        }
        s_publish<NB>(m.v, v, n, lane);
        cfloat y[NB];
        s_hermv<NB>(m.R, n, m.v, y, lane);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < NB; ++q) s += v[q].re * y[q].re + v[q].im * y[q].im;
        lambda = warp_sum(s);
    }
    __syncwarp();
    // CRLB (needs |Gamma|^{-1} in W1; FIM in W2, its inverse factor in the R region)
    if (a.compute_crlb) {
        const int ref = a.crlb_ref;
        for (int i = 0; i < n; ++i)
            for (int j = lane; j <= i; j += 32) {
                float f;
                if (i == ref || j == ref) {
                    f = i == j ? 1.f : 0.f;
                } else {
                    const float x = fmul(a.crlb_factor,
                                         fsub(fmul(s_gamma(a, C[pk(i, j)], i == j), m.W1[pk(i, j)]), i == j ? 1.f : 0.f));
                    f = i == j ? fadd(x, 1e-6f) : x;
                }
                m.W2[pk(i, j)] = f;
            }
        const bool ok = s_chol_real(m.W2, n, lane);
        if (ok) s_tri_inverse(m.W2, reinterpret_cast<float*>(m.R), n, lane, m.d);
        for (int t = lane; t < n; t += 32) a.crlb[p * n + t] = t == ref ? 0.f : (ok ? fsqrt(m.d[t]) : nanf(""));
        __syncwarp();
    } else {
        for (int t = lane; t < n; t += 32) a.crlb[p * n + t] = 0.f;
    }

    // reference to reference_idx
    const cfloat rot = cconj(cphasor(s_bcast<NB>(v, a.ref_idx)));
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        v[q] = cmul(v[q], rot);
        if (i < n) a.vout[p * n + i] = v[q];
    }
    if (lane == 0) {
        a.eig[p] = lambda;
        a.est[p] = evd ? 0 : 1;
    }
    s_publish<NB>(m.v, v, n, lane);
    // temporal coherence over pairs i < j (stored as packed (j, i))
    float sre = 0.f, sim = 0.f;
    int cnt = 0;
    for (int r = 1; r < n; ++r) {
        const cfloat vr = m.v[r];
        for (int c = lane; c < r; c += 32) {
            const cfloat u = cphasor(cconj(C[pk(r, c)]));    // phasor of C_cr
            const cfloat w = cphasor(cmulc(m.v[c], vr));     // v_c conj(v_r)
            const cfloat t = cmulc(u, w);
            if (!cisnan(t)) {
                sre += t.re;
                sim += t.im;
                ++cnt;
            }
        }
    }
    sre = warp_sum(sre);
    sim = warp_sum(sim);
    cnt = warp_sum_int(cnt);
    if (lane == 0) {
        const float fc = (float)cnt;
        const float tc = hypotf(fdiv(sre, fc), fdiv(sim, fc));
        a.tcoh[p] = isfinite(tc) ? tc : 0.f;
    }
    __syncwarp();
}

}  // namespace dpl
