// Per-pixel solver: one warp per pixel, matrices in the warp's shared memory.
//
// Storage: the coherence matrix C and the EMI factor R are packed lower-triangular
// complex (element (i, j), j <= i, at i(i+1)/2 + j); the real |Gamma| work matrix G
// is full with an odd row stride (conflict-free column access).  Loops run over rows
// with the lanes over columns; triangular solves keep the iterate in registers
// (lane i owns entry i, and entry i + 32 when N > 32) and broadcast with shuffles.
//
// Algorithms (all float32, as the reference):
//   |Gamma| (+ beta I, zero threshold) + 1e-6 I, inverted in place by Gauss-Jordan
//        elimination (the symmetric positive definite case needs no pivoting; a
//        non-positive pivot means "not positive definite", where the reference's
//        cho_factor fails and the pixel falls back to EVD)      (_core.py:452-515)
//   EMI: A - 0.99 I = R R^H (complex Cholesky of the Hermitian shifted matrix) and
//        inverse iteration v <- (R R^H)^{-1} v / |.|, <= 49 steps, stop at
//        |v_new - v| <= 1e-5 (_eigenvalues.py:139-205).  These are the iterates of
//        the reference's LU solve.  Where A - 0.99 I is not positive definite the
//        pixel is listed and a second pass runs the same iteration on an LU
//        factorisation with partial pivoting (the reference's algorithm).
//        lambda = v^H A v = |R^H v|^2 + 0.99 |v|^2.
//   EVD: power iteration on C o |C| (_eigenvalues.py:93-136) for use_evd and for
//        pixels whose |Gamma|^{-1} has NaNs.
//   CRLB: FIM = 2L (Gamma o Gamma^{-1} - I) with row/column `ref` replaced by the
//        identity, + 1e-6 I, inverted by Gauss-Jordan; sigma = sqrt(diag FIM^{-1}),
//        0 at `ref` (crlb.py:132-189).
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
    float* G;    // n x ldg real work matrix
    int ldg;
    cfloat* R;   // packed complex (EMI factor, or C o |C| for EVD); full n x n LU in the LU pass
    cfloat* v;   // 64 published vector entries
    float* d;    // 64 floats (inverse diagonal of R)
    int* piv;    // 128 ints (LU pass)
};

// unit phasor exp(i angle(c)) via rsqrt, without branches; angle(+0) = 0,
// angle(-0 + 0j) = pi, NaN stays NaN
__device__ __forceinline__ cfloat fphasor(cfloat c) {
    const float m2 = c.re * c.re + c.im * c.im;
    const float r = rsqrtf(m2);
    const bool z = m2 == 0.f;
    return cmake(z ? copysignf(1.f, c.re) : c.re * r, z ? 0.f : c.im * r);
}

// In-place inverse of a symmetric positive definite n x n matrix by Gauss-Jordan
// elimination.  Returns false (uniformly) on a non-positive pivot.  Lanes own
// columns; column k is left unchanged by the row sweep (its multiplier is 0) and
// rewritten afterwards.
template <int NB>
__device__ bool s_gauss_jordan_spd(float* A, int n, int ld, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        const float piv = A[k * ld + k];
        if (!(piv > 0.f)) return false;
        const float inv = 1.f / piv;
        float rk[NB], rm[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int j = lane + 32 * q;
            rk[q] = j < n ? (j == k ? inv : A[k * ld + j] * inv) : 0.f;
            rm[q] = j == k ? 0.f : rk[q];
        }
        const float* colk = A + k;
        float* mine = A + lane;
#pragma unroll 4
        for (int i = 0; i < k; ++i) {
            const float f = colk[i * ld];
#pragma unroll
            for (int q = 0; q < NB; ++q)
                if (lane + 32 * q < n) mine[i * ld + 32 * q] -= f * rm[q];
        }
#pragma unroll 4
        for (int i = k + 1; i < n; ++i) {
            const float f = colk[i * ld];
#pragma unroll
            for (int q = 0; q < NB; ++q)
                if (lane + 32 * q < n) mine[i * ld + 32 * q] -= f * rm[q];
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

// Complex Cholesky in place on packed R (Hermitian, lower stored); dinv[k] = 1/R_kk.
__device__ inline bool s_chol_complex(cfloat* R, float* dinv, int n, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        const float d = R[pk(k, k)].re;
        if (!(d > 0.f)) return false;
        const float lkk = sqrtf(d);
        const float il = 1.f / lkk;
        for (int i = k + 1 + lane; i < n; i += 32) R[pk(i, k)] = cscale(R[pk(i, k)], il);
        __syncwarp();
        if (lane == 0) {
            R[pk(k, k)] = cmake(lkk, 0.f);
            dinv[k] = il;
        }
        // trailing update R_ij -= R_ik conj(R_jk), k < j <= i; lanes own columns j
        const int j0 = k + 1 + lane, j1 = j0 + 32;
        const cfloat l0 = j0 < n ? R[pk(j0, k)] : cmake(0.f, 0.f);
        const cfloat l1 = j1 < n ? R[pk(j1, k)] : cmake(0.f, 0.f);
        int bi = tri(k + 1);
#pragma unroll 2
        for (int i = k + 1; i < n; ++i) {
            const cfloat lik = R[bi + k];
            if (j0 <= i) R[bi + j0] = csub(R[bi + j0], cmulc(lik, l0));
            if (j1 <= i) R[bi + j1] = csub(R[bi + j1], cmulc(lik, l1));
            bi += i + 1;
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

// x <- (R R^H)^{-1} x with packed lower R and dinv = 1 / diag(R)
template <int NB>
__device__ void s_chol_solve(const cfloat* R, const float* dinv, int n, cfloat (&x)[NB], int lane) {
    int base[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) base[q] = tri(lane + 32 * q);
    for (int k = 0; k < n; ++k) {
        const float dk = dinv[k];
#pragma unroll
        for (int q = 0; q < NB; ++q)
            if (lane + 32 * q == k) x[q] = cscale(x[q], dk);
        const cfloat yk = s_bcast<NB>(x, k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i > k && i < n) x[q] = csub(x[q], cmul(R[base[q] + k], yk));
        }
    }
    for (int k = n - 1; k >= 0; --k) {
        const float dk = dinv[k];
#pragma unroll
        for (int q = 0; q < NB; ++q)
            if (lane + 32 * q == k) x[q] = cscale(x[q], dk);
        const cfloat xk = s_bcast<NB>(x, k);
        const int bk = tri(k);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int i = lane + 32 * q;
            if (i < k) x[q] = csub(x[q], cmul(cconj(R[bk + i]), xk));
        }
    }
}

// LU with partial pivoting (getrf: first maximum of |re| + |im|) on a full n x n
// matrix (ld = n); piv[k] = pivot row of step k.
__device__ inline void s_lu(cfloat* A, int n, int* piv, int lane) {
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
    // |c|: the correctly rounded square root where the zero-correlation threshold
    // compares it, the approximate one (relative error below 2^-22) otherwise
    const float m2 = c.re * c.re + c.im * c.im;
    float g;
    if (a.zct > 0.f) g = sqrtf(m2);
    else asm("sqrt.approx.f32 %0, %1;" : "=f"(g) : "f"(m2));
    if (a.beta_on) g = fadd(fmul(a.one_minus_beta, g), diag ? a.beta : 0.f);
    return g < a.zct ? 0.f : g;
}

// y = H x for Hermitian H in packed lower storage; x published in vpub
template <int NB>
__device__ void s_hermv(const cfloat* H, int n, const cfloat* vpub, cfloat (&y)[NB], int lane) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        cfloat acc = cmake(0.f, 0.f);
        if (i < n) {
            const int bi = tri(i);
            for (int j = 0; j <= i; ++j) acc = cadd(acc, cmul(H[bi + j], vpub[j]));
            for (int j = i + 1; j < n; ++j) acc = cadd(acc, cmul(cconj(H[tri(j) + i]), vpub[j]));
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

// Normalising iteration x <- op(v) / |op(v)| until |x - v| <= 1e-5 or 49 steps; true
// if the stopping rule was met.
template <int NB, class Op>
__device__ bool s_iterate(cfloat (&v)[NB], Op&& op) {
    float diff = 1.f;
    for (int it = 1; diff > 1e-5f && it < 50; ++it) {
        cfloat x[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) x[q] = v[q];
        op(x);
        const float nrm = sqrtf(s_norm2<NB>(x));
        const float inv = 1.f / nrm;
        float dd = 0.f;
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            x[q] = cscale(x[q], inv);
            dd += cabs2(csub(x[q], v[q]));
            v[q] = x[q];
        }
        diff = sqrtf(warp_sum(dd));
    }
    return !(diff > 1e-5f);  // a NaN difference ends the loop too, as in the reference
}

// Full solve for one pixel whose packed coherence matrix is in m.C.  With kLU the
// EMI step uses LU with partial pivoting; otherwise a pixel whose shifted matrix is
// not positive definite is appended to a.fb_list and left for the LU pass.
template <int NB, bool kLU>
__device__ void solve_pixel(const PixArgs& a, int64_t p, const SolveMats& m, int lane) {
    const int n = a.n, ld = m.ldg;
    cfloat* C = m.C;
    float* G = m.G;
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
    // |Gamma| + 1e-6 I (full) -> |Gamma|^{-1}
    for (int i = 0; i < n; ++i)
        for (int j = lane; j < n; j += 32) {
            const int r = j <= i ? i : j, c = j <= i ? j : i;
            G[i * ld + j] = fadd(s_gamma(a, C[pk(r, c)], i == j), i == j ? 1e-6f : 0.f);
        }
    bool inv_nan;
    if (s_gauss_jordan_spd<NB>(G, n, ld, lane)) {
        bool bad = false;
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) bad |= isnan(G[i * ld + j]);
        inv_nan = warp_any(bad);
    } else {
        __syncwarp();
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) G[i * ld + j] = nanf("");
        inv_nan = true;
    }
    __syncwarp();
    const bool evd = a.use_evd || inv_nan;

    cfloat v[NB];
    const float inv_sqrt_n = 1.f / sqrtf((float)n);
#pragma unroll
    for (int q = 0; q < NB; ++q) v[q] = lane + 32 * q < n ? cmake(inv_sqrt_n, 0.f) : cmake(0.f, 0.f);
    float lambda;
    bool converged;
    if (!evd) {
        if (!kLU) {
            // packed A - 0.99 I, complex Cholesky, inverse iteration
            for (int i = 0; i < n; ++i)
                for (int j = lane; j <= i; j += 32) {
                    cfloat x = cscale(C[pk(i, j)], G[i * ld + j]);
                    if (i == j) x.re = fsub(x.re, 0.99f);
                    m.R[pk(i, j)] = x;
                }
            __syncwarp();
            if (!s_chol_complex(m.R, m.d, n, lane)) {
                if (lane == 0) a.fb_list[atomicAdd(a.fb_count, 1)] = (int)p;
                __syncwarp();
                return;
            }
            converged = s_iterate<NB>(v, [&](cfloat(&x)[NB]) { s_chol_solve<NB>(m.R, m.d, n, x, lane); });
            s_publish<NB>(m.v, v, n, lane);
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                const int i = lane + 32 * q;
                if (i < n) {
                    cfloat acc = cmake(0.f, 0.f);  // (R^H v)_i = sum_{k >= i} conj(R_ki) v_k
                    for (int k = i; k < n; ++k) acc = cadd(acc, cmulc(m.v[k], m.R[pk(k, i)]));
                    s += cabs2(acc);
                }
            }
            lambda = fadd(warp_sum(s), fmul(0.99f, s_norm2<NB>(v)));
        } else {
            // LU with partial pivoting on the full shifted matrix
            cfloat* A = m.R;
            for (int i = 0; i < n; ++i)
                for (int j = lane; j < n; j += 32) {
                    cfloat x = cscale(cget(C, i, j), G[i * ld + j]);
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
            converged = s_iterate<NB>(v, [&](cfloat(&x)[NB]) { s_lu_solve<NB>(A, n, src, x, lane); });
            s_publish<NB>(m.v, v, n, lane);
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                const int i = lane + 32 * q;
                if (i < n) {
                    cfloat acc = cmake(0.f, 0.f);
                    for (int j = 0; j < n; ++j) acc = cadd(acc, cmul(cscale(cget(C, i, j), G[i * ld + j]), m.v[j]));
                    s += v[q].re * acc.re + v[q].im * acc.im;
                }
            }
            lambda = warp_sum(s);
        }
        const float scale = sqrtf((float)n) / sqrtf(s_norm2<NB>(v));
#pragma unroll
        for (int q = 0; q < NB; ++q) v[q] = cscale(v[q], scale);
    } else {
        const int T = tri(n);
        for (int e = lane; e < T; e += 32) {
            const cfloat c = C[e];
            m.R[e] = cscale(c, sqrtf(c.re * c.re + c.im * c.im));
        }
        __syncwarp();
        converged = s_iterate<NB>(v, [&](cfloat(&x)[NB]) {
            s_publish<NB>(m.v, x, n, lane);
            s_hermv<NB>(m.R, n, m.v, x, lane);
        });
        s_publish<NB>(m.v, v, n, lane);
        cfloat y[NB];
        s_hermv<NB>(m.R, n, m.v, y, lane);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < NB; ++q) s += v[q].re * y[q].re + v[q].im * y[q].im;
        lambda = warp_sum(s);
    }
    __syncwarp();
    // CRLB: FIM in place of |Gamma|^{-1} (row/col `ref` -> identity), Gauss-Jordan
    if (a.compute_crlb) {
        const int ref = a.crlb_ref;
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) {
                float f;
                if (i == ref || j == ref) {
                    f = i == j ? 1.f : 0.f;
                } else {
                    const int r = j <= i ? i : j, c = j <= i ? j : i;
                    const float x = fmul(a.crlb_factor,
                                         fsub(fmul(s_gamma(a, C[pk(r, c)], i == j), G[i * ld + j]), i == j ? 1.f : 0.f));
                    f = i == j ? fadd(x, 1e-6f) : x;
                }
                G[i * ld + j] = f;
            }
        const bool ok = s_gauss_jordan_spd<NB>(G, n, ld, lane);
        for (int t = lane; t < n; t += 32) a.crlb[p * n + t] = t == ref ? 0.f : (ok ? sqrtf(G[t * ld + t]) : nanf(""));
        __syncwarp();
    } else {
        for (int t = lane; t < n; t += 32) a.crlb[p * n + t] = 0.f;
    }
    // reference to reference_idx
    const cfloat rot = cconj(fphasor(s_bcast<NB>(v, a.ref_idx)));
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int i = lane + 32 * q;
        v[q] = cmul(v[q], rot);
        if (i < n) a.vout[p * n + i] = v[q];
    }
    if (lane == 0) {
        a.eig[p] = lambda;
        a.est[p] = evd ? 0 : 1;
        // the stopping rule not met within 49 steps: listed for the dense eigensolver
        if (!converged && a.nc_list) a.nc_list[atomicAdd(a.nc_count, 1)] = (int)p;
    }
    // temporal coherence over pairs i < j: phasor(C_ij) conj(phasor(v_i conj v_j)),
    // with C_ij = conj(C_ji) (packed (j, i)) and phasor(v_i conj v_j) = w_i conj(w_j)
    cfloat w[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) w[q] = fphasor(v[q]);
    s_publish<NB>(m.v, w, n, lane);
    float sre = 0.f, sim = 0.f;
    int cnt = 0;
    for (int r = 1; r < n; ++r) {
        const cfloat wr = m.v[r];
        const int br = tri(r);
        for (int c = lane; c < r; c += 32) {
            const cfloat u = fphasor(C[br + c]);                   // phasor of C_rc = conj phasor of C_cr
            const cfloat t = cconj(cmulc(cmul(u, m.v[c]), wr));   // conj(u_rc w_c conj(w_r))
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
        const float tc = hypotf(sre / fc, sim / fc);
        a.tcoh[p] = isfinite(tc) ? tc : 0.f;
    }
    __syncwarp();
}

}  // namespace dpl
