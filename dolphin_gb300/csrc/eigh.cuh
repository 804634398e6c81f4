// Non-convergence fallback: a dense Hermitian eigensolver for the pixels whose eigen-
// iteration missed its stopping rule.
//
// The reference iterates at most 49 times and returns the last iterate, with no flag
// (phase_link/_eigenvalues.py:194-202).  Where the two eigenvalues nearest the target
// are close, that iterate is still a mix of their eigenvectors.  Here such pixels are
// listed by the solvers and solved again, one warp per pixel:
//   EMI: |Gamma| (+ beta I, zero threshold) + 1e-6 I is inverted in double precision
//        (the symmetric sweep operator on its lower triangle), A = |Gamma|^{-1} o C,
//        and the eigenvector is the one whose eigenvalue is nearest the inverse
//        iteration's shift 0.99 (the vector that iteration converges to), scaled to
//        norm sqrt(N) (_core.py:486-490).
//   EVD: A = C o |C|; the eigenvector of the eigenvalue of largest magnitude (the one
//        power iteration converges to), unit norm.
// Only one eigenpair is wanted, so the solver is the one LAPACK's subset drivers use
// (Golub & Van Loan, Matrix Computations, sections 8.3-8.4): Householder reduction of A
// to a real symmetric tridiagonal T = Q^H A Q, the wanted eigenvalue of T by Sturm-
// sequence multisection (32 shifts per round, one per lane), its eigenvector by inverse
// iteration on T - lambda I (Gaussian elimination with partial pivoting), and Q applied
// to it.  It runs in float32 on the float32 A.  The pixel is then referenced and its
// temporal coherence recomputed as in the solvers, and flagged.
#pragma once

namespace dpl {

constexpr int kEighMaxN = 64;

// Shared-memory layout of one warp's pixel: C and A (n x ld complex, ld odd; the double
// |Gamma| work matrix shares A's storage, element for element, until A is formed), two
// n-long double work columns and the per-pixel vectors.
struct EighLayout {
    int ld;
    size_t off_C, off_A, off_col, off_w, off_vec, bytes;
};

// the float vectors of one pixel, each kEighMaxN long
struct EighVec {
    cfloat* w;    // phasors of the result / work
    cfloat* pw;   // p = A v, then w, of the current Householder step
    cfloat* tau;  // Householder scalars
    float* d;     // diagonal of T
    float* e;     // off-diagonal of T
    float* e2;    // its squares
    float* u0;    // elimination rows of T - lambda I
    float* u1;
    float* u2;
    float* r;     // right-hand side, then the eigenvector of T
};

inline EighLayout make_eigh_layout(int n) {
    EighLayout L{};
    L.ld = n | 1;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align_up(o + bytes, 16);
        return at;
    };
    L.off_C = take((size_t)n * L.ld * sizeof(cfloat));
    L.off_A = take((size_t)n * L.ld * sizeof(cfloat));
    L.off_col = take(2 * kEighMaxN * sizeof(double));
    L.off_w = take(kEighMaxN * sizeof(cfloat));
    L.off_vec = take(kEighMaxN * (2 * sizeof(cfloat) + 7 * sizeof(float)));
    L.bytes = align_up(o, 128);
    return L;
}

__device__ inline EighVec eigh_vectors(unsigned char* smem, const EighLayout& L) {
    EighVec v;
    v.w = reinterpret_cast<cfloat*>(smem + L.off_w);
    v.pw = reinterpret_cast<cfloat*>(smem + L.off_vec);
    v.tau = v.pw + kEighMaxN;
    float* f = reinterpret_cast<float*>(v.tau + kEighMaxN);
    v.d = f;
    v.e = f + kEighMaxN;
    v.e2 = f + 2 * kEighMaxN;
    v.u0 = f + 3 * kEighMaxN;
    v.u1 = f + 4 * kEighMaxN;
    v.u2 = f + 5 * kEighMaxN;
    v.r = f + 6 * kEighMaxN;
    return v;
}

// Lane's next element (i, j), j <= i, of a lower triangle walked row by row in steps of
// 32 elements.
__device__ __forceinline__ void tri_step(int& i, int& j, int step) {
    j += step;
    while (j > i) {
        j -= i + 1;
        ++i;
    }
}

// In-place inverse of the symmetric positive definite n x n double matrix G (row stride
// ld; lower triangle read and written) by the sweep operator: sweeping pivot k maps
// g_kk -> -1/g_kk, g_ik -> g_ik/g_kk, g_ij -> g_ij - g_ik g_kj / g_kk; after all n pivots
// G holds -G^{-1}, negated at the end.  col and cinv are n-long double work vectors
// (column k, and column k / g_kk, so that each update is one fused multiply-add on the
// narrow FP64 pipe).  False on a non-positive pivot (not positive definite).
__device__ inline bool e_inverse_spd(double* G, int ld, double* col, double* cinv, int n, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        const double piv = G[k * ld + k];
        if (!(piv > 0.0)) return false;
        const double inv = 1.0 / piv;
        for (int i = lane; i < n; i += 32) {
            const double c = i >= k ? G[i * ld + k] : G[k * ld + i];
            col[i] = c;
            cinv[i] = c * inv;
        }
        __syncwarp();
        int i = 0, j = lane;
        tri_step(i, j, 0);
        for (; i < n; tri_step(i, j, 32))
            if (i != k && j != k) G[i * ld + j] = fma(-col[i], cinv[j], G[i * ld + j]);
        __syncwarp();
        for (int t = lane; t < n; t += 32) {
            if (t == k) continue;
            if (t > k) G[t * ld + k] = cinv[t];
            else G[k * ld + t] = cinv[t];
        }
        if (lane == 0) G[k * ld + k] = -inv;
    }
    __syncwarp();
    int i = 0, j = lane;
    tri_step(i, j, 0);
    for (; i < n; tri_step(i, j, 32)) G[i * ld + j] = -G[i * ld + j];
    __syncwarp();
    return true;
}

// Householder reduction of the Hermitian A (n x ld; the lower triangle is read and
// updated) to the real symmetric tridiagonal T (V.d, V.e), A = Q T Q^H with
// Q = H_0 ... H_{n-2}, H_k = I - tau_k u_k u_k^H acting on rows k+1..n-1, u_k = (1, v)
// with v kept in column k below the subdiagonal.  Each H_k^H maps column k's part below
// the diagonal, x, to (beta, 0, ...): beta = -sign(Re x_0) ||x||, tau = (beta - x_0) /
// beta, v = x_{1:} / (x_0 - beta), and with p = A22 u, s = u^H p, w = tau p -
// |tau|^2 s u / 2 the trailing block becomes A22 - w u^H - u w^H.
__device__ inline void e_tridiag(cfloat* A, int n, int ld, const EighVec& V, int lane) {
    for (int k = 0; k + 1 < n; ++k) {
        __syncwarp();
        const cfloat alpha = A[(k + 1) * ld + k];
        float xn2 = 0.f;
        for (int i = k + 2 + lane; i < n; i += 32) xn2 += cabs2(A[i * ld + k]);
        xn2 = warp_sum(xn2);  // butterfly: the same value on every lane
        if (xn2 == 0.f && alpha.im == 0.f) {
            if (lane == 0) {
                V.tau[k] = cmake(0.f, 0.f);
                V.e[k] = alpha.re;
            }
            continue;
        }
        const float beta = -copysignf(sqrtf(alpha.re * alpha.re + alpha.im * alpha.im + xn2), alpha.re);
        const cfloat tau = cmake((beta - alpha.re) / beta, -alpha.im / beta);
        const cfloat den = cmake(alpha.re - beta, alpha.im);
        const float dd = 1.f / cabs2(den);
        const cfloat scal = cmake(den.re * dd, -den.im * dd);  // 1 / (x_0 - beta)
        for (int i = k + 2 + lane; i < n; i += 32) A[i * ld + k] = cmul(A[i * ld + k], scal);
        if (lane == 0) {
            V.tau[k] = tau;
            V.e[k] = beta;
        }
        __syncwarp();
        // p = A22 u from the lower triangle, s = u^H p
        float s = 0.f;
        // element (i, j) of the Hermitian A22 from the lower triangle
        auto a22 = [&](int i, int j) {
            cfloat x = j <= i ? A[i * ld + j] : A[j * ld + i];
            if (j > i) x.im = -x.im;
            return x;
        };
        for (int i = k + 1 + lane; i < n; i += 32) {
            cfloat acc = A[i * ld + k + 1];  // u_{k+1} = 1
            if (i == k + 1) acc.im = 0.f;
            cfloat acc2 = cmake(0.f, 0.f);  // two chains
            int j = k + 2;
            for (; j + 1 < n; j += 2) {
                acc = cfma(acc, a22(i, j), A[j * ld + k]);
                acc2 = cfma(acc2, a22(i, j + 1), A[(j + 1) * ld + k]);
            }
            if (j < n) acc = cfma(acc, a22(i, j), A[j * ld + k]);
            acc = cadd(acc, acc2);
            const cfloat vi = i == k + 1 ? cmake(1.f, 0.f) : A[i * ld + k];
            s += vi.re * acc.re + vi.im * acc.im;
            V.pw[i] = acc;
        }
        s = warp_sum(s);
        const float h = 0.5f * cabs2(tau) * s;
        for (int i = k + 1 + lane; i < n; i += 32) {
            const cfloat vi = i == k + 1 ? cmake(1.f, 0.f) : A[i * ld + k];
            const cfloat pi = V.pw[i];
            V.pw[i] = cmake(tau.re * pi.re - tau.im * pi.im - h * vi.re, tau.re * pi.im + tau.im * pi.re - h * vi.im);
        }
        __syncwarp();
        // A22 -= w u^H + u w^H on the lower triangle (i, j relative to k + 1)
        const int m = n - k - 1, o = k + 1;
        int i = 0, j = lane;
        tri_step(i, j, 0);
#pragma unroll 2
        for (; i < m; tri_step(i, j, 32)) {
            const cfloat wi = V.pw[o + i], wj = V.pw[o + j];
            const cfloat vi = i == 0 ? cmake(1.f, 0.f) : A[(o + i) * ld + k];
            const cfloat vj = j == 0 ? cmake(1.f, 0.f) : A[(o + j) * ld + k];
            cfloat& x = A[(o + i) * ld + o + j];
            x = csub(x, cadd(cmulc(wi, vj), cmulc(vi, wj)));  // w_i conj(v_j) + v_i conj(w_j)
        }
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
        V.d[i] = A[i * ld + i].re;
        if (i + 1 < n) V.e2[i] = V.e[i] * V.e[i];
    }
    __syncwarp();
}

// Number of eigenvalues of T below x (Sturm sequence of the LDL^T pivots).
__device__ __forceinline__ int e_sturm(const float* d, const float* e2, int n, float x, float pivmin) {
    float q = d[0] - x;
    if (fabsf(q) < pivmin) q = -pivmin;
    int c = q < 0.f;
    for (int i = 1; i < n; ++i) {
        q = (d[i] - x) - __fdividef(e2[i - 1], q);
        if (fabsf(q) < pivmin) q = -pivmin;
        c += q < 0.f;
    }
    return c;
}

// The k-th smallest eigenvalue of T (k from 0): each round splits [lo, hi) into 33
// parts at the lanes' shifts and keeps the part that holds it.
__device__ inline float e_kth(const float* d, const float* e2, int n, int k, float lo, float hi, float pivmin,
                              int lane) {
    for (int it = 0; it < 12; ++it) {
        if (!(hi - lo > 2.4e-7f * fmaxf(fabsf(lo), fabsf(hi)) + pivmin)) break;
        const float x = lo + (hi - lo) * ((float)(lane + 1) * (1.f / 33.f));
        const unsigned above = __ballot_sync(0xffffffffu, e_sturm(d, e2, n, x, pivmin) > k);
        const int jx = above ? __ffs(above) - 1 : 32;
        const float xl = __shfl_sync(0xffffffffu, x, jx > 0 ? jx - 1 : 0);
        const float xh = __shfl_sync(0xffffffffu, x, jx < 32 ? jx : 31);
        if (jx > 0) lo = xl;
        if (jx < 32) hi = xh;
    }
    return 0.5f * (lo + hi);
}

// Eigenvector of T for the eigenvalue lam by three steps of inverse iteration (one lane):
// (T - lam I) y = b by Gaussian elimination with partial pivoting, pivots below tiny
// replaced by tiny.  The result, scaled to a largest entry of 1, is left in V.r.
__device__ inline void e_inverse_iteration(const EighVec& V, int n, float lam, float tiny) {
    const float* d = V.d;
    const float* e = V.e;
    float* r = V.r;
    for (int i = 0; i < n; ++i) r[i] = 1.f + 0.1f * (float)((7 * i) % 5);
    for (int step = 0; step < 3; ++step) {
        float p0 = d[0] - lam, p1 = n > 1 ? e[0] : 0.f, p2 = 0.f, rr = r[0];
        for (int i = 0; i + 1 < n; ++i) {
            const float q0 = e[i], q1 = d[i + 1] - lam, q2 = i + 2 < n ? e[i + 1] : 0.f, rq = r[i + 1];
            if (fabsf(p0) >= fabsf(q0)) {
                if (fabsf(p0) < tiny) p0 = p0 < 0.f ? -tiny : tiny;
                const float m = q0 / p0;
                V.u0[i] = p0, V.u1[i] = p1, V.u2[i] = p2, r[i] = rr;
                p0 = q1 - m * p1, p1 = q2 - m * p2, p2 = 0.f, rr = rq - m * rr;
            } else {
                const float m = p0 / q0;
                V.u0[i] = q0, V.u1[i] = q1, V.u2[i] = q2, r[i] = rq;
                p0 = p1 - m * q1, p1 = p2 - m * q2, p2 = 0.f, rr = rr - m * rq;
            }
        }
        if (fabsf(p0) < tiny) p0 = p0 < 0.f ? -tiny : tiny;
        V.u0[n - 1] = p0, r[n - 1] = rr;
        float big = 0.f;
        for (int i = n - 1; i >= 0; --i) {
            float t = r[i];
            if (i + 1 < n) t -= V.u1[i] * r[i + 1];
            if (i + 2 < n) t -= V.u2[i] * r[i + 2];
            r[i] = t / V.u0[i];
            big = fmaxf(big, fabsf(r[i]));
        }
        const float sc = big > 0.f && isfinite(big) ? 1.f / big : 1.f;
        for (int i = 0; i < n; ++i) r[i] *= sc;
    }
}

// The wanted eigenpair of the Hermitian A (n x ld, lower triangle; destroyed): EMI
// (evd false) the eigenvalue nearest 0.99, ties to the smaller; EVD the largest in
// magnitude, ties to the smaller.  Returns lambda; the eigenvector (unnormalised)
// is left in xv.
__device__ inline float e_eigpair(cfloat* A, int n, int ld, bool evd, const EighVec& V, cfloat* xv, int lane) {
    e_tridiag(A, n, ld, V, lane);
    // Gershgorin bounds of T
    float lo = INFINITY, hi = -INFINITY, tn = 0.f, e2max = 0.f;
    for (int i = 0; i < n; ++i) {
        const float rad = (i > 0 ? fabsf(V.e[i - 1]) : 0.f) + (i + 1 < n ? fabsf(V.e[i]) : 0.f);
        lo = fminf(lo, V.d[i] - rad);
        hi = fmaxf(hi, V.d[i] + rad);
        tn = fmaxf(tn, fabsf(V.d[i]) + rad);
        if (i + 1 < n) e2max = fmaxf(e2max, V.e2[i]);
    }
    const float pivmin = 1.18e-38f * fmaxf(1.f, e2max);
    const float pad = 2.4e-7f * (float)n * fmaxf(fabsf(lo), fabsf(hi)) + 2.f * pivmin;
    lo -= pad;
    hi += pad;
    float lam;
    if (evd) {
        const float l0 = e_kth(V.d, V.e2, n, 0, lo, hi, pivmin, lane);
        const float l1 = e_kth(V.d, V.e2, n, n - 1, lo, hi, pivmin, lane);
        lam = fabsf(l1) > fabsf(l0) ? l1 : l0;
    } else {
        const int m = e_sturm(V.d, V.e2, n, 0.99f, pivmin);
        if (m == 0) {
            lam = e_kth(V.d, V.e2, n, 0, lo, hi, pivmin, lane);
        } else if (m == n) {
            lam = e_kth(V.d, V.e2, n, n - 1, lo, hi, pivmin, lane);
        } else {
            const float la = e_kth(V.d, V.e2, n, m - 1, lo, hi, pivmin, lane);
            const float lb = e_kth(V.d, V.e2, n, m, lo, hi, pivmin, lane);
            lam = fabsf(lb - 0.99f) < fabsf(la - 0.99f) ? lb : la;
        }
    }
    if (lane == 0) e_inverse_iteration(V, n, lam, 1.2e-7f * fmaxf(tn, 1.18e-38f));
    __syncwarp();
    // x = Q y = H_0 (H_1 (... H_{n-2} y)), two rows per lane in registers
    cfloat x[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = lane + 32 * h;
        x[h] = cmake(i < n ? V.r[i] : 0.f, 0.f);
    }
    for (int k = n - 2; k >= 0; --k) {
        const cfloat t = V.tau[k];
        if (t.re == 0.f && t.im == 0.f) continue;
        float dre = 0.f, dim = 0.f;  // u^H x
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = lane + 32 * h;
            if (i > k && i < n) {
                const cfloat u = i == k + 1 ? cmake(1.f, 0.f) : A[i * ld + k];
                dre += u.re * x[h].re + u.im * x[h].im;
                dim += u.re * x[h].im - u.im * x[h].re;
            }
        }
        const cfloat dot = cmake(warp_sum(dre), warp_sum(dim));
        const cfloat td = cmul(t, dot);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = lane + 32 * h;
            if (i > k && i < n) {
                const cfloat u = i == k + 1 ? cmake(1.f, 0.f) : A[i * ld + k];
                x[h] = csub(x[h], cmul(u, td));
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = lane + 32 * h;
        if (i < n) xv[i] = x[h];
    }
    __syncwarp();
    return lam;
}

}  // namespace dpl
