// Non-convergence fallback: a dense Hermitian eigensolver for the pixels whose eigen-
// iteration missed its stopping rule.
//
// The reference iterates at most 49 times and returns the last iterate, with no flag
// (phase_link/_eigenvalues.py:194-202).  Where the two eigenvalues nearest the target
// are close, that iterate is still a mix of their eigenvectors.  Here such pixels are
// listed by the solvers and solved again, one warp per pixel:
//   EMI: |Gamma| (+ beta I, zero threshold) + 1e-6 I is inverted in double precision
//        (Gauss-Jordan on the symmetric positive definite matrix), A = |Gamma|^{-1} o C,
//        and the eigenvector is the one whose eigenvalue is nearest the inverse
//        iteration's shift 0.99 (the vector that iteration converges to), scaled to
//        norm sqrt(N) (_core.py:486-490).
//   EVD: A = C o |C|; the eigenvector of the eigenvalue of largest magnitude (the one
//        power iteration converges to), unit norm.
// The eigen-decomposition is the cyclic Jacobi method for Hermitian matrices (Golub &
// Van Loan, Matrix Computations, section 8.5): each rotation removes the phase of the
// pivot element with a diagonal unitary, then applies the real symmetric Jacobi
// rotation; the accumulated rotations give the eigenvectors.  It runs in float32 on
// the float32 A: GB300's FP64 rate (1.04 TFLOP/s measured) would make a double-
// precision Jacobi cost about a millisecond of an SM per pixel.  The pixel is then
// referenced and its temporal coherence recomputed as in the solvers, and flagged.
#pragma once

namespace dpl {

constexpr int kEighMaxSweeps = 30;

// Shared-memory layout of one warp's pixel: C, A and V (n x ld complex, ld odd) and
// the double |Gamma| work matrix (n x n).
struct EighLayout {
    int ld;
    size_t off_C, off_A, off_V, off_G, off_w, bytes;
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
    L.off_V = take((size_t)n * L.ld * sizeof(cfloat));
    L.off_G = take((size_t)n * n * sizeof(double));
    L.off_w = take(64 * sizeof(cfloat));
    L.bytes = align_up(o, 128);
    return L;
}

// In-place inverse of the symmetric positive definite n x n double matrix G by
// Gauss-Jordan elimination (lanes own columns).  False on a non-positive pivot.
__device__ inline bool e_inverse_spd(double* G, int n, int lane) {
    for (int k = 0; k < n; ++k) {
        __syncwarp();
        const double piv = G[k * n + k];
        if (!(piv > 0.0)) return false;
        const double inv = 1.0 / piv;
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            const double f = G[i * n + k] * inv;
            for (int j = lane; j < n; j += 32)
                if (j != k) G[i * n + j] -= f * G[k * n + j];
        }
        __syncwarp();
        for (int j = lane; j < n; j += 32) {
            if (j != k) {
                G[k * n + j] *= inv;
                G[j * n + k] = -G[j * n + k] * inv;
            }
        }
        __syncwarp();
        if (lane == 0) G[k * n + k] = inv;
    }
    __syncwarp();
    return true;
}

// Cyclic Jacobi on the Hermitian A (n x ld, both triangles); V receives the
// eigenvectors as columns.  On return diag(A) holds the eigenvalues.
__device__ inline void e_jacobi(cfloat* A, cfloat* V, int n, int ld, int lane) {
    for (int i = 0; i < n; ++i)
        for (int j = lane; j < n; j += 32) V[i * ld + j] = cmake(i == j ? 1.f : 0.f, 0.f);
    __syncwarp();
    for (int sweep = 0; sweep < kEighMaxSweeps; ++sweep) {
        // stop once the off-diagonal part is below float32 resolution of the whole
        float off = 0.f, tot = 0.f;
        for (int i = 0; i < n; ++i)
            for (int j = lane; j < n; j += 32) {
                const float m2 = cabs2(A[i * ld + j]);
                tot += m2;
                if (j != i) off += m2;
            }
        off = warp_sum(off);
        tot = warp_sum(tot);
        if (!(off > 1e-14f * tot)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const cfloat b = A[p * ld + q];
                const float e = sqrtf(cabs2(b));
                if (!(e > 0.f)) continue;  // uniform: every lane reads the same element
                const float a = A[p * ld + p].re, d = A[q * ld + q].re;
                const float zeta = (d - a) / (2.f * e);
                const float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
                const float c = 1.f / sqrtf(1.f + t * t), s = t * c;
                const cfloat ph = cmake(b.re / e, b.im / e);     // e^{i phi}
                const cfloat sm = cmake(s * ph.re, -s * ph.im);  // s e^{-i phi}
                const cfloat cm = cmake(c * ph.re, -c * ph.im);  // c e^{-i phi}
                __syncwarp();
                // columns p, q of A and V: A <- A J, V <- V J
                for (int k = lane; k < n; k += 32) {
                    const cfloat xp = A[k * ld + p], xq = A[k * ld + q];
                    A[k * ld + p] = csub(cscale(xp, c), cmul(sm, xq));
                    A[k * ld + q] = cadd(cscale(xp, s), cmul(cm, xq));
                    const cfloat vp = V[k * ld + p], vq = V[k * ld + q];
                    V[k * ld + p] = csub(cscale(vp, c), cmul(sm, vq));
                    V[k * ld + q] = cadd(cscale(vp, s), cmul(cm, vq));
                }
                __syncwarp();
                // rows p, q: A <- J^H A
                for (int k = lane; k < n; k += 32) {
                    const cfloat xp = A[p * ld + k], xq = A[q * ld + k];
                    A[p * ld + k] = csub(cscale(xp, c), cmul(cconj(sm), xq));
                    A[q * ld + k] = cadd(cscale(xp, s), cmul(cconj(cm), xq));
                }
                __syncwarp();
                if (lane == 0) {
                    A[p * ld + q] = cmake(0.f, 0.f);
                    A[q * ld + p] = cmake(0.f, 0.f);
                    A[p * ld + p] = cmake(a - t * e, 0.f);
                    A[q * ld + q] = cmake(d + t * e, 0.f);
                }
                __syncwarp();
            }
    }
    __syncwarp();
}

}  // namespace dpl
