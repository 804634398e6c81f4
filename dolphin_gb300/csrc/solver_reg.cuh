// Register-resident per-pixel solver for N <= K: a group of G warps solves one pixel
// (K = 16 or 32 with one warp, K = 64 with two warps); thread i of the group owns row i
// of each matrix in registers.
//
// Same algorithms, iteration rules and outputs as solve_pixel (solver.cuh), laid out
// for the register file instead of shared memory:
//   |Gamma| + 1e-6 I  -> symmetric sweep (Gauss-Jordan in the "sweep" form: after
//        sweeping every index the matrix holds -A^{-1}).  A non-positive pivot is
//        the reference's Cholesky failure (_core.py:466-472, 496-515): EVD fallback.
//   CRLB: the Fisher matrix (crlb.py:132-189) is swept the same way.
//   EMI: A - 0.99 I (A = |Gamma|^{-1} o C) is inverted by the Hermitian sweep, and
//        inverse iteration (_eigenvalues.py:139-205) is a matrix-vector product per
//        step.  The sweep's pivots are those of the Cholesky/LDL^H factorisation, so
//        a non-positive pivot is exactly "not positive definite": such a pixel is
//        listed for the LU pass (the reference's LU algorithm), as in solve_pixel.
//   EVD: power iteration on C o |C| with the rows in registers (_eigenvalues.py:93-136).
//
// Register rotation keeps the sweeps in compact loops: before step k, slot s of a
// row holds column (k + s) mod K, so the pivot column is always slot 0 and each
// update writes slot s - 1 from slot s (the shift costs nothing).  The column is
// broadcast through shared memory at position (row - k) mod K, so slot s reads
// position s.  Rows and columns >= N are zero and stay zero.
#pragma once

namespace dpl {

// Shared memory per pixel group: full Hermitian C (n x ld, ld odd: a thread-per-row
// access of one column is conflict-free), |Gamma| / |Gamma|^{-1} (n x ld floats), a
// 128-entry broadcast buffer, a 64-entry vector buffer and reduction slots.
struct RegLayout {
    int ld;
    size_t off_C, off_G, off_b, off_w, off_x, bytes;
};

inline RegLayout make_reg_layout(int n) {
    RegLayout L{};
    L.ld = n | 1;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align_up(o + bytes, 16);
        return at;
    };
    L.off_C = take((size_t)n * L.ld * sizeof(cfloat));
    L.off_G = take((size_t)n * L.ld * sizeof(float));
    L.off_b = take(128 * sizeof(cfloat));  // the sweeps' two broadcast halves
    L.off_w = take(64 * sizeof(cfloat));
    L.off_x = take(16 * sizeof(float));
    L.bytes = align_up(o, 128);
    return L;
}

// A pixel group of G threads: G = 8, 16 or 32 lanes of one warp (a warp holds 32 / G
// pixels) or G = 64, two whole warps: row index, synchronisation, reductions.
template <int G>
struct Grp {
    int gl;         // thread (= row) index within the group, 0 .. G - 1
    int lane;       // lane within its warp
    int wig;        // warp within the group (G == 64)
    int bar;        // named barrier of the group (G == 64)
    int base;       // first lane of the group in its warp (G <= 32)
    unsigned mask;  // the group's lanes (G <= 32)
    float* x;       // reduction slots (shared memory, 16 floats)

    __device__ __forceinline__ void sync() const {
        if (G <= 32) {
            __syncwarp(mask);
        } else {
            __syncwarp();  // bar.sync counts a warp as arrived when any of its lanes arrives
            asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(64) : "memory");
        }
    }
    // sum over the group, the same value in every thread
    __device__ __forceinline__ float sum(float v) const {
        if (G <= 32) {
#pragma unroll
            for (int o = (G >> 1); o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
            return v;
        }
        v = warp_sum(v);
        if (lane == 0) x[wig] = v;
        sync();
        const float r = x[0] + x[1];
        sync();
        return r;
    }
    __device__ __forceinline__ bool any(bool v) const {
        if (G <= 32) return __any_sync(mask, v);
        v = warp_any(v);
        if (lane == 0) x[2 + wig] = v ? 1.f : 0.f;
        sync();
        const bool r = x[2] + x[3] > 0.f;
        sync();
        return r;
    }
    // value of thread k (uniform k)
    __device__ __forceinline__ cfloat bcast(cfloat v, int k) const {
        if (G <= 32) return {__shfl_sync(mask, v.re, base + k), __shfl_sync(mask, v.im, base + k)};
        if (gl == k) {
            x[4] = v.re;
            x[5] = v.im;
        }
        sync();
        const cfloat r = cmake(x[4], x[5]);
        sync();
        return r;
    }
};

// 1/p to about an ulp: the approximate reciprocal refined by one Newton step.
__device__ __forceinline__ float frcp_nr(float p) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(p));
    return fmaf(r, fmaf(-p, r, 1.f), r);
}

// The sweeps broadcast the pivot column through `buf`, two halves used alternately so
// that one barrier per step suffices: step k writes half k & 1, whose readers (step
// k - 2) all passed step k - 1's barrier before this thread did.  Row `gl` writes its
// pivot-column entry at position (gl - k) mod K, so slot s of every row reads position s.

// Real symmetric sweep over indices 0..n-1 of the matrix whose row `gl` is g; on
// success g holds row `gl` of -A^{-1}.  Returns false (uniformly) if any pivot was
// <= 0 (the remaining steps then run on meaningless values, without branching).
// buf: 2 * ((K + 3) & ~3) floats.
template <int K, int G>
__device__ __forceinline__ bool r_sweep(float (&g)[K], int n, float* buf, const Grp<G>& gr) {
    constexpr int KB = (K + 3) & ~3;  // half stride: 16-byte aligned
    bool bad = false;                 // uniform: every thread reads the same pivot
    int pos = gr.gl;
    gr.sync();  // earlier users of buf are done with it
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        float* bk = buf + (k & 1) * KB;
        if (gr.gl < K) bk[pos] = g[0];  // A[row][k] (= A[k][row])
        gr.sync();
        float r[K];
        const float4* b4 = reinterpret_cast<const float4*>(bk);
#pragma unroll
        for (int q = 0; q < K / 4; ++q) {
            const float4 t = b4[q];
            r[4 * q] = t.x;
            r[4 * q + 1] = t.y;
            r[4 * q + 2] = t.z;
            r[4 * q + 3] = t.w;
        }
        if (K % 4) {  // K = 4m + 2: the last two slots
            const float2 t = reinterpret_cast<const float2*>(bk)[K / 2 - 1];
            r[K - 2] = t.x;
            r[K - 1] = t.y;
        }
        const float p = r[0];
        bad |= !(p > 0.f);
        const float ip = frcp_nr(p);
        const bool me = gr.gl == k;
        // rows i != k: a_ij - (a_ik / p) a_kj; row k: a_kj / p, written as
        // a_kj - (1 - 1/p) a_kj so that every thread runs the same FMA
        const float t = me ? 1.f - ip : g[0] * ip;
        const float last = me ? -ip : g[0] * ip;
#pragma unroll
        for (int s = 0; s < K - 1; ++s) g[s] = fmaf(-t, r[s + 1], g[s + 1]);
        g[K - 1] = last;
        pos = pos == 0 ? K - 1 : pos - 1;
    }
#pragma unroll 1
    for (int k = n; k < K; ++k) {  // finish the rotation: slot s holds column s again
        const float t0 = g[0];
#pragma unroll
        for (int s = 0; s < K - 1; ++s) g[s] = g[s + 1];
        g[K - 1] = t0;
    }
    gr.sync();
    return !bad;
}

// Hermitian sweep: on success a holds row `gl` of -A^{-1}.  False if a pivot was <= 0.
// buf: 2 * K complex.
template <int K, int G>
__device__ __forceinline__ bool r_sweep_c(cfloat (&a)[K], int n, cfloat* buf, const Grp<G>& gr) {
    bool bad = false;  // uniform: every thread reads the same pivot
    int pos = gr.gl;
    gr.sync();
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        cfloat* bk = buf + (k & 1) * K;  // K even: 16-byte aligned halves
        if (gr.gl < K) bk[pos] = a[0];   // A[row][k] = conj(A[k][row])
        gr.sync();
        const float p = bk[0].re;
        bad |= !(p > 0.f);
        const float ip = frcp_nr(p);
        const bool me = gr.gl == k;
        const cfloat t = me ? cmake(1.f - ip, 0.f) : cscale(a[0], ip);
        const cfloat last = me ? cmake(-ip, 0.f) : cscale(a[0], ip);
        const float4* b4 = reinterpret_cast<const float4*>(bk);
#pragma unroll
        for (int q = 0; q < K / 2; ++q) {
            const float4 b = b4[q];
            // slot s: a_ij - t a_kj, a_kj = conj(buffer entry s)
            if (q > 0) a[2 * q - 1] = cfms_conj(a[2 * q], t, cmake(b.x, b.y));
            a[2 * q] = cfms_conj(a[2 * q + 1], t, cmake(b.z, b.w));
        }
        a[K - 1] = last;
        pos = pos == 0 ? K - 1 : pos - 1;
    }
#pragma unroll 1
    for (int k = n; k < K; ++k) {
        const cfloat t0 = a[0];
#pragma unroll
        for (int s = 0; s < K - 1; ++s) a[s] = a[s + 1];
        a[K - 1] = t0;
    }
    gr.sync();
    return !bad;
}

// y_row = sum_j h[j] x_j (row `gl` of a matrix in registers); x published in vb
template <int K, int G>
__device__ __forceinline__ cfloat r_matvec(const cfloat (&h)[K], cfloat x, cfloat* vb, const Grp<G>& gr) {
    gr.sync();
    vb[gr.gl] = x;
    gr.sync();
    const float4* v4 = reinterpret_cast<const float4*>(vb);
    cfloat acc0 = cmake(0.f, 0.f), acc1 = cmake(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < K / 2; ++q) {
        const float4 t = v4[q];
        acc0 = cfma(acc0, h[2 * q], cmake(t.x, t.y));
        acc1 = cfma(acc1, h[2 * q + 1], cmake(t.z, t.w));
    }
    return cadd(acc0, acc1);
}

// Asynchronous copy of one pixel's planar coherence (count floats) into shared memory.
template <int G>
__device__ __forceinline__ void r_prefetch(float* dst, const float* src, int count, const Grp<G>& gr) {
    gr.sync();
    // 4-byte pieces: 16-byte copies measured slower here (the solve is issue-bound and
    // the copy has the whole temporal-coherence pass to land)
    for (int e = gr.gl; e < count; e += G)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst + e)),
                     "l"(src + e)
                     : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Normalising iteration x <- op(v) / |op(v)| until |x - v| <= 1e-5 or 49 steps
// (the reference's while-loop: iteration count starts at 1, stops below 50).  Adds the
// steps taken to `steps`; returns the last step's difference (NaN also ends the loop).
template <int G, class Op>
__device__ __forceinline__ float r_iterate(cfloat& v, const Grp<G>& gr, int& steps, Op&& op) {
    float diff = 1.f;
    for (int it = 1; diff > 1e-5f && it < 50; ++it) {
        cfloat x = op(v);
        const float inv = rsqrtf(gr.sum(cabs2(x)));
        x = cscale(x, inv);
        diff = sqrtf(gr.sum(cabs2(csub(x, v))));
        v = x;
        ++steps;
    }
    return diff;
}

// Full solve for one pixel whose Hermitian coherence matrix is in Cf (n x ld, both
// triangles).  A pixel whose shifted EMI matrix is not positive definite is appended
// to a.fb_list and left for the LU pass.  Once Gs is no longer needed, the planar
// coherence of the group's next pixel (`next`, if any) is prefetched into it.
template <int K, int G>
__device__ void solve_pixel_reg(const PixArgs& a, int64_t p, const cfloat* Cf, float* Gs, int ld, cfloat* cb,
                                cfloat* wb, const uint32_t* ptab, const float* next, const Grp<G>& gr) {
    const int n = a.n, me = gr.gl;
    const bool row = me < n;
    const cfloat* Ci = Cf + (row ? me : 0) * ld;
    if (a.closure && me < n - 2) {
        const cfloat c = cmulc(cmul(Cf[me * ld + me + 1], Cf[(me + 1) * ld + me + 2]), Cf[me * ld + me + 2]);
        a.closure[p * (n - 2) + me] = atan2f(c.im, c.re);
    }
    // |Gamma| + 1e-6 I -> -|Gamma|^{-1} (round 0), then the CRLB's Fisher matrix
    // FIM = 2L (Gamma o Gamma^{-1} - I), row/col `ref` -> identity, + 1e-6 I (round 1).
    // Gs holds |Gamma| during round 0 and |Gamma|^{-1} afterwards.
    float* Gi = Gs + (row ? me : 0) * ld;
    const int ref = a.crlb_ref;
    bool inv_nan = true;
    bool crlb_ok = false;
    float dg = 0.f;
    if (!(a.use_evd && !a.compute_crlb)) {
        // |Gamma| + 1e-6 I into shared memory by lower pairs (every thread busy), the
        // diagonal of |Gamma| itself kept in gdiag, then into the register slots
        const int nr = row ? n : 0;  // this row's live columns
        const int npairs = n * (n - 1) / 2;
        for (int e = me; e < npairs; e += G) {
            const uint32_t rc = ptab[e];
            const int r = rc & 0xffff, c = rc >> 16;
            const float gm = s_gamma(a, Cf[r * ld + c], false);
            Gs[r * ld + c] = gm;
            Gs[c * ld + r] = gm;
        }
        float gdiag = 0.f;
        if (row) {
            gdiag = s_gamma(a, Ci[me], true);
            Gi[me] = fadd(gdiag, 1e-6f);
        }
        gr.sync();
        float g[K];
#pragma unroll
        for (int j = 0; j < K; ++j) g[j] = j < nr ? Gi[j] : 0.f;
#pragma unroll 1
        for (int round = 0; round < 2; ++round) {
            const bool ok = r_sweep<K, G>(g, n, reinterpret_cast<float*>(cb), gr);
            if (round == 1) {
                crlb_ok = ok;
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if (j == me) dg = g[j];
                break;
            }
            inv_nan = !ok;
            if (ok) {
                bool bad = false;
#pragma unroll
                for (int j = 0; j < K; ++j) bad |= isnan(g[j]);
                inv_nan = gr.any(bad);
            }
            // keep |Gamma|^{-1} and build the FIM in place of it
            const bool refrow = me == ref;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const float ginv = -g[j];
                float x = 0.f;
                if (j < nr) {
                    const bool dj = j == me;
                    x = fmul(a.crlb_factor, fsub(fmul(dj ? gdiag : Gi[j], ginv), dj ? 1.f : 0.f));
                    if (dj) x = fadd(x, 1e-6f);
                    if (refrow || j == ref) x = dj ? 1.f : 0.f;
                    Gi[j] = ginv;
                }
                g[j] = x;
            }
            if (!a.compute_crlb || inv_nan) break;
        }
    }
    const bool evd = a.use_evd || inv_nan;
    if (row) a.crlb[p * n + me] = !a.compute_crlb || me == ref ? 0.f : (crlb_ok ? sqrtf(-dg) : nanf(""));

    cfloat v = row ? cmake(1.f / sqrtf((float)n), 0.f) : cmake(0.f, 0.f);
    float lambda;
    int steps = 0;
    // one matrix slot array and one iteration for both estimators: EMI iterates with
    // -(A - 0.99 I)^{-1} (the negated sweep result), EVD with C o |C|
    cfloat mat[K];
    if (!evd) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            cfloat x = cmake(0.f, 0.f);
            if (row && j < n) {
                x = cscale(Ci[j], Gi[j]);
                if (j == me) x.re = fsub(x.re, 0.99f);
            }
            mat[j] = x;
        }
        if (!r_sweep_c<K, G>(mat, n, cb, gr)) {
            if (me == 0) a.fb_list[atomicAdd(a.fb_count, 1)] = (int)p;
            if (next) r_prefetch<G>(Gs, next, n * n, gr);
            gr.sync();
            return;
        }
    } else {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            cfloat x = cmake(0.f, 0.f);
            if (row && j < n) {
                const cfloat c = Ci[j];
                x = cscale(c, sqrtf(c.re * c.re + c.im * c.im));
            }
            mat[j] = x;
        }
    }
    const float sgn = evd ? 1.f : -1.f;
    auto op = [&](cfloat x) { return cscale(r_matvec<K, G>(mat, x, wb, gr), sgn); };
    bool warm = false;
    if (a.vstart && !evd) {
        // learned starting vector; plain EMI (constant start) if it is unusable or the
        // iteration from it does not meet the stopping rule
        const cfloat w0 = row ? a.vstart[p * n + me] : cmake(0.f, 0.f);
        const float w2 = gr.sum(cabs2(w0));
        if (w2 > 0.f && w2 <= 3.4e38f) {
            v = cscale(w0, 1.f / sqrtf(w2));
            warm = true;
        }
    }
    float diff = r_iterate<G>(v, gr, steps, op);
    if (!(diff <= 1e-5f) && warm) {  // a warm start that misses the rule (or goes NaN): plain EMI
        v = row ? cmake(1.f / sqrtf((float)n), 0.f) : cmake(0.f, 0.f);
        diff = r_iterate<G>(v, gr, steps, op);
    }
    // 49 steps without meeting the stopping rule (a NaN difference stops the loop, as in
    // the reference): listed for the dense eigensolver
    if (diff > 1e-5f && a.nc_list && me == 0) a.nc_list[atomicAdd(a.nc_count, 1)] = (int)p;
    if (!evd) {
        // lambda = Re v^H A v, A_ij = |Gamma|^{-1}_ij C_ij
        gr.sync();
        wb[me] = v;
        gr.sync();
        cfloat acc = cmake(0.f, 0.f);
        if (row) {
            for (int j = 0; j < n; ++j) acc = cfma(acc, cscale(Ci[j], Gi[j]), wb[j]);
        }
        if (next) r_prefetch<G>(Gs, next, n * n, gr);
        const float n2 = gr.sum(cabs2(v));
        lambda = gr.sum(v.re * acc.re + v.im * acc.im);
        v = cscale(v, sqrtf((float)n) / sqrtf(n2));
    } else {
        if (next) r_prefetch<G>(Gs, next, n * n, gr);
        const cfloat y = op(v);
        lambda = gr.sum(v.re * y.re + v.im * y.im);
    }
    // reference to reference_idx
    const cfloat rot = cconj(fphasor(gr.bcast(v, a.ref_idx)));
    v = cmul(v, rot);
    if (row) a.vout[p * n + me] = v;
    if (me == 0) {
        a.eig[p] = lambda;
        a.est[p] = evd ? 0 : 1;
        if (a.iters) a.iters[p] = (int16_t)steps;
    }
    // temporal coherence over pairs c < r (ptab: the lower pairs r | c << 16, row by
    // row): conj(phasor(C_rc) w_c conj(w_r))
    gr.sync();
    wb[me] = fphasor(v);
    gr.sync();
    float sre = 0.f, sim = 0.f, cnt = 0.f;
    const int npairs = n * (n - 1) / 2;
#pragma unroll 2
    for (int e = me; e < npairs; e += G) {
        const uint32_t rc = ptab[e];
        const int r = rc & 0xffff, c = rc >> 16;
        const cfloat u = fphasor(Cf[r * ld + c]);
        const cfloat t = cconj(cmulc(cmul(u, wb[c]), wb[r]));
        if (!cisnan(t)) {
            sre += t.re;
            sim += t.im;
            cnt += 1.f;
        }
    }
    sre = gr.sum(sre);
    sim = gr.sum(sim);
    cnt = gr.sum(cnt);  // exact: at most 2016 pairs
    if (me == 0) {
        const float tc = hypotf(sre / cnt, sim / cnt);
        a.tcoh[p] = isfinite(tc) ? tc : 0.f;
    }
    gr.sync();
}

// Solve-only pass over all pixels with the register solver (n <= K), one pixel per
// group of G warps.  The coherence comes planar (diagonal, then (Re, Im) of the
// lower pair (i, j), i > j, at o = i(i-1)/2 + j) or as full (npix, n, n) matrices
// of which the lower triangle is read.
// Two CTAs per SM (128 registers) wherever two CTAs' shared memory fits, K <= 46: the
// two-warp instances would take 150-250 registers and one CTA; bounded, K <= 46 compiles
// without spills and runs 14-16 % faster at N = 36-45.
template <int K, int G>
__global__ void __launch_bounds__(256, (G == 64 && K > 46) ? 1 : 2) k_solve_reg(PixArgs a, RegLayout L) {
    extern __shared__ __align__(16) unsigned char reg_smem[];
    const int warp = threadIdx.x >> 5;
    Grp<G> gr;
    gr.lane = threadIdx.x & 31;
    int group, ngroups;
    if (G <= 32) {
        constexpr int per_warp = 32 / (G <= 32 ? G : 32);
        ngroups = (blockDim.x >> 5) * per_warp;
        group = warp * per_warp + gr.lane / G;
        gr.base = gr.lane & ~(G - 1);
        gr.mask = G == 32 ? 0xffffffffu : ((1u << (G & 31)) - 1u) << gr.base;
        gr.wig = 0;
        gr.gl = gr.lane - gr.base;
        gr.bar = 0;
    } else {
        ngroups = (blockDim.x >> 5) / 2;
        group = warp / 2;
        gr.base = 0;
        gr.mask = 0xffffffffu;
        gr.wig = warp - group * 2;
        gr.gl = gr.wig * 32 + gr.lane;
        gr.bar = 1 + group;
    }
    unsigned char* base = reg_smem + group * L.bytes;
    gr.x = reinterpret_cast<float*>(base + L.off_x);
    cfloat* Cf = reinterpret_cast<cfloat*>(base + L.off_C);
    float* Gs = reinterpret_cast<float*>(base + L.off_G);
    cfloat* cb = reinterpret_cast<cfloat*>(base + L.off_b);
    cfloat* wb = reinterpret_cast<cfloat*>(base + L.off_w);
    uint32_t* ptab = reinterpret_cast<uint32_t*>(reg_smem + ngroups * L.bytes);  // shared by the CTA
    const int n = a.n, ld = L.ld, lag = a.baseline_lag, me = gr.gl;
    for (int o = threadIdx.x; o < n * (n - 1) / 2; o += blockDim.x) {
        int r = (int)((sqrtf(8.f * o + 1.f) + 1.f) * 0.5f);  // o = r(r-1)/2 + c, 0 <= c < r
        while (r * (r - 1) / 2 > o) --r;
        while ((r + 1) * r / 2 <= o) ++r;
        ptab[o] = (uint32_t)r | ((uint32_t)(o - r * (r - 1) / 2) << 16);
    }
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * ngroups;
    bool staged = false;  // Gs holds this pixel's planar coherence (prefetched)
    for (int64_t p = (int64_t)blockIdx.x * ngroups + group; p < a.npix; p += stride) {
        gr.sync();
        if (a.Cplanar) {
            if (staged) asm volatile("cp.async.wait_group 0;" ::: "memory");
            gr.sync();
            const float* src = staged ? Gs : a.Cplanar + p * n * n;
            // the planar sums are unnormalised: C_ij = numer_ij r_i r_j with r = 1 / sqrt(amp)
            // (amp = the diagonal sum), 0 where r_i r_j >= 1e6 (covariance.py:131-142)
            float* rv = reinterpret_cast<float*>(wb);
            const float rme = me < n ? __frsqrt_rn(src[me]) : 0.f;
            if (me < n) rv[me] = rme;
            gr.sync();
            if (me < n) {
                const float f = rme * rme;
                Cf[me * ld + me] = cmake(f < 1e6f ? src[me] * f : 0.f, 0.f);
            }
            const int npairs = n * (n - 1) / 2;
#pragma unroll 2
            for (int e = me; e < npairs; e += G) {
                const uint32_t rc = ptab[e];
                const int r = rc & 0xffff, c = rc >> 16;
                const float f = rv[r] * rv[c];
                cfloat v = f < 1e6f ? cmake(src[n + 2 * e] * f, src[n + 2 * e + 1] * f) : cmake(0.f, 0.f);
                if (lag > 0 && r - c >= lag) v = cmake(0.f, 0.f);
                Cf[r * ld + c] = v;
                Cf[c * ld + r] = cconj(v);
            }
        } else {
            const cfloat* src = a.Cin + p * n * n;
            for (int i = 0; i < n; ++i) {
                if (me <= i) {
                    cfloat c = src[i * n + me];
                    if (lag > 0 && i - me >= lag) c = cmake(0.f, 0.f);
                    Cf[i * ld + me] = c;
                    if (me < i) Cf[me * ld + i] = cconj(c);
                }
            }
        }
        gr.sync();
        const float* next = a.Cplanar && p + stride < a.npix ? a.Cplanar + (p + stride) * n * n : nullptr;
        solve_pixel_reg<K, G>(a, p, Cf, Gs, ld, cb, wb, ptab, next, gr);
        staged = next != nullptr;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Host launch of the instance with K slots and G threads per pixel: 8 warps per CTA,
// 256 / G pixel groups; a persistent grid of at most 8 waves.
template <int K, int G>
dpl_status launch_solve_reg_k(const PixArgs& a, cudaStream_t s) {
    const RegLayout L = make_reg_layout(a.n);
    const int warps = 8;
    const int groups = warps * 32 / G;
    const size_t smem = (size_t)groups * L.bytes + (size_t)a.n * (a.n - 1) / 2 * sizeof(uint32_t);
    if (smem > 227 * 1024) return fail(DPL_ERR_UNSUPPORTED, "register solver: shared memory exceeds the SM limit");
    int dev = 0, sms = 0;
    DPL_CUDA_TRY(cudaGetDevice(&dev));
    DPL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DPL_CUDA_TRY(cudaFuncSetAttribute(k_solve_reg<K, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    DPL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_reg<K, G>, warps * 32, smem));
    const int64_t resident = (int64_t)std::max(1, per_sm) * std::max(1, sms);
    const int64_t grid = std::min<int64_t>((a.npix + groups - 1) / groups, resident * 8);
    k_solve_reg<K, G><<<(unsigned)std::max<int64_t>(grid, 1), warps * 32, smem, s>>>(a, L);
    return check_launch("k_solve_reg");
}

}  // namespace dpl
