// Per-pixel kernel arguments and shared-memory layouts shared by the phase-linking
// translation units (the pipeline in phase_link.cu, the register-solver instances in
// solver_reg_*.cu).
#pragma once

#include <algorithm>

#include "dpl_common.cuh"

namespace dpl {

// ---------------------------------------------------------------------------------
// k_pixel: per-warp shared-memory layout
// ---------------------------------------------------------------------------------
// C (packed complex) | W1 (packed real) | S: staging for the window rows, or R (packed
// complex) + W2 (packed real), or the full n x n LU of the fallback | v | d | piv
struct PixLayout {
    int n, np, stg, ldg;
    size_t off_C, off_G, off_S, off_v, off_d, off_piv, bytes;
};

// C (packed complex) | G (n x ldg real) | S: staging for the covariance's window rows,
// or R (packed complex), or the full n x n LU of the LU pass | v | d | piv
inline PixLayout make_layout(int n, int wx, bool lu) {
    PixLayout L{};
    const size_t T = (size_t)n * (n + 1) / 2;
    L.n = n;
    L.np = (n + 1) & ~1;
    L.stg = wx * L.np + 32;
    L.ldg = n | 1;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align_up(o + bytes, 16);
        return at;
    };
    L.off_C = take(T * sizeof(cfloat));
    L.off_G = take((size_t)n * L.ldg * sizeof(float));
    size_t s_bytes = std::max((size_t)L.stg * sizeof(cfloat), T * sizeof(cfloat));
    if (lu) s_bytes = std::max(s_bytes, (size_t)n * n * sizeof(cfloat));
    L.off_S = take(s_bytes);
    L.off_v = take(64 * sizeof(cfloat));
    L.off_d = take(64 * sizeof(float));
    L.off_piv = take(128 * sizeof(int));
    L.bytes = align_up(o, 128);
    return L;
}

enum PixMode { kCovOnly = 0, kSolveOnly = 1, kFused = 2 };

struct PixArgs {
    int n, rows, cols, hy, hx, sy, sx, out_rows, out_cols;
    int64_t npix;
    int np, stg, ldg;
    size_t off_C, off_G, off_S, off_v, off_d, off_piv, warp_bytes;
    const cfloat* zt;        // (rows, cols, n) masked, pixel-major
    const uint8_t* nb_u8;    // (out_rows, out_cols, wy, wx) or null
    const uint32_t* nb_bits; // (out_rows, out_cols, wy, wpr) or null
    int wpr;
    const cfloat* Cin;       // solve-only input: (npix, n, n)
    const cfloat* vstart;    // optional EMI starting vectors (npix, n); plain start when null
    int16_t* iters;          // optional: eigen-iterations used per pixel (npix)
    const float* Cplanar;    // solve-only input, planar per pixel: diagonal | (Re, Im) per lower pair
    int use_evd, beta_on;
    float one_minus_beta, beta, zct;
    int ref_idx, compute_crlb, crlb_ref, baseline_lag;
    float crlb_factor;
    double beta_d, zct_d, crlb_factor_d;  // the same parameters unrounded (FP64 form)
    cfloat* Cout;            // cov-only output: (npix, n, n)
    cfloat* vout;            // (npix, n) referenced eigenvectors
    float* eig;
    uint8_t* est;
    float* crlb;             // (npix, n)
    float* tcoh;
    float* closure;          // (npix, n - 2) or null
    int32_t* counts;         // (npix) or null
    int* fb_list;            // pixels whose EMI shifted matrix is indefinite (for the LU pass)
    int* fb_count;
    const int* list;         // LU pass: pixels list[0 .. *list_count)
    const int* list_count;
    int lanes;               // register solver: threads per pixel (8, 16, 32; 0 = the smallest that fits)
    int* nc_list;            // pixels whose eigen-iteration missed its stopping rule (null: not listed)
    int* nc_count;
    uint8_t* nc_flag;        // (npix) 1 where the dense eigensolver replaced the iterate, or null
    int eigh;                // FP64 form: the dense eigensolver for iterations that miss the rule
    int slots;               // register solver: row slots K (even, >= n; 0 = n rounded up to even)
};

// Threads per pixel group for K slots: `req` if it is 8, 16 or 32 and at least K,
// else the smallest of them that is (K <= 32); 64 above 32 slots.
inline int solver_lanes(int K, int req) {
    if (K > 32) return 64;
    int P = 8;
    while (P < K) P *= 2;
    if (req >= P && req <= 32 && (req & (req - 1)) == 0) P = req;
    return P;
}

// Register-solver launch for any n <= 64 (instances per even slot count K and group
// size, spread over the solver_reg_*.cu translation units); a.slots and a.lanes pick a
// tuned instance.
dpl_status launch_solve_reg(const PixArgs& a, cudaStream_t s);

}  // namespace dpl
