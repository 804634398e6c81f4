// Learned EMI warm start: the kernels of a small multilayer perceptron that reads the
// coherence magnitudes of a pixel and proposes the starting vector of the EMI inverse
// iteration (no counterpart in the reference, whose iteration starts from a constant
// vector, _eigenvalues.py:139-205; plain EMI stays the fallback).
//
//   k_mlp_features : coherence (planar, or full complex) -> |C_ij| of the N(N-1)/2
//                    lower pairs, the network input
//   k_mlp_frame    : rotates vectors into / out of the frame of the data's phases
//   k_gemm         : C = act(alpha * op(A) op(B)^T + bias) (+ beta C) in fp32, 64 x 64 tiles
//                    staged through shared memory, 4 x 4 outputs per thread; any strides,
//                    so the same kernel runs the forward pass and both backward products
//   k_relu_grad, k_mse_grad, k_adam, k_colsum : the rest of a training step
#include <cstdio>

#include "dpl_common.cuh"

namespace dpl {

// layout 0: planar (npix, N^2) floats; layout 1: full (npix, N, N) complex (lower part read)
__global__ void k_mlp_features(const float* __restrict__ C, int n, int64_t npix, int layout, float* __restrict__ X) {
    const int nf = n * (n - 1) / 2;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= npix * nf) return;
    const int64_t p = e / nf;
    const int o = (int)(e - p * nf);
    const float* src;
    if (layout == 0) {
        src = C + p * n * n + n + 2 * o;
    } else {
        int i = (int)((sqrtf(8.f * o + 1.f) + 1.f) * 0.5f);  // o = i(i-1)/2 + j, 0 <= j < i
        while (i * (i - 1) / 2 > o) --i;
        while ((i + 1) * i / 2 <= o) ++i;
        const int j = o - i * (i - 1) / 2;
        src = C + ((p * n + i) * n + j) * 2;
    }
    X[e] = hypotf(src[0], src[1]);
}

// out_j = V_j * f_j (or * conj(f_j)), f_j = exp(i angle C_j0) the phase of SLC j's
// interferogram with SLC 0 (f_0 = 1); C full (npix, N, N) complex, V and out (npix, N)
// complex.  The network works in this frame: the data supply the phases, the network
// the rest.
__global__ void k_mlp_frame(const cfloat* __restrict__ C, int n, int64_t npix, const cfloat* __restrict__ V,
                            int conj_frame, cfloat* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= npix * n) return;
    const int64_t p = e / n;
    const int j = (int)(e - p * n);
    cfloat f = cmake(1.f, 0.f);
    if (j > 0) {
        const cfloat c = C[(p * n + j) * n];
        const float m = hypotf(c.re, c.im);
        if (m > 0.f) f = cmake(c.re / m, c.im / m);
    }
    out[e] = conj_frame ? cmulc(V[e], f) : cmul(V[e], f);
}

constexpr int kGT = 64;  // output tile
constexpr int kGK = 16;  // k step

struct GemmArgs {
    int M, N, K;
    const float* A;  // element (i, k) at A[i * sai + k * sak]
    int64_t sai, sak;
    const float* B;  // element (j, k) at B[j * sbj + k * sbk]
    int64_t sbj, sbk;
    float* C;        // element (i, j) at C[i * sci + j]
    int64_t sci;
    const float* bias;  // per column j, or null
    float alpha, beta;
    int relu;
};

__global__ void __launch_bounds__(256) k_gemm(GemmArgs g) {
    __shared__ float As[kGK][kGT + 4];
    __shared__ float Bs[kGK][kGT + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int i0 = blockIdx.y * kGT, j0 = blockIdx.x * kGT;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < g.K; k0 += kGK) {
        for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
            const int kk = e / kGT, r = e - kk * kGT;
            const int i = i0 + r, j = j0 + r, k = k0 + kk;
            As[kk][r] = (i < g.M && k < g.K) ? g.A[i * g.sai + k * g.sak] : 0.f;
            Bs[kk][r] = (j < g.N && k < g.K) ? g.B[j * g.sbj + k * g.sbk] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = As[kk][ty * 4 + q];
                b[q] = Bs[kk][tx * 4 + q];
            }
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) acc[x][y] = fmaf(a[x], b[y], acc[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int i = i0 + ty * 4 + x;
        if (i >= g.M) continue;
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const int j = j0 + tx * 4 + y;
            if (j >= g.N) continue;
            float v = g.alpha * acc[x][y];
            if (g.bias) v += g.bias[j];
            float* c = g.C + i * g.sci + j;
            if (g.beta != 0.f) v += g.beta * *c;
            if (g.relu) v = v > 0.f ? v : 0.f;
            *c = v;
        }
    }
}

// dZ = dH * (H > 0) for H = relu(Z), in place on dH
__global__ void k_relu_grad(const float* __restrict__ H, float* __restrict__ dH, int64_t count) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count && !(H[e] > 0.f)) dH[e] = 0.f;
}

// mean squared error over `count` values: dY = 2 (Y - T) / count; per-block partial
// sums of the squared error into loss[blockIdx.x]
__global__ void k_mse_grad(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY,
                           int64_t count, float* __restrict__ loss) {
    __shared__ float part[8];
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float sq = 0.f;
    if (e < count) {
        const float d = Y[e] - T[e];
        dY[e] = 2.f * d / (float)count;
        sq = d * d;
    }
    sq = warp_sum(sq);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
        loss[blockIdx.x] = s;
    }
}

// column sums of an (M, N) row-major matrix: out[j] = sum_i X[i, j]
__global__ void k_colsum(const float* __restrict__ X, int M, int N, float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int i = 0; i < M; ++i) s += X[(int64_t)i * N + j];
    out[j] = s;
}

// Adam (Kingma & Ba 2015) with bias correction; step t >= 1
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ gw, float* __restrict__ m,
                       float* __restrict__ v, int64_t count, float lr, float b1, float b2, float eps, int t) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const float g = gw[e];
    const float mm = b1 * m[e] + (1.f - b1) * g;
    const float vv = b2 * v[e] + (1.f - b2) * g * g;
    m[e] = mm;
    v[e] = vv;
    const float mh = mm / (1.f - powf(b1, (float)t));
    const float vh = vv / (1.f - powf(b2, (float)t));
    w[e] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace dpl

using namespace dpl;

extern "C" dpl_status dpl_mlp_features(const float* C, int nslc, int64_t npix, int layout, float* X,
                                       dpl_stream_t stream) {
    if (nslc < 2 || nslc > 64 || npix < 0 || (layout != 0 && layout != 1))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_features: bad shape or layout");
    if (npix == 0) return DPL_OK;
    if (!C || !X) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_features: null pointer");
    const int64_t tot = npix * (int64_t)(nslc * (nslc - 1) / 2);
    k_mlp_features<<<(unsigned)ceil_div(tot, 256), 256, 0, (cudaStream_t)stream>>>(C, nslc, npix, layout, X);
    return check_launch("k_mlp_features");
}

extern "C" dpl_status dpl_mlp_frame(const float* C, int nslc, int64_t npix, const float* V, int conj_frame,
                                    float* out, dpl_stream_t stream) {
    if (nslc < 1 || nslc > 64 || npix < 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_frame: bad shape");
    if (npix == 0) return DPL_OK;
    if (!C || !V || !out) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_frame: null pointer");
    if (misaligned_c8(C) || misaligned_c8(V) || misaligned_c8(out))
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_frame: complex arrays must be 8-byte aligned");
    const int64_t tot = npix * nslc;
    k_mlp_frame<<<(unsigned)ceil_div(tot, 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const cfloat*>(C), nslc, npix, reinterpret_cast<const cfloat*>(V), conj_frame,
        reinterpret_cast<cfloat*>(out));
    return check_launch("k_mlp_frame");
}

extern "C" dpl_status dpl_gemm_f32(int M, int N, int K, const float* A, int64_t sai, int64_t sak, const float* B,
                                   int64_t sbj, int64_t sbk, float* C, int64_t sci, const float* bias, float alpha,
                                   float beta, int relu, dpl_stream_t stream) {
    if (M < 0 || N < 0 || K < 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_gemm_f32: bad shape");
    if (M == 0 || N == 0) return DPL_OK;
    if (!A || !B || !C) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_gemm_f32: null pointer");
    GemmArgs g{M, N, K, A, sai, sak, B, sbj, sbk, C, sci, bias, alpha, beta, relu};
    dim3 grid((unsigned)ceil_div(N, kGT), (unsigned)ceil_div(M, kGT));
    k_gemm<<<grid, 256, 0, (cudaStream_t)stream>>>(g);
    return check_launch("k_gemm");
}

extern "C" dpl_status dpl_relu_grad(const float* H, float* dH, int64_t count, dpl_stream_t stream) {
    if (count <= 0) return DPL_OK;
    k_relu_grad<<<(unsigned)ceil_div(count, 256), 256, 0, (cudaStream_t)stream>>>(H, dH, count);
    return check_launch("k_relu_grad");
}

extern "C" dpl_status dpl_mse_grad(const float* Y, const float* T, float* dY, int64_t count, float* loss_parts,
                                   dpl_stream_t stream) {
    if (count <= 0) return DPL_OK;
    k_mse_grad<<<(unsigned)ceil_div(count, 256), 256, 0, (cudaStream_t)stream>>>(Y, T, dY, count, loss_parts);
    return check_launch("k_mse_grad");
}

extern "C" dpl_status dpl_colsum(const float* X, int M, int N, float* out, dpl_stream_t stream) {
    if (N <= 0) return DPL_OK;
    k_colsum<<<(unsigned)ceil_div(N, 128), 128, 0, (cudaStream_t)stream>>>(X, M, N, out);
    return check_launch("k_colsum");
}

extern "C" dpl_status dpl_adam(float* w, const float* grad, float* m, float* v, int64_t count, float lr, float b1,
                               float b2, float eps, int step, dpl_stream_t stream) {
    if (count <= 0) return DPL_OK;
    if (step < 1) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_adam: step must be >= 1");
    k_adam<<<(unsigned)ceil_div(count, 256), 256, 0, (cudaStream_t)stream>>>(w, grad, m, v, count, lr, b1, b2, eps,
                                                                             step);
    return check_launch("k_adam");
}
