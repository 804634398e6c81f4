// Tensor-core forward pass of the learned warm start's network (inference; training
// stays in fp32, mlp.cu): Y = L3(relu(L2(relu(L1(X))))), L_l(h) = h W_l^T + b_l.
//
// k_mlp_pack -- once per set of weights: W_l (out, in) fp32 -> bf16 blocks of 64 input
//               columns (K), rows padded to a multiple of 16, zero-filled, each block
//               in the canonical K-major no-swizzle layout (8-row x 16-byte core
//               matrices, LBO 128 B, SBO 1024 B) so that one 1-D bulk copy stages it.
// k_mlp_tc   -- persistent, 128 threads, one 128-pixel tile at a time (the MMA's M):
//               the tile's features are converted to bf16 into the A operand (128 x 256,
//               canonical K-major, SBO 4096 B); per layer, thread 0 streams the weight
//               blocks through a two-buffer ring (cp.async.bulk, mbarrier completion)
//               and issues tcgen05.mma.kind::f16 (bf16 x bf16 -> fp32 in tensor memory,
//               N = the layer's padded width); all four warps then read the accumulator
//               (tcgen05.ld, lane = pixel), add the bias, apply ReLU and write bf16 into
//               the A operand of the next layer, or fp32 to Y after the last one.  Layer
//               1 accumulates in TMEM columns 0-255, layer 2 in 256-511, layer 3 in 0-255
//               again.  Every wait is bounded; a timeout sets the status word, and the
//               kernel waits (bounded) for its MMAs in flight and frees TMEM before it
//               returns.
#include <cuda_bf16.h>

#include <cstdio>

#include "dpl_common.cuh"
#include "tc_common.cuh"

namespace dpl {

constexpr int kMlpM = 128;        // pixels per tile
constexpr int kMlpKC = 64;        // input columns per packed weight block
constexpr int kMlpKMax = 256;     // widest layer input held in the A operand
constexpr int kMlpNMax = 256;     // widest layer output
constexpr int kMlpThreads = 128;  // four warps: TMEM lane quarters 0-3
constexpr uint32_t kMlpAStride = kMlpKMax / 8 * 128;           // A: bytes per 8 rows
constexpr uint32_t kMlpBBytes = (uint32_t)kMlpNMax * kMlpKC * 2;  // one weight block buffer
constexpr uint32_t kMlpABytes = (uint32_t)kMlpM * kMlpKMax * 2;

inline int pad_up(int v, int m) { return (v + m - 1) / m * m; }

__device__ __forceinline__ uint32_t mlp_a_off(int row, int k) {
    return (uint32_t)(row >> 3) * kMlpAStride + (uint32_t)(k >> 3) * 128u + (uint32_t)(row & 7) * 16u +
           (uint32_t)(k & 7) * 2u;
}

__global__ void k_mlp_pack(const float* __restrict__ W, int nout, int nin, int np, int nchunks,
                           uint16_t* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t per = (int64_t)np * kMlpKC;
    if (e >= per * nchunks) return;
    const int c = (int)(e / per);
    const int rem = (int)(e - (int64_t)c * per);
    const int r = rem / kMlpKC, kl = rem - r * kMlpKC;
    const int k = c * kMlpKC + kl;
    const float w = (r < nout && k < nin) ? W[(int64_t)r * nin + k] : 0.f;
    const int64_t byte = (int64_t)c * np * 128 + (r >> 3) * (kMlpKC / 8 * 128) + (kl >> 3) * 128 + (r & 7) * 16 +
                         (kl & 7) * 2;
    out[byte / 2] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
}

struct MlpTcArgs {
    const float* X;
    int64_t npix;
    int n[4];               // input width, hidden widths, output width
    const unsigned char* W[3];  // packed weights
    const float* b[3];
    int np[3];              // padded layer widths (multiples of 16)
    int nch[3];             // 64-column weight blocks per layer
    float* Y;
    int* status;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__global__ void __launch_bounds__(kMlpThreads, 1) k_mlp_tc(MlpTcArgs a) {
    extern __shared__ __align__(16) unsigned char mlp_smem[];
    const uint32_t mis = tc_smem(mlp_smem) & 127u;
    unsigned char* sm = mlp_smem + ((128u - mis) & 127u);
    unsigned char* A = sm;
    unsigned char* B = sm + kMlpABytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(B + 2 * kMlpBBytes);
    uint64_t* empty = full + 2;
    uint64_t* done = full + 4;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(full + 5);
    int* sfail = reinterpret_cast<int*>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(done)));
        *sfail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    uint32_t ph_full = 0, ph_empty = 0, ph_done = 0, pend = 0;  // thread 0: ring state
    int g = 0;                                                  // thread 0: blocks issued
    const int64_t ntiles = (a.npix + kMlpM - 1) / kMlpM;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t p0 = tile * kMlpM;
        // features -> bf16 A operand, zero beyond the input width and the last pixel
        const int k0 = a.nch[0] * kMlpKC;
        for (int row = warp; row < kMlpM; row += kMlpThreads / 32) {
            const int64_t p = p0 + row;
            for (int k = lane; k < k0; k += 32) {
                const float x = (p < a.npix && k < a.n[0]) ? a.X[p * a.n[0] + k] : 0.f;
                *reinterpret_cast<__nv_bfloat16*>(A + mlp_a_off(row, k)) = __float2bfloat16_rn(x);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int l = 0; l < 3; ++l) {
            const uint32_t dcol = l == 1 ? 256u : 0u;
            const uint32_t bbytes = (uint32_t)a.np[l] * 128u;  // np rows x 64 columns x 2 bytes
            if (tid == 0) {
                const uint32_t idesc = tc_idesc_bf16(kMlpM, a.np[l]);
                bool ok = true;
                for (int c = 0; c < a.nch[l] && ok; ++c, ++g) {
                    const int s = g & 1;
                    if ((pend >> s) & 1u) {  // the MMAs that read this buffer must be done
                        ok = tc_wait(&empty[s], (ph_empty >> s) & 1u);
                        ph_empty ^= 1u << s;
                        pend &= ~(1u << s);
                        if (!ok) break;
                    }
                    unsigned char* dst = B + s * kMlpBBytes;
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc_smem(&full[s])),
                                 "r"(bbytes)
                                 : "memory");
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            tc_smem(dst)),
                        "l"(a.W[l] + (size_t)c * bbytes), "r"(bbytes), "r"(tc_smem(&full[s]))
                        : "memory");
                    ok = tc_wait(&full[s], (ph_full >> s) & 1u);
                    if (!ok) {
                        // the copy may still be in flight: a second bounded wait before leaving
                        tc_wait(&full[s], (ph_full >> s) & 1u);
                        break;
                    }
                    ph_full ^= 1u << s;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                    for (int kk = 0; kk < kMlpKC; kk += 16) {
                        const int k = c * kMlpKC + kk;
                        const uint64_t ad = tc_desc(tc_smem(A) + (uint32_t)(k / 8) * 128u, 128u, kMlpAStride);
                        const uint64_t bd = tc_desc(tc_smem(dst) + (uint32_t)(kk / 8) * 128u, 128u, kMlpKC / 8 * 128);
                        const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem + dcol),
                            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     tc_smem(&empty[s]))
                                 : "memory");
                    pend |= 1u << s;
                }
                if (ok) {
                    // arrives once every MMA issued so far has completed
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     tc_smem(done))
                                 : "memory");
                } else {
                    *sfail = 1;
                }
            }
            __syncthreads();
            if (*(volatile int*)sfail) break;
            const bool waited = tc_wait(done, ph_done);
            ph_done ^= 1u;
            if (__syncthreads_or(!waited)) {
                if (tid == 0) *sfail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // epilogue: TMEM lane = pixel row of the tile
            const int row = warp * 32 + lane;
            const int64_t p = p0 + row;
            const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
            const int nout = a.n[l + 1];
            const float* bias = a.b[l];
            int j = 0;
            for (; j < a.np[l]; j += 32) {
                uint32_t r[32];
                tc_ld32(tmem + lane_base + dcol + (uint32_t)j, r);
                if (l < 2) {
#pragma unroll
                    for (int q8 = 0; q8 < 4; ++q8) {
                        float v[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const int col = j + 8 * q8 + q;
                            v[q] = col < nout ? fmaxf(__uint_as_float(r[8 * q8 + q]) + bias[col], 0.f) : 0.f;
                        }
                        uint4 w;
                        w.x = pack_bf16x2(v[0], v[1]);
                        w.y = pack_bf16x2(v[2], v[3]);
                        w.z = pack_bf16x2(v[4], v[5]);
                        w.w = pack_bf16x2(v[6], v[7]);
                        *reinterpret_cast<uint4*>(A + mlp_a_off(row, j + 8 * q8)) = w;
                    }
                } else if (p < a.npix) {
#pragma unroll
                    for (int q = 0; q < 32; ++q) {
                        const int col = j + q;
                        if (col < nout) a.Y[p * nout + col] = __uint_as_float(r[q]) + bias[col];
                    }
                }
            }
            if (l < 2) {
                // the next layer reads 64-column blocks: zero the columns beyond this one
                for (; j < a.nch[l + 1] * kMlpKC; j += 8)
                    *reinterpret_cast<uint4*>(A + mlp_a_off(row, j)) = make_uint4(0u, 0u, 0u, 0u);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        if (*(volatile int*)sfail) break;
    }
    if (tid == 0) {
        // no MMA may still be writing TMEM when it is released (bounded waits)
        for (int s = 0; s < 2; ++s)
            if ((pend >> s) & 1u) tc_wait(&empty[s], (ph_empty >> s) & 1u);
        if (*(volatile int*)sfail) atomicExch(a.status, (int)DPL_ERR_TIMEOUT);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

}  // namespace dpl

using namespace dpl;

extern "C" size_t dpl_mlp_packed_bytes(int nout, int nin) {
    if (nout <= 0 || nin <= 0) return 0;
    return (size_t)pad_up(nout, 16) * 128u * (size_t)(pad_up(nin, kMlpKC) / kMlpKC);
}

extern "C" dpl_status dpl_mlp_pack(const float* W, int nout, int nin, void* packed, dpl_stream_t stream) {
    if (nout <= 0 || nin <= 0 || nout > kMlpNMax || nin > kMlpKMax)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_pack: layer widths must be 1..256");
    if (!W || !packed) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_pack: null pointer");
    if (((uintptr_t)packed & 15u) != 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_pack: packed not 16-byte aligned");
    const int np = pad_up(nout, 16), nch = pad_up(nin, kMlpKC) / kMlpKC;
    const int64_t total = (int64_t)np * kMlpKC * nch;
    k_mlp_pack<<<ceil_div(total, 256), 256, 0, (cudaStream_t)stream>>>(W, nout, nin, np, nch,
                                                                       static_cast<uint16_t*>(packed));
    return check_launch("k_mlp_pack");
}

extern "C" dpl_status dpl_mlp_forward_tc(const float* X, int64_t npix, int n0, int n1, int n2, int n3,
                                         const void* W1, const float* b1, const void* W2, const float* b2,
                                         const void* W3, const float* b3, float* Y, int* status,
                                         dpl_stream_t stream) {
    const int n[4] = {n0, n1, n2, n3};
    for (int i = 0; i < 4; ++i)
        if (n[i] <= 0 || n[i] > 256) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_forward_tc: widths must be 1..256");
    if (npix < 0) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_forward_tc: negative pixel count");
    if (npix == 0) return DPL_OK;
    if (!X || !W1 || !W2 || !W3 || !b1 || !b2 || !b3 || !Y || !status)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_forward_tc: null pointer");
    const void* W[3] = {W1, W2, W3};
    for (int i = 0; i < 3; ++i)
        if (((uintptr_t)W[i] & 15u) != 0)
            return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_mlp_forward_tc: packed weights not 16-byte aligned");
    MlpTcArgs a{};
    a.X = X;
    a.npix = npix;
    for (int i = 0; i < 4; ++i) a.n[i] = n[i];
    a.W[0] = static_cast<const unsigned char*>(W1);
    a.W[1] = static_cast<const unsigned char*>(W2);
    a.W[2] = static_cast<const unsigned char*>(W3);
    a.b[0] = b1;
    a.b[1] = b2;
    a.b[2] = b3;
    for (int l = 0; l < 3; ++l) {
        a.np[l] = pad_up(n[l + 1], 16);
        a.nch[l] = pad_up(n[l], kMlpKC) / kMlpKC;
    }
    a.Y = Y;
    a.status = status;
    const size_t smem = kMlpABytes + 2 * kMlpBBytes + 5 * sizeof(uint64_t) + 16 + 128;
    int dev = 0, sms = 0;
    DPL_CUDA_TRY(cudaGetDevice(&dev));
    DPL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DPL_CUDA_TRY(cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t ntiles = (npix + kMlpM - 1) / kMlpM;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, (int64_t)sms);
    k_mlp_tc<<<grid, kMlpThreads, smem, (cudaStream_t)stream>>>(a);
    return check_launch("k_mlp_tc");
}
