// Helpers shared by the kernels that drive the 5th-generation tensor cores (tcgen05):
// shared-memory matrix descriptors (K-major, no swizzle), the kind::f16 instruction
// descriptor for bf16 operands and an fp32 accumulator, bounded mbarrier waits and the
// 32-lane x 32- and x 16-column tensor-memory loads.
#pragma once

#include <stdint.h>

namespace dpl {

constexpr uint32_t kTcWaitLimit = 1u << 25;  // bound on the polls of a wait (>= 64 ns apart)

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; swizzle none
    return d;
}

__device__ __forceinline__ uint32_t tc_idesc_bf16(int m, int nn) {
    uint32_t d = 0;
    d |= 1u << 4;   // D: f32
    d |= 1u << 7;   // A: bf16
    d |= 1u << 10;  // B: bf16
    d |= (uint32_t)(nn >> 3) << 17;
    d |= (uint32_t)(m >> 4) << 24;
    return d;
}

// kind::tf32 with tf32 A and B (format code 2 in both fields) and an fp32 accumulator
__device__ __forceinline__ uint32_t tc_idesc_tf32(int m, int nn) {
    uint32_t d = 0;
    d |= 1u << 4;   // D: f32
    d |= 2u << 7;   // A: tf32
    d |= 2u << 10;  // B: tf32
    d |= (uint32_t)(nn >> 3) << 17;
    d |= (uint32_t)(m >> 4) << 24;
    return d;
}

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// one test of an mbarrier phase with a suspend-time hint: the thread is suspended
// (taking no issue slots) until the phase completes or about kTcSuspendNs have passed
constexpr uint32_t kTcSuspendNs = 1000;
__device__ __forceinline__ bool tc_try_wait_suspend(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(tc_smem(bar)), "r"(parity), "r"(kTcSuspendNs)
        : "memory");
    return ok != 0;
}

// bounded wait: suspended waits with a short sleep after each one that times out;
// returns false after kTcWaitLimit / 8 of them (between ~0.3 and ~4 s)
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kTcWaitLimit / 8; ++it) {
        if (tc_try_wait_suspend(bar, parity)) return true;
        __nanosleep(64);
    }
    return false;
}

// tcgen05.ld is warp-collective (.sync.aligned): the __syncwarp() reconverges a warp
// whose lanes took different branches before the load
__device__ __forceinline__ void tc_ld32(uint32_t addr, uint32_t (&r)[32]) {
    __syncwarp();
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// the same for 16 columns
__device__ __forceinline__ void tc_ld16(uint32_t addr, uint32_t (&r)[16]) {
    __syncwarp();
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace dpl
