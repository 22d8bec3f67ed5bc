// tc.cuh -- fifth-generation tensor-core (tcgen05) building blocks shared by
// the coarse correlator (xcorr_tc.cu) and the tensor-core IPFB row stage
// (row_tc.cu): fences, the shared-memory and instruction descriptors of a
// kind::f16 MMA on K-major operands in the 128-byte swizzled layout, the MMA
// itself, commits to mbarriers, tensor-memory loads, and the integer tricks
// that turn packed 4-bit levels into fp16.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

namespace ab {

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand in the 128-byte
// swizzled layout: rows of 128 bytes (64 fp16 samples), 8-row atoms of 1024
// bytes (stride-dimension offset), the leading-dimension offset unused (16
// bytes), descriptor version 1, swizzle mode 2 (128 B).
__device__ __forceinline__ uint64_t sw128_kmajor_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: fp32 accumulators, fp16 A and B, both
// K-major, M = 128, N = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate,
                                       uint32_t idesc = kTcIdesc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive fp32 columns of this warp's 32 tensor-memory lanes.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Nibble-wise (v + 7) mod 16 of the 8 nibbles of w (no carries between
// nibbles): the low 3 bits plus 7 carry into bit 3, which is then flipped by
// the nibble's own bit 3.  The decoded level is then n - 7 for n = (v+7)&15
// (v > 8 -> v - 16, else v).
__device__ __forceinline__ uint32_t nib_plus7(uint32_t w) {
  return ((w & 0x77777777u) + 0x77777777u) ^ (w & 0x88888888u);
}
// fp16 pair (n_lo - 7, n_hi - 7) from 4-bit fields n in the low bits of each
// 16-bit half: 0x6400 | n is the fp16 value 1024 + n, and 1031 = 0x6407.
__device__ __forceinline__ uint32_t nib_to_h2(uint32_t n2) {
  uint32_t r;
  const uint32_t x = (n2 & 0x000F000Fu) | 0x64006400u;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(x), "r"(0x64076407u));
  return r;
}

// Byte offset of (row, 16-byte chunk c) in a 128-row K-major tile of 128-byte
// rows with the 128-byte swizzle (chunk index XOR row mod 8).
__device__ __forceinline__ uint32_t sw128_offset(int row, int c) {
  return (uint32_t)(row * 128 + (((c ^ row) & 7) << 4));
}

// Decode one (antenna, 8-sample group kc) item of a stage: w[i] holds the
// packet words of the group's i-th sample (every selected channel's two pols,
// nib_plus7 already applied); each byte b = 2 j + pol of channel j gives the
// rows (.., re) from its high nibbles and (.., im) from its low ones, 8
// samples = one 16-byte chunk of a 128-byte swizzled row.

}  // namespace ab
