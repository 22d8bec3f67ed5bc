// xcorr_tc.cu -- the all-baseline coarse correlator on the fifth-generation
// tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// Same Gram matrix as the warp-level forms in xcorr.cu: per channel, the
// matrix A has one row per (antenna, pol, re|im) and one column per time
// sample, G = A A^T, Re V_ij = G[r_i, r_j] + G[m_i, m_j] and
// Im V_ij = G[m_i, r_j] - G[r_i, m_j] (the X X^H of
// albatros_analysis/src/correlations/correlations_gpu.py:95-121, replacing the
// cuBLAS CGEMM of albatros_analysis/src/correlations/cgemm_batch.cu:8-53).
//
// Exactness.  The decoded nibbles are integers in [-7, 8] (0x8 decodes to +8,
// as in albatros_analysis/src/correlations/unpacking.c:187-202), exact in
// fp16; products are at most 64, and a CTA sums at most kTcMaxSlice = 2^17
// samples, so every partial sum is an integer of magnitude at most 2^23 and
// the fp32 accumulation in tensor memory is exact in any order.  The
// partials are converted to int64 exactly and added into the per-chunk sums
// with int64 atomics (order-independent, bit-reproducible).
//
// Tiles.  A 128-row operand tile holds CPT channels' rows (CPT = 2 with 64
// rows a channel for up to 16 antennas, CPT = 1 with 128 rows for up to 32);
// the rows of absent antennas stay zero.  One MMA of M = N = 128, K = 16 runs
// the tile against itself, accumulating the 128 x 128 fp32 product in 128
// tensor-memory columns; the channel blocks on its diagonal are the Gram
// matrices.  A CTA owns kTcTiles tiles (4 * CPT channels, all 512 columns of
// tensor memory) and a slice of time samples.
//
// Pipeline (one CTA per SM):
//   * warps 0-7 produce: two groups of 4 warps take alternate stages of
//     kTcKt = 64 samples; a thread loads 8 consecutive samples of one
//     antenna (16 or 8 bytes each: every selected channel's two pols),
//     decodes the nibbles to fp16 with integer tricks (below) and writes
//     whole 16-byte rows of 8 samples into the stage's K-major tiles in the
//     128-byte swizzled layout; then fence.proxy.async and an mbarrier arrive;
//   * warp 8 allocates the tensor memory, and its lane 0 waits for each full
//     stage, issues 4 tiles x 4 k-steps of tcgen05.mma and commits to the
//     stage's "empty" barrier, which frees the stage for the producers;
//   * after the last stage a commit to the "done" barrier releases warps 0-3,
//     which read their 32 tensor-memory lanes each (tcgen05.ld) and add the
//     Gram entries into the int64 sums.
// Every mbarrier wait is bounded (about 2 s of wall time); a thread whose wait
// runs out sets the call's fault word, stops issuing work and drains, the
// tensor memory is freed on every path, CTAs starting after it do nothing,
// and the finalize kernel then writes INT64_MIN to every output of the call
// (so a fault cannot pass for data).  AB_OPT_FAULT_TEST 1 makes the next call's
// producers withhold their first stage, so that path can be tested without
// a fault.
#include <cuda_fp16.h>

#include "async.cuh"
#include "common.cuh"
#include "tc.cuh"

namespace ab {

constexpr int kTcKt = 64;                          // samples per stage
constexpr int kTcStages = 3;                       // stage ring
constexpr int kTcTiles = 4;                        // 128-row tiles per CTA (4 x 128 TMEM columns)
constexpr int kTcTileBytes = 128 * kTcKt * 2;      // 16 KB of fp16 per tile
constexpr int kTcStageBytes = kTcTiles * kTcTileBytes;
constexpr int kTcProducers = 256;                  // warps 0-7
constexpr int kTcThreads = kTcProducers + 32;      // + the MMA / tensor-memory warp
constexpr int kTcGroup = kTcProducers / 2;         // producer threads per stage
constexpr int64_t kTcMaxSlice = 1 << 17;           // samples a CTA may sum (exactness bound)
constexpr size_t kTcSmemBytes = (size_t)kTcStages * kTcStageBytes + 1024 /* alignment */ + 128 /* barriers */;

template <int CPT>
__device__ __forceinline__ void tc_store_item(const uint32_t (&w)[8][CPT == 2 ? 4 : 2], int ant, int kc,
                                              uint8_t* stage) {
  constexpr int CPC = kTcTiles * CPT, BPT = 2 * CPC, ROWS = 128 / CPT;
#pragma unroll
  for (int b = 0; b < BPT; b++) {
    const int j = b >> 1, pol = b & 1;
    const int tile = j / CPT, h = j % CPT;
    const int row_re = h * ROWS + 4 * ant + 2 * pol;
    const uint32_t sel = (uint32_t)(b & 3) * 0x1111u + 0x4400u;  // byte b%4 of each word -> bytes 0|1 and 2|3
    uint32_t re[4], im[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const uint32_t p = __byte_perm(w[2 * m][b >> 2], w[2 * m + 1][b >> 2], sel);
      im[m] = nib_to_h2(p);
      re[m] = nib_to_h2(p >> 4);
    }
    uint8_t* tb = stage + tile * kTcTileBytes;
    *reinterpret_cast<uint4*>(tb + sw128_offset(row_re, kc)) = make_uint4(re[0], re[1], re[2], re[3]);
    *reinterpret_cast<uint4*>(tb + sw128_offset(row_re + 1, kc)) = make_uint4(im[0], im[1], im[2], im[3]);
  }
}

template <int CPT>  // channels per 128-row tile: 2 (nant <= 16) or 1 (nant <= 32)
__global__ void __launch_bounds__(kTcThreads, 1)
    coarse_xcorr_tc_kernel(const uint8_t* __restrict__ raw, int64_t ant_stride, int64_t row_bytes, int nant,
                           int64_t rowstart, int64_t nrows, const int32_t* __restrict__ rows,
                           const int64_t* __restrict__ channels, int ncols, int64_t chunk_rows, int64_t slice,
                           int64_t slices_per_chunk, int Rp, long long* __restrict__ G, int* __restrict__ fault,
                           int withhold) {
  constexpr int CPC = kTcTiles * CPT;   // channels per CTA
  constexpr int BPT = 2 * CPC;          // packet bytes per (antenna, sample): CPC channels x 2 pols
  constexpr int WPT = BPT / 4;          // 32-bit words per (antenna, sample)
  constexpr int ROWS = 128 / CPT;       // tile rows per channel
  constexpr int NA = ROWS / 4;          // antennas a channel's rows can hold
  constexpr int IPT = NA * 8 / kTcGroup;  // (antenna, 8-sample group) items per producer thread
  static_assert(IPT * kTcGroup == NA * 8, "items must divide evenly over a producer group");
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte aligned stage ring (the swizzle atoms), then the barriers
  const uint32_t raw_s = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (raw_s & 1023u)) & 1023u;
  uint8_t* stages = smem_raw + pad;
  const uint32_t stages_s = raw_s + pad;
  uint64_t* bars = reinterpret_cast<uint64_t*>(stages + kTcStages * kTcStageBytes);
  const uint32_t bar_s = stages_s + kTcStages * kTcStageBytes;
  auto full_bar = [&](int i) { return bar_s + 8u * (uint32_t)i; };
  auto empty_bar = [&](int i) { return bar_s + 8u * (uint32_t)(kTcStages + i); };
  const uint32_t done_bar = bar_s + 8u * (2 * kTcStages);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kTcStages + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.x * CPC;
  const int64_t chunk = blockIdx.y / slices_per_chunk;
  const int64_t sl = blockIdx.y % slices_per_chunk;
  const int64_t k_begin = chunk * chunk_rows + sl * slice;
  const int64_t chunk_end = min((chunk + 1) * chunk_rows, nrows);
  const int64_t k_end = min(k_begin + slice, chunk_end);
  const int nst = k_end > k_begin ? (int)((k_end - k_begin + kTcKt - 1) / kTcKt) : 0;

  // a call whose fault word is already set (an earlier CTA's wait ran out)
  // does no more work: its outputs become INT64_MIN anyway
  __shared__ int skip;
  if (tid == 0) skip = *reinterpret_cast<volatile int*>(fault);
  __syncthreads();
  if (skip) return;

  // zero the stage ring once: rows of absent antennas and channels stay zero
  for (int i = tid; i < kTcStages * kTcStageBytes / 16; i += kTcThreads)
    reinterpret_cast<uint4*>(stages)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    for (int i = 0; i < kTcStages; i++) {
      mbar_init(full_bar(i), kTcGroup);
      mbar_init(empty_bar(i), 1);
    }
    mbar_init(done_bar, 1);
    mbar_init_fence();
  }
  if (warp == kTcProducers / 32) {  // the MMA warp owns the tensor memory
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTcTiles * 128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // zeroed tiles visible to the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < kTcProducers / 32) {
    // ---------------- producers ----------------
    const int g = tid / kTcGroup, pt = tid % kTcGroup;
    // 16- or 8-byte packet loads need the CTA's channels contiguous and aligned
    bool vec = ((uintptr_t)raw % 16 == 0) && ant_stride % 16 == 0 && row_bytes % 16 == 0 && c0 + CPC <= ncols;
    if (vec) {
      const int64_t ch0 = channels[c0];
      vec = (2 * ch0) % BPT == 0;
#pragma unroll
      for (int j = 1; j < CPC; j++) vec = vec && channels[c0 + j] == ch0 + j;
    }
    // The packet words of one stage for this thread's IPT items (antenna,
    // 8-sample group): 8 samples x WPT words each, zero past the slice end
    // and for absent antennas.  A stage's words are loaded before the
    // previous stage of the group is decoded, so the loads stay in flight
    // while the thread decodes.
    auto load_stage = [&](int s, uint32_t (&w)[IPT][8][WPT]) {
      const int64_t kt = k_begin + (int64_t)s * kTcKt;
#pragma unroll
      for (int it = 0; it < IPT; it++) {
        const int item = pt + it * kTcGroup, ant = item >> 3, kc = item & 7;
#pragma unroll
        for (int i = 0; i < 8; i++) {
#pragma unroll
          for (int q = 0; q < WPT; q++) w[it][i][q] = 0u;
          const int64_t k = kt + 8 * kc + i;
          if (ant < nant && s < nst && k < k_end) {
            const int64_t r = rows ? (int64_t)rows[(int64_t)ant * nrows + k] : rowstart + k;
            const uint8_t* src = raw + (int64_t)ant * ant_stride + r * row_bytes;
            if (vec) {
              const uint8_t* p = src + 2 * channels[c0];
              if constexpr (WPT == 4) {
                const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
                w[it][i][0] = v.x;
                w[it][i][1] = v.y;
                w[it][i][2] = v.z;
                w[it][i][3] = v.w;
              } else {
                const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
                w[it][i][0] = v.x;
                w[it][i][1] = v.y;
              }
            } else {
#pragma unroll
              for (int j = 0; j < CPC; j++) {
                uint32_t b2 = 0u;  // absent channel: nibble 0 decodes to 0
                if (c0 + j < ncols) {
                  const uint8_t* p = src + 2 * channels[c0 + j];
                  b2 = (uint32_t)__ldg(p) | ((uint32_t)__ldg(p + 1) << 8);
                }
                w[it][i][j >> 1] |= b2 << (16 * (j & 1));
              }
            }
          }
        }
      }
    };
    uint32_t w[IPT][8][WPT];
    load_stage(g, w);
    bool ok = true;
    for (int s = g; s < nst && ok; s += 2) {
      const int slot = s % kTcStages, use = s / kTcStages;
      uint32_t wn[IPT][8][WPT];
      load_stage(s + 2, wn);  // nothing past the last stage
      if (use > 0 && !mbar_wait(empty_bar(slot), (uint32_t)((use - 1) & 1))) {
        atomicExch(fault, 1);
        ok = false;
        break;
      }
      uint8_t* stage = stages + slot * kTcStageBytes;
#pragma unroll
      for (int it = 0; it < IPT; it++) {
        const int item = pt + it * kTcGroup, ant = item >> 3, kc = item & 7;
        if (ant >= nant) continue;  // its rows stay zero
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
          for (int q = 0; q < WPT; q++) w[it][i][q] = nib_plus7(w[it][i][q]);
        tc_store_item<CPT>(w[it], ant, kc, stage);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (!(withhold && s == 0)) mbar_arrive(full_bar(slot));  // withhold: failure-path test, the MMA wait runs out
#pragma unroll
      for (int it = 0; it < IPT; it++)
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
          for (int q = 0; q < WPT; q++) w[it][i][q] = wn[it][i][q];
    }
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    for (int s = 0; s < nst; s++) {
      const int slot = s % kTcStages, use = s / kTcStages;
      if (!mbar_wait(full_bar(slot), (uint32_t)(use & 1))) {
        atomicExch(fault, 1);
        break;
      }
      tc_fence_after();
      const uint32_t st = stages_s + slot * kTcStageBytes;
#pragma unroll
      for (int t = 0; t < kTcTiles; t++) {
#pragma unroll
        for (int kk = 0; kk < kTcKt / 16; kk++) {
          const uint64_t d = sw128_kmajor_desc(st + t * kTcTileBytes + kk * 32);
          tc_mma(tmem + 128u * t, d, d, (s > 0 || kk > 0) ? 1u : 0u);
        }
      }
      tc_commit(empty_bar(slot));
    }
    tc_commit(done_bar);  // arrives once every MMA issued above has completed
  }

  // ---------------- epilogue: warps 0-3 read lanes 32w .. 32w+31 ----------------
  if (warp < 4) {
    const bool done = nst > 0 && mbar_wait(done_bar, 0u);
    if (nst > 0 && !done) atomicExch(fault, 1);
    tc_fence_after();
    if (done) {
      const int row = 32 * warp + lane;  // tensor-memory lane = row of the tile
      const int h = row / ROWS, rr = row % ROWS;
      const int R = 4 * nant;
#pragma unroll 1
      for (int t = 0; t < kTcTiles; t++) {
        const int ch = c0 + t * CPT + h;
#pragma unroll 1
        for (int cb = 0; cb < ROWS; cb += 32) {
          float v[32];
          // every lane of the warp takes part in the load, whatever its row
          tc_ld32(tmem + ((uint32_t)(32 * warp) << 16) + 128u * t + (uint32_t)(h * ROWS + cb), v);
          if (ch < ncols && rr < R) {
            long long* Gr = G + (((int64_t)chunk * ncols + ch) * Rp + rr) * Rp;
#pragma unroll
            for (int c = 0; c < 32; c++)
              if (cb + c < R) atomicAdd((unsigned long long*)&Gr[cb + c], (unsigned long long)__float2ll_rn(v[c]));
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kTcProducers / 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTiles * 128));
  }
}

// TMA form (CPT = 2: up to 16 antennas, 8 channels a CTA; contiguous channel
// groups on 16-byte boundaries, no row lists).  A stage's packet bytes, 16
// bytes (8 channels x 2 pols) of 64 samples of each of 16 antennas, arrive as
// one cp.async.bulk.tensor box in a ring of 16 KB slots (antennas past nant
// and rows past the array read as zero), issued by warp 17 ahead of the
// decoders; the decoders read them from shared memory instead of issuing
// 16-byte global loads of rows 512 bytes apart, whose scattered lines kept
// the L1 data pipe busy.  A decoder orders its reads of a slot before the
// slot's next box with fence.proxy.async before it releases the slot: the
// box is written by the asynchronous proxy, and without the fence a box
// could land before the reads were done (measured: wrong sums in up to 40 %
// of the outputs).
//
// Decoders: 16 warps in two groups of 8 taking alternate stages.  Thread
// (antenna, half, kc) takes half of the sample record (4 channels x 2 pols,
// 8 bytes) of the samples kc + 8 i (i < 8): the 8-byte reads of a half-warp
// cover 128 consecutive bytes and the 16-byte stores of a quarter-warp one
// 128-byte row (no bank conflicts), and the 8 samples fill the chunk kc of
// the operand rows.  That permutes the stage's 64 samples in the same way
// for every row, which leaves the Gram sums unchanged.
//
// Levels are stored as 16 x (n - 7) (n = (v + 7) mod 16 of the raw nibble
// v): a low nibble n in the mantissa of 0x7400 is the fp16 value 16384 +
// 16 n, a high nibble in place (n << 4) under 0x6400 is 1024 + 16 n, so one
// subtraction each gives 16 (n - 7) with no shift.  Every product is then a
// multiple of 256 and every partial sum a multiple of 256 of magnitude at
// most 2^31 (64 x 256 x kTcMaxSlice), exact in fp32; the epilogue divides by
// 256 (exact).
//
// Waits are bounded as in the form above; before exiting, warp 17 waits
// (bounded) for every box it issued, so no copy lands after the CTA ends.
constexpr int kTmaSlotBytes = 16 * kTcKt * 16;  // 16 ant x 64 samples x 16 bytes
constexpr int kTcProducersT = 512;                 // warps 0-15
constexpr int kTcGroupT = kTcProducersT / 2;       // decoder threads per stage
constexpr int kTcThreadsT = kTcProducersT + 64;    // + the MMA warp (16) + the TMA warp (17)
// NOP operand stages, NRG packet slots
__host__ __device__ constexpr size_t tc_tma_smem(int nop, int nrg) {
  return (size_t)nop * kTcStageBytes + (size_t)nrg * kTmaSlotBytes + 1024 /* alignment */ + 256 /* barriers */;
}
// Two operand stages and four packet slots (measured on 16 antennas x 256
// channels x 2^18 spectra: 0.89 ms; three operand stages with two slots, the
// most that fit: 0.90 ms)
constexpr int kTcOpStagesTma = 2, kTcRingTma = 4;
constexpr size_t kTcSmemBytesTma = tc_tma_smem(kTcOpStagesTma, kTcRingTma);

// fp16 pairs 16 (n - 7) from the low nibbles (lo) and high nibbles (hi) of
// bytes 0 and 2 of p.
__device__ __forceinline__ uint32_t nib_lo_h2x16(uint32_t p) {
  uint32_t r;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"((p & 0x000F000Fu) | 0x74007400u), "r"(0x74077407u));
  return r;
}
__device__ __forceinline__ uint32_t nib_hi_h2x16(uint32_t p) {
  uint32_t r;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"((p & 0x00F000F0u) | 0x64006400u), "r"(0x64706470u));
  return r;
}

// Half an item: bytes 8 half + b (b < 8) of the 8 samples in w[i] (2 words
// each, nib_plus7 applied) into the operand rows, 16 x the levels.
__device__ __forceinline__ void tc_store_half(const uint32_t (&w)[8][2], int ant, int kc, int half, uint8_t* stage) {
  constexpr int ROWS = 64;  // CPT = 2
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const int j = 4 * half + (b >> 1), pol = b & 1;  // channel j of the CTA's 8
    const int tile = j >> 1, h = j & 1;
    const int row_re = h * ROWS + 4 * ant + 2 * pol;
    const uint32_t sel = (uint32_t)(b & 3) * 0x1111u + 0x4400u;
    uint32_t re[4], im[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const uint32_t p = __byte_perm(w[2 * m][b >> 2], w[2 * m + 1][b >> 2], sel);
      im[m] = nib_lo_h2x16(p);
      re[m] = nib_hi_h2x16(p);
    }
    uint8_t* tb = stage + tile * kTcTileBytes;
    *reinterpret_cast<uint4*>(tb + sw128_offset(row_re, kc)) = make_uint4(re[0], re[1], re[2], re[3]);
    *reinterpret_cast<uint4*>(tb + sw128_offset(row_re + 1, kc)) = make_uint4(im[0], im[1], im[2], im[3]);
  }
}

template <int kTcOpStagesT, int kTmaRing>
__global__ void __launch_bounds__(kTcThreadsT, 1)
    coarse_xcorr_tc_tma_kernel(const __grid_constant__ CUtensorMap tmap, const uint8_t* __restrict__ raw,
                               int64_t ant_stride, int64_t row_bytes, int nant, int64_t rowstart, int64_t nrows,
                               const int64_t* __restrict__ channels, int ncols, int64_t chunk_rows, int64_t slice,
                               int64_t slices_per_chunk, int Rp, long long* __restrict__ G, int* __restrict__ fault,
                               int withhold) {
  constexpr int CPT = 2, CPC = kTcTiles * CPT, ROWS = 128 / CPT;
  constexpr int MMA_WARP = kTcProducersT / 32, TMA_WARP = MMA_WARP + 1;
  // Layout: barriers and the tensor-memory address (256 bytes), then from
  // the next 1024-byte boundary the packet ring, then the operand stages
  // (1024-byte aligned for the swizzle atoms).
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw_s = smem_u32(smem_raw);
  const uint32_t bar_s = raw_s;
  const uint32_t pad = (1024u - ((raw_s + 256u) & 1023u)) & 1023u;
  uint8_t* ring = smem_raw + 256 + pad;
  const uint32_t ring_s = raw_s + 256u + pad;
  uint8_t* stages = ring + kTmaRing * kTmaSlotBytes;
  const uint32_t stages_s = ring_s + kTmaRing * kTmaSlotBytes;
  // Operand barriers per virtual slot v = s mod NV (NV = lcm(2, stages)):
  // each is waited on, phase after phase, by one decoder group or by the MMA
  // thread alone, so no parity wait can pass a phase early.
  constexpr int NV = kTcOpStagesT % 2 ? 2 * kTcOpStagesT : kTcOpStagesT;
  auto op_full = [&](int v) { return bar_s + 8u * (uint32_t)v; };
  auto op_empty = [&](int v) { return bar_s + 8u * (uint32_t)(NV + v); };
  auto rg_full = [&](int i) { return bar_s + 8u * (uint32_t)(2 * NV + i); };
  auto rg_empty = [&](int i) { return bar_s + 8u * (uint32_t)(2 * NV + kTmaRing + i); };
  const uint32_t done_bar = bar_s + 8u * (2 * NV + 2 * kTmaRing);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem_raw + 8 * (2 * NV + 2 * kTmaRing + 1));
  static_assert(8 * (2 * NV + 2 * kTmaRing + 1) + 4 <= 256, "barrier space");

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.x * CPC;
  const int64_t chunk = blockIdx.y / slices_per_chunk;
  const int64_t sl = blockIdx.y % slices_per_chunk;
  const int64_t k_begin = chunk * chunk_rows + sl * slice;
  const int64_t chunk_end = min((chunk + 1) * chunk_rows, nrows);
  const int64_t k_end = min(k_begin + slice, chunk_end);
  const int nst = k_end > k_begin ? (int)((k_end - k_begin + kTcKt - 1) / kTcKt) : 0;

  __shared__ int skip;
  if (tid == 0) skip = *reinterpret_cast<volatile int*>(fault);
  __syncthreads();
  if (skip) return;
  // this CTA's channels: contiguous and 16-byte aligned -> TMA; else
  // (a ragged last group, scattered channels) byte loads
  bool tma = c0 + CPC <= ncols;
  if (tma) {
    const int64_t ch0 = channels[c0];
    tma = (2 * ch0) % 16 == 0;
#pragma unroll
    for (int j = 1; j < CPC; j++) tma = tma && channels[c0 + j] == ch0 + j;
  }

  for (int i = tid; i < kTcOpStagesT * kTcStageBytes / 16; i += kTcThreadsT)
    reinterpret_cast<uint4*>(stages)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    for (int v = 0; v < NV; v++) {
      mbar_init(op_full(v), kTcGroupT);
      mbar_init(op_empty(v), 1);
    }
    for (int i = 0; i < kTmaRing; i++) {
      mbar_init(rg_full(i), 1);
      mbar_init(rg_empty(i), kTcGroupT);
    }
    mbar_init(done_bar, 1);
    mbar_init_fence();
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTcTiles * 128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < MMA_WARP) {
    // ---------------- decoders: group g takes stages g, g + 2, ... ----------------
    const int g = tid / kTcGroupT, pt = tid % kTcGroupT;
    // kc fastest: a quarter-warp's 16-byte stores fill one 128-byte row
    const int ant = pt >> 4, half = (pt >> 3) & 1, kc = pt & 7;
    for (int s = g; s < nst; s += 2) {
      const int oslot = s % kTcOpStagesT;
      const int64_t kt = k_begin + (int64_t)s * kTcKt;
      uint32_t w[8][2];
      if (tma) {
        const int r = s % kTmaRing;
        if (!mbar_wait(rg_full(r), (uint32_t)((s / kTmaRing) & 1))) {
          atomicExch(fault, 1);
          break;
        }
        const uint8_t* slot = ring + r * kTmaSlotBytes + ant * (kTcKt * 16) + 8 * half;
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const int smp = kc + 8 * i;
          const uint2 v = *reinterpret_cast<const uint2*>(slot + smp * 16);
          const bool in = kt + smp < k_end;  // rows of the box past the slice read as zero
          w[i][0] = in ? v.x : 0u;
          w[i][1] = in ? v.y : 0u;
        }
        // the slot's next box is written by the asynchronous proxy: order
        // these generic reads before it, then release the slot
        fence_proxy_async();
        mbar_arrive(rg_empty(r));
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const int64_t k = kt + kc + 8 * i;
          w[i][0] = 0u;
          w[i][1] = 0u;
          if (ant < nant && k < k_end) {
            const uint8_t* src = raw + (int64_t)ant * ant_stride + (rowstart + k) * row_bytes;
#pragma unroll
            for (int jj = 0; jj < 4; jj++) {
              const int j = 4 * half + jj;
              uint32_t b2 = 0u;
              if (c0 + j < ncols) {
                const uint8_t* p = src + 2 * channels[c0 + j];
                b2 = (uint32_t)__ldg(p) | ((uint32_t)__ldg(p + 1) << 8);
              }
              w[i][jj >> 1] |= b2 << (16 * (jj & 1));
            }
          }
        }
      }
      // the slot's previous stage, s - kTcOpStagesT, has left the tensor cores
      const int sp = s - kTcOpStagesT;
      if (sp >= 0 && !mbar_wait(op_empty(sp % NV), (uint32_t)((sp / NV) & 1))) {
        atomicExch(fault, 1);
        break;
      }
      if (ant < nant) {
#pragma unroll
        for (int i = 0; i < 8; i++) {
          w[i][0] = nib_plus7(w[i][0]);
          w[i][1] = nib_plus7(w[i][1]);
        }
        tc_store_half(w, ant, kc, half, stages + oslot * kTcStageBytes);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (!(withhold && s == 0)) mbar_arrive(op_full(s % NV));
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      for (int s = 0; s < nst; s++) {
        const int slot = s % kTcOpStagesT;
        if (!mbar_wait(op_full(s % NV), (uint32_t)((s / NV) & 1))) {
          atomicExch(fault, 1);
          break;
        }
        tc_fence_after();
        const uint32_t st = stages_s + slot * kTcStageBytes;
#pragma unroll
        for (int t = 0; t < kTcTiles; t++) {
#pragma unroll
          for (int kk = 0; kk < kTcKt / 16; kk++) {
            const uint64_t d = sw128_kmajor_desc(st + t * kTcTileBytes + kk * 32);
            tc_mma(tmem + 128u * t, d, d, (s > 0 || kk > 0) ? 1u : 0u);
          }
        }
        tc_commit(op_empty(s % NV));
      }
      tc_commit(done_bar);
    }
  } else if (warp == TMA_WARP && lane == 0 && tma) {
    // ---------------- TMA issuer ----------------
    const int x = (int)(2 * channels[c0]);
    int issued = 0;
    for (int s = 0; s < nst; s++) {
      const int r = s % kTmaRing, use = s / kTmaRing;
      if (use > 0 && !mbar_wait(rg_empty(r), (uint32_t)((use - 1) & 1))) {
        atomicExch(fault, 1);
        break;
      }
      mbar_arrive_expect_tx(rg_full(r), (uint32_t)kTmaSlotBytes);
      tma_load_3d(ring_s + r * kTmaSlotBytes, &tmap, x, (int)(rowstart + k_begin + (int64_t)s * kTcKt), 0, rg_full(r));
      issued = s + 1;
    }
    // every box issued has landed before the CTA may end
    for (int s = max(0, issued - kTmaRing); s < issued; s++)
      if (!mbar_wait(rg_full(s % kTmaRing), (uint32_t)((s / kTmaRing) & 1))) atomicExch(fault, 1);
  }

  // ---------------- epilogue: warps 0-3 read lanes 32w .. 32w+31 ----------------
  if (warp < 4) {
    const bool done = nst > 0 && mbar_wait(done_bar, 0u);
    if (nst > 0 && !done) atomicExch(fault, 1);
    tc_fence_after();
    if (done) {
      const int row = 32 * warp + lane;
      const int h = row / ROWS, rr = row % ROWS;
      const int R = 4 * nant;
#pragma unroll 1
      for (int t = 0; t < kTcTiles; t++) {
        const int ch = c0 + t * CPT + h;
#pragma unroll 1
        for (int cb = 0; cb < ROWS; cb += 32) {
          float v[32];
          tc_ld32(tmem + ((uint32_t)(32 * warp) << 16) + 128u * t + (uint32_t)(h * ROWS + cb), v);
          if (ch < ncols && rr < R) {
            long long* Gr = G + (((int64_t)chunk * ncols + ch) * Rp + rr) * Rp;
#pragma unroll
            for (int c = 0; c < 32; c++)  // sums of 256 x the level products (exact)
              if (cb + c < R)
                atomicAdd((unsigned long long*)&Gr[cb + c], (unsigned long long)__float2ll_rn(v[c] * (1.0f / 256.0f)));
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == MMA_WARP) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTiles * 128));
  }
}

// Launch the tensor-core form for 1 <= nant <= 32 into G (zeroed by the
// caller, stride Rp >= 4*nant); *fault must be zero before the launch.
int launch_coarse_tc(ab_ctx* ctx, const uint8_t* raw, int64_t ant_stride, int64_t nant, int64_t nchan,
                     int64_t rowstart, int64_t nrows, const int32_t* rows, const int64_t* channels, int64_t ncols,
                     int64_t chunk_rows, int Rp, long long* G, int* fault, cudaStream_t s) {
  AB_CHECK_ARG(nant >= 1 && nant <= 32 && 4 * nant <= Rp, "coarse xcorr (tensor cores): nant %lld unsupported",
               (long long)nant);
  AB_CHECK_ARG(kTcSmemBytes <= ctx->smem_optin, "coarse xcorr (tensor cores): %zu bytes of shared memory needed",
               kTcSmemBytes);
  const int cpt = nant <= 16 ? 2 : 1;
  const int64_t cpc = (int64_t)kTcTiles * cpt;
  const int64_t groups = (ncols + cpc - 1) / cpc;
  const int64_t nchunks = (nrows + chunk_rows - 1) / chunk_rows;
  // about four CTAs per SM in total, slices of whole stages, at most kTcMaxSlice samples
  int64_t per = std::max<int64_t>(1, (4 * (int64_t)ctx->num_sms + groups * nchunks - 1) / (groups * nchunks));
  int64_t slice = (chunk_rows + per - 1) / per;
  slice = std::min<int64_t>(std::max<int64_t>((slice + kTcKt - 1) / kTcKt * kTcKt, kTcKt), kTcMaxSlice);
  if (ctx->coarse_tc_slice > 0) slice = ctx->coarse_tc_slice;
  const int64_t spc = (chunk_rows + slice - 1) / slice;
  AB_CHECK_ARG(groups <= 0x7fffffff && nchunks * spc <= 65535,
               "coarse xcorr (tensor cores): %lld chunks x %lld slices exceed the grid limit; use larger chunks",
               (long long)nchunks, (long long)spc);
  dim3 grid((unsigned)groups, (unsigned)(nchunks * spc));
  int withhold = 0;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->test_withhold_stage == 1) {  // one call only
      withhold = 1;
      ctx->test_withhold_stage = 0;
    }
  }
  // TMA staging: 16 antennas at most, no row lists, 16-byte aligned rows
  const int64_t row_bytes = 2 * nchan;
  if (cpt == 2 && ctx->coarse_tc_tma && !rows && (uintptr_t)raw % 16 == 0 && ant_stride % 16 == 0 &&
      row_bytes % 16 == 0 && rowstart + nrows + kTcKt < (1LL << 31) && kTcSmemBytesTma <= ctx->smem_optin) {
    CUtensorMap tmap;
    const uint64_t dims[3] = {(uint64_t)row_bytes, (uint64_t)(rowstart + nrows), (uint64_t)nant};
    const uint64_t strides[2] = {(uint64_t)row_bytes, (uint64_t)ant_stride};
    const uint32_t box[3] = {16, (uint32_t)kTcKt, 16};
    if (encode_tmap(&tmap, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, raw, dims, strides, box) == AB_OK) {
      AB_CUDA(cudaFuncSetAttribute(coarse_xcorr_tc_tma_kernel<kTcOpStagesTma, kTcRingTma>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemBytesTma));
      coarse_xcorr_tc_tma_kernel<kTcOpStagesTma, kTcRingTma><<<grid, kTcThreadsT, kTcSmemBytesTma, s>>>(
          tmap, raw, ant_stride, row_bytes, (int)nant, rowstart, nrows, channels, (int)ncols, chunk_rows, slice, spc,
          Rp, G, fault, withhold);
      AB_LAUNCH_CHECK();
      return AB_OK;
    }
    set_error("");  // the map was refused: the register-load form below
  }
  if (cpt == 2) {
    AB_CUDA(cudaFuncSetAttribute(coarse_xcorr_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTcSmemBytes));
    coarse_xcorr_tc_kernel<2><<<grid, kTcThreads, kTcSmemBytes, s>>>(raw, ant_stride, 2 * nchan, (int)nant, rowstart,
                                                                     nrows, rows, channels, (int)ncols, chunk_rows,
                                                                     slice, spc, Rp, G, fault, withhold);
  } else {
    AB_CUDA(cudaFuncSetAttribute(coarse_xcorr_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTcSmemBytes));
    coarse_xcorr_tc_kernel<1><<<grid, kTcThreads, kTcSmemBytes, s>>>(raw, ant_stride, 2 * nchan, (int)nant, rowstart,
                                                                     nrows, rows, channels, (int)ncols, chunk_rows,
                                                                     slice, spc, Rp, G, fault, withhold);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

}  // namespace ab
