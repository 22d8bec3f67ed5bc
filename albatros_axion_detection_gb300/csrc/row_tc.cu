// row_tc.cu -- the IPFB row stage (inverse real FFT of every spectrum) on the
// fifth-generation tensor cores, for packed 4-bit or 1-bit spectra with at
// most 64 selected channels.
//
// Reference: cupy_ipfb (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91)
// starts with an irfft of every (nslice, 2049) spectrum row to 4096 samples;
// the streaming driver fills only the selected channels
// (scripts/xcorr/helper_gpu_stream_clean.py:295-402, unpacked by
// albatros_analysis/src/correlations/unpacking.py:140-155).  With X_k the
// spectrum, the sample at phase n is
//   x[n] = sum_k a_k (Re X_k cos(2 pi k n / P) - Im X_k sin(2 pi k n / P)),
// a_k = 1/P at k = 0 and P/2 (where the sine vanishes) and 2/P elsewhere,
// the sum running over the selected channels only.  For a tile of spectra
// that is a matrix product D[n][t] = sum_j A[n][j] B[t][j] with
// j = 2 k' + (0: Re, 1: Im) over the nsel selected channels k':
//   * B holds the decoded levels (4-bit: integers in [-7, 8]; 1-bit: signs
//     +-1), exact in fp16;
//   * A is the basis, scaled by 2^11 so that its entries lie in [-1, 1], and
//     split as A = A_hi + A_lo with both parts fp16 (A_hi the rounding of A,
//     A_lo of the remainder), computed once per channel set in FP64 on the
//     host: |A - A_hi - A_lo| <= 2^-23 per entry;
//   * D accumulates A_hi B + A_lo B in fp32 in tensor memory (kind::f16 MMA,
//     M = 128 phases, N = 128 spectra, K = 16) and the epilogue scales it by
//     2^-11 (exact).
// It replaces a 4096-point FFT per spectrum, most of whose inputs are zero,
// by 2 x 2 nsel multiply-adds per output on the tensor pipe: the stage is
// then bound by writing its output (4 bytes per sample) instead of by the
// shared-memory passes of the FFT.
//
// Work items: (spectrum tile of 128 rows, antenna, half of the 32 phase
// tiles), walked by persistent CTAs (one per SM):
//   * warps 0-7 decode both pols' B tiles of the item (each 128 rows x 2 nsel
//     fp16, K-major in the 128-byte swizzled layout) from the packets (rows
//     through the spectrum map; missing rows and rows past the window are
//     zero), then run the epilogue of every phase tile: tcgen05.ld of their
//     32 tensor-memory lanes (phases) x 32 columns (spectra) at a time,
//     staged in shared memory and written by a TMA tensor store (32 rows of
//     128 bytes of the (n, t) output per store);
//   * warp 9 streams the basis tiles (A_hi and A_lo of 128 phases, one bulk
//     copy of the pre-swizzled image, 2 x KB x 16 KB) into a 2-slot ring;
//   * warp 8 issues per phase tile 2 pols x 2 parts x 4 KB MMAs into one of
//     two tensor-memory accumulator pairs (2 x 256 columns), and commits to
//     the ring's "empty" barrier, the accumulator's "full" barrier and, after
//     the item's last tile, the B tiles' "free" barrier.
// Every barrier is waited on by one role only, phase after phase.  Waits are
// bounded (about 2 s); one that runs out sets the stream's fault word (its
// visibilities become NaN), and the copy warp waits for its copies in flight
// before the CTA ends.  For a test of that path without any fault, withhold
// makes the workers keep back their first item's "B full" arrival: the MMA
// thread's wait runs out, and with it the workers' and the copy warp's.
#include <math.h>

#include <vector>

#include "async.cuh"
#include "common.cuh"
#include "fft.cuh"
#include "ipfb.cuh"
#include "tc.cuh"

namespace ab {

constexpr int kRtTile = 128;                // phases per MMA (tensor-memory lanes) and spectra per item
constexpr int kRtWorkers = 256;             // warps 0-7
constexpr int kRtThreads = kRtWorkers + 64;  // + MMA warp (8) + copy warp (9)
constexpr int kRtSplit = 2;                 // phase ranges per (spectrum tile, antenna)
constexpr double kRtScale = 2048.0;         // basis scale 2^11
constexpr int kRtKbBytes = kRtTile * 128;   // one K-block of a 128-row operand: 64 fp16 a row

constexpr int kRtStageBytes = 32 * 32 * 4;  // a worker warp's output staging tile: 32 phases x 32 spectra

// shared memory: barriers (256 B), alignment, A ring (2 slots x 2 parts x KB
// K-blocks), B (2 pols x KB K-blocks), 8 output staging tiles
__host__ __device__ constexpr size_t row_tc_smem(int kb) {
  return 256 + 1024 + (size_t)2 * 2 * kb * kRtKbBytes + (size_t)2 * kb * kRtKbBytes + (size_t)8 * kRtStageBytes;
}

// fp16 bits of x (|x| <= 2), rounded to nearest even, subnormals included.
static uint16_t half_bits(double x) {
  const uint16_t sign = x < 0 ? 0x8000 : 0;
  double a = fabs(x);
  if (a == 0.0) return sign;
  int e;
  frexp(a, &e);  // a = f 2^e, f in [0.5, 1)
  int ex = e - 1;  // a = 1.m 2^ex
  if (ex < -14) ex = -14;  // subnormal range: fixed quantum 2^-24
  const double q = ldexp(1.0, ex - 10);
  double m = nearbyint(a / q);  // round to nearest even (default rounding mode)
  if (m >= 2048.0) {  // rounded up to the next binade
    m /= 2.0;
    ex += 1;
  }
  if (m < 1024.0) return sign | (uint16_t)m;  // subnormal (ex == -14)
  return sign | (uint16_t)(((ex + 15) << 10) | ((int)m - 1024));
}
static double half_value(uint16_t h) {
  const int ex = (h >> 10) & 31, m = h & 1023;
  const double v = ex == 0 ? ldexp((double)m, -24) : ldexp(1024.0 + m, ex - 25);
  return (h & 0x8000) ? -v : v;
}

// The basis image of a channel set: for phase tile m, part (hi, lo), K-block
// kb: 128 rows of 128 bytes in the 128-byte swizzled K-major layout, so one
// bulk copy lands a tile ready for the MMA.  Cached in the context.
int get_row_tc_basis(ab_ctx* ctx, int P, const std::vector<int32_t>& kabs, const uint16_t** out, int* kb_out) {
  *out = nullptr;
  const int nsel = (int)kabs.size();
  const int KB = (2 * nsel + 63) / 64;
  AB_CHECK_ARG(P % kRtTile == 0 && nsel >= 1 && KB <= 2, "row stage (tensor cores): unsupported shape");
  std::vector<int> key = {P};
  key.insert(key.end(), kabs.begin(), kabs.end());
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->row_bases.find(key);
    if (it != ctx->row_bases.end()) {
      *out = it->second;
      *kb_out = KB;
      return AB_OK;
    }
  }
  const int ntile = P / kRtTile;
  const size_t tile_halves = (size_t)2 * KB * kRtKbBytes / 2;
  std::vector<uint16_t> img((size_t)ntile * tile_halves, 0);
  for (int n = 0; n < P; n++) {
    const int m = n / kRtTile, rr = n % kRtTile;
    for (int j = 0; j < 2 * nsel; j++) {
      const int k = kabs[j >> 1];
      const double ak = (k == 0 || 2 * k == P) ? 1.0 / P : 2.0 / P;
      const long long e = ((long long)k * n) % P;  // exact angle index
      const double th = 2.0 * M_PI * (double)e / (double)P;
      const double v = kRtScale * ak * ((j & 1) ? -sin(th) : cos(th));
      const uint16_t hi = half_bits(v);
      const uint16_t lo = half_bits(v - half_value(hi));
      const int kb = j / 64, c = (j % 64) / 8, el = j % 8;
      const size_t off = (size_t)rr * 128 + ((size_t)((c ^ rr) & 7) << 4) + 2 * el;  // bytes within the K-block
      for (int part = 0; part < 2; part++) {
        const size_t byte = (size_t)m * (2 * tile_halves) + (size_t)part * KB * kRtKbBytes + (size_t)kb * kRtKbBytes + off;
        img[byte / 2] = part ? lo : hi;
      }
    }
  }
  uint16_t* d = nullptr;
  if (cudaMalloc(&d, sizeof(uint16_t) * img.size()) != cudaSuccess) {
    set_error("row stage (tensor cores): device allocation failed");
    return AB_ERR_NOMEM;
  }
  if (cudaMemcpy(d, img.data(), sizeof(uint16_t) * img.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    set_error("row stage (tensor cores): upload failed");
    return AB_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->row_bases.find(key);
  if (it != ctx->row_bases.end()) {
    cudaFree(d);
  } else {
    it = ctx->row_bases.emplace(key, d).first;
  }
  *out = it->second;
  *kb_out = KB;
  return AB_OK;
}

// fp16 pair (re, im) = (level of the high nibble, level of the low nibble) of byte b.
__device__ __forceinline__ uint32_t byte_to_h2(uint32_t b) {
  return nib_to_h2(nib_plus7((b >> 4) | ((b & 15u) << 16)));
}

// fp16 pair (re, im) = (+1 if bit 1 of v is set, else -1; the same for bit
// 0): one pol of a 1-bit channel, whose nibble holds r0 i0 r1 i1 from the
// top bit down (albatros_analysis/src/correlations/unpacking.c:207-246).
__device__ __forceinline__ uint32_t bits_to_h2(uint32_t v) {
  return 0x3C003C00u | ((~v & 2u) << 14) | ((~v & 1u) << 31);
}

template <int KB>
__global__ void __launch_bounds__(kRtThreads, 1)
    row_stage_tc_kernel(const __grid_constant__ CUtensorMap omap, Packed4Src src, int nrows, int P, int nant,
                        const uint16_t* __restrict__ basis, float* __restrict__ out, int64_t ld, int nitems,
                        int* __restrict__ fault, int withhold) {
  constexpr int SLOT = 2 * KB * kRtKbBytes;  // one basis tile (hi, lo)
  constexpr int BPOL = KB * kRtKbBytes;      // one pol's B tile
  const int TPI = P / kRtTile / kRtSplit;    // phase tiles per item
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw_s = smem_u32(smem_raw);
  const uint32_t bar_s = raw_s;
  const uint32_t pad = (1024u - ((raw_s + 256u) & 1023u)) & 1023u;
  uint8_t* abuf = smem_raw + 256 + pad;
  const uint32_t abuf_s = raw_s + 256u + pad;
  uint8_t* bbuf = abuf + 2 * SLOT;
  const uint32_t bbuf_s = abuf_s + 2 * SLOT;
  uint8_t* obuf = bbuf + 2 * BPOL;  // 8 staging tiles, 1024-byte aligned (128-byte swizzle)
  const uint32_t obuf_s = bbuf_s + 2 * BPOL;
  auto a_full = [&](int i) { return bar_s + 8u * (uint32_t)i; };
  auto a_empty = [&](int i) { return bar_s + 8u * (uint32_t)(2 + i); };
  auto d_full = [&](int i) { return bar_s + 8u * (uint32_t)(4 + i); };
  auto d_empty = [&](int i) { return bar_s + 8u * (uint32_t)(6 + i); };
  const uint32_t b_full = bar_s + 64u, b_free = bar_s + 72u;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem_raw + 80);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  __shared__ int skip;
  if (tid == 0) skip = *reinterpret_cast<volatile int*>(fault);
  __syncthreads();
  if (skip) return;
  // zero B once: K past 2 nsel stays zero
  for (int i = tid; i < 2 * BPOL / 16; i += kRtThreads)
    reinterpret_cast<uint4*>(bbuf)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    for (int i = 0; i < 2; i++) {
      mbar_init(a_full(i), 1);
      mbar_init(a_empty(i), 1);
      mbar_init(d_full(i), 1);
      mbar_init(d_empty(i), kRtWorkers);
    }
    mbar_init(b_full, kRtWorkers);
    mbar_init(b_free, 1);
    mbar_init_fence();
  }
  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int nsel4 = (src.nsel + 3) / 4;

  if (warp < 8) {
    // ---------------- workers: decode B, then the epilogues ----------------
    const int c4 = tid % 16;  // channel quad of this thread (16 quads = 64 channels)
    int cols[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int k = 4 * c4 + j;
      cols[j] = k < src.nsel ? __ldg(&src.chan_cols[k]) : -1;
    }
    const int q = warp & 3, pol_e = warp >> 2;  // epilogue: lane quadrant, pol
    int T = 0;  // phase tiles done
    bool ok = true;
    for (int it = blockIdx.x, li = 0; it < nitems && ok; it += gridDim.x, li++) {
      const int ph = it % kRtSplit, rest = it / kRtSplit;
      const int a = rest % nant, rt = rest / nant;
      const int t0 = rt * kRtTile;
      if (li > 0 && !mbar_wait(b_free, (uint32_t)((li - 1) & 1))) {
        atomicExch(fault, 1);
        break;
      }
      if (c4 < nsel4) {
        for (int r = tid / 16; r < kRtTile; r += kRtWorkers / 16) {
          const int t = t0 + r;
          const int64_t g = src.g0 + t;
          int32_t row = -1;
          if (t < nrows && g >= 0) row = src.spec_map ? __ldg(&src.spec_map[(int64_t)a * src.map_stride + g]) : (int32_t)g;
          uint32_t w0[4] = {0u, 0u, 0u, 0u}, w1[4] = {0u, 0u, 0u, 0u};
          if (row >= 0) {
            const uint8_t* prow = src.raw + (int64_t)a * src.ant_stride + (int64_t)row * src.row_bytes;
            if (src.bits == 4) {  // bytes 2c (pol 0) and 2c + 1 (pol 1)
#pragma unroll
              for (int j = 0; j < 4; j++) {
                if (cols[j] < 0) continue;
                const uint32_t pb = __ldg(reinterpret_cast<const unsigned short*>(prow + 2 * cols[j]));
                w0[j] = byte_to_h2(pb & 0xffu);
                w1[j] = byte_to_h2(pb >> 8);
              }
            } else {  // 1-bit: the high nibble of byte c/2 for even c, the low one for odd c
#pragma unroll
              for (int j = 0; j < 4; j++) {
                if (cols[j] < 0) continue;
                const uint32_t q = ((uint32_t)__ldg(prow + (cols[j] >> 1)) >> ((cols[j] & 1) ? 0 : 4)) & 15u;
                w0[j] = bits_to_h2(q >> 2);
                w1[j] = bits_to_h2(q);
              }
            }
          }
          const uint32_t off = (uint32_t)(c4 / 8) * kRtKbBytes + sw128_offset(r, c4 % 8);
          *reinterpret_cast<uint4*>(bbuf + off) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
          *reinterpret_cast<uint4*>(bbuf + BPOL + off) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
        }
      }
      fence_proxy_async();
      if (!(withhold && li == 0)) mbar_arrive(b_full);
      const float inv = (float)(1.0 / kRtScale);
      for (int j = 0; j < TPI; j++, T++) {
        const int slot = T & 1;
        if (!mbar_wait(d_full(slot), (uint32_t)((T >> 1) & 1))) {
          atomicExch(fault, 1);
          ok = false;
          break;
        }
        tc_fence_after();
        // this warp's 32 phases (rows of the output) and the 128 spectra of
        // the item, in four 32 x 32 blocks: each staged in shared memory in
        // the 128-byte swizzled layout (row = phase, 16-byte chunk c at
        // c ^ (row mod 8): the 8 lanes of a store phase hit distinct banks)
        // and written by one TMA tensor store; the TMA engine skips rows of
        // the output past nrows.
        const int row0 = (2 * a + pol_e) * P + (ph * TPI + j) * kRtTile + 32 * q;
        uint8_t* st = obuf + warp * kRtStageBytes;
        const uint32_t st_s = obuf_s + warp * kRtStageBytes;
#pragma unroll 1
        for (int c = 0; c < kRtTile / 32; c++) {
          float v[32];
          tc_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(slot * 256 + pol_e * 128 + 32 * c), v);
          if (lane == 0) bulk_wait_read_all();  // the previous block has left the staging tile
          __syncwarp();
#pragma unroll
          for (int i = 0; i < 8; i++)
            *reinterpret_cast<float4*>(st + lane * 128 + ((i ^ (lane & 7)) << 4)) =
                make_float4(v[4 * i] * inv, v[4 * i + 1] * inv, v[4 * i + 2] * inv, v[4 * i + 3] * inv);
          fence_proxy_async();
          __syncwarp();
          if (lane == 0 && t0 + 32 * c < nrows) {
            tma_store_2d(&omap, t0 + 32 * c, row0, st_s);
            bulk_commit();
          }
        }
        tc_fence_before();
        mbar_arrive(d_empty(slot));
      }
    }
    if (lane == 0) bulk_wait_all();  // every output block written before the CTA ends
  } else if (warp == 8) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      int T = 0;
      bool ok = true;
      for (int it = blockIdx.x, li = 0; it < nitems && ok; it += gridDim.x, li++) {
        if (!mbar_wait(b_full, (uint32_t)(li & 1))) {
          atomicExch(fault, 1);
          break;
        }
        for (int j = 0; j < TPI; j++, T++) {
          const int slot = T & 1;
          if (!mbar_wait(a_full(slot), (uint32_t)((T >> 1) & 1)) ||
              (T >= 2 && !mbar_wait(d_empty(slot), (uint32_t)(((T >> 1) - 1) & 1)))) {
            atomicExch(fault, 1);
            ok = false;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int pol = 0; pol < 2; pol++) {
#pragma unroll
            for (int part = 0; part < 2; part++) {
#pragma unroll
              for (int kk = 0; kk < 4 * KB; kk++) {
                const uint64_t ad = sw128_kmajor_desc(abuf_s + slot * SLOT + part * BPOL + (kk >> 2) * kRtKbBytes +
                                                      (kk & 3) * 32);
                const uint64_t bd = sw128_kmajor_desc(bbuf_s + pol * BPOL + (kk >> 2) * kRtKbBytes + (kk & 3) * 32);
                tc_mma(tmem + (uint32_t)(slot * 256 + pol * 128), ad, bd, (part > 0 || kk > 0) ? 1u : 0u);
              }
            }
          }
          tc_commit(a_empty(slot));
          tc_commit(d_full(slot));
        }
        if (ok) tc_commit(b_free);
      }
    }
  } else if (lane == 0) {
    // ---------------- basis copies ----------------
    int T = 0;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
      const int ph = it % kRtSplit;
      bool ok = true;
      for (int j = 0; j < TPI; j++, T++) {
        const int slot = T & 1;
        if (T >= 2 && !mbar_wait(a_empty(slot), (uint32_t)(((T >> 1) - 1) & 1))) {
          atomicExch(fault, 1);
          ok = false;
          break;
        }
        mbar_arrive_expect_tx(a_full(slot), (uint32_t)SLOT);
        bulk_load(abuf_s + slot * SLOT, basis + (size_t)(ph * TPI + j) * (SLOT / 2), (uint32_t)SLOT, a_full(slot));
      }
      if (!ok) break;
    }
    // every copy issued has landed before the CTA may end
    for (int u = (T >= 2 ? T - 2 : 0); u < T; u++)
      if (!mbar_wait(a_full(u & 1), (uint32_t)((u >> 1) & 1))) atomicExch(fault, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 8) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

int launch_row_stage_tc(ab_ctx* ctx, const Packed4Src& src, int nant, int nrows, int P, const uint16_t* basis, int kb,
                        float* out, int64_t ld, int* fault, cudaStream_t s) {
  AB_CHECK_ARG((src.bits == 4 || src.bits == 1) && src.nsel >= 1 && src.nsel <= 64 && kb >= 1 && kb <= 2 && P % (kRtTile * kRtSplit) == 0 &&
                   ld % 8 == 0 && ((uintptr_t)out & 31) == 0 && nrows >= 1,
               "row stage (tensor cores): unsupported shape");
  const size_t smem = row_tc_smem(kb);
  AB_CHECK_ARG(smem <= ctx->smem_optin, "row stage (tensor cores): %zu bytes of shared memory needed", smem);
  const int64_t nitems = (int64_t)((nrows + kRtTile - 1) / kRtTile) * nant * kRtSplit;
  AB_CHECK_ARG(nitems < (1LL << 31), "row stage (tensor cores): too many work items");
  const int grid = (int)std::min<int64_t>(nitems, ctx->num_sms);
  // output tensor: rows (input, phase) of nrows floats, ld apart; 32 x 32 boxes, 128-byte swizzle
  CUtensorMap omap;
  const uint64_t dims[2] = {(uint64_t)nrows, (uint64_t)2 * nant * P};
  const uint64_t strides[1] = {(uint64_t)ld * sizeof(float)};
  const uint32_t box[2] = {32, 32};
  AB_TRY(encode_tmap(&omap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, out, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B));
  int withhold = 0;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->test_withhold_stage == 2) {  // one launch only
      withhold = 1;
      ctx->test_withhold_stage = 0;
    }
  }
  if (kb == 1) {
    AB_CUDA(cudaFuncSetAttribute(row_stage_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    row_stage_tc_kernel<1><<<grid, kRtThreads, smem, s>>>(omap, src, nrows, P, nant, basis, out, ld, (int)nitems,
                                                           fault, withhold);
  } else {
    AB_CUDA(cudaFuncSetAttribute(row_stage_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    row_stage_tc_kernel<2><<<grid, kRtThreads, smem, s>>>(omap, src, nrows, P, nant, basis, out, ld, (int)nitems,
                                                           fault, withhold);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

}  // namespace ab
