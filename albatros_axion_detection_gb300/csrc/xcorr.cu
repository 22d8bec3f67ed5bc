// xcorr.cu -- correlators.
//
//  * fine (float) all-antenna correlator: avg_xcorr_all_ant_gpu
//    (albatros_analysis/src/correlations/correlations_gpu.py:95-121), which the
//    reference runs as cublasCgemmStridedBatched (cgemm_batch.cu:8-53);
//  * the streaming chain's per-job accumulation of the same products;
//  * exact integer coarse correlator on raw 4-bit packets with tensor cores,
//    flushed into int64: by default mma.sync m16n8k16 with fp16 operands and
//    fp32 partial sums, exact because the levels (-7..8) are exact in fp16,
//    products are at most 64 and a CTA's partial sums over at most 4096
//    samples stay below 2^24; or mma.sync m16n8k32 s8 -> s32
//    (AB_OPT_COARSE_MMA_BITS = 8).  tcgen05 kind::i8 is not offered for
//    sm_103a;
//  * pairwise 4-bit / 1-bit correlators on sortpols'd bytes
//    (albatros_analysis/src/correlations/correlations_cpu.c:128-638).
#include <cuda_fp16.h>

#include "common.cuh"

namespace ab {

// ---------------------------------------------------------------------------
// Fine correlator: x F-ordered (M, T, F); out F-ordered (M, M, F).
constexpr int kXcTile = 4;
constexpr int kXcThreads = 256;

__global__ void __launch_bounds__(kXcThreads)
    xcorr_fine_kernel(const float2* __restrict__ x, int M, int64_t T, int64_t F, float2* __restrict__ out,
                      float inv_t) {
  const int64_t f = blockIdx.x;
  const int ntile = (M + kXcTile - 1) / kXcTile;
  const int ti = blockIdx.y / ntile, tj = blockIdx.y % ntile;
  const int i0 = ti * kXcTile, j0 = tj * kXcTile;
  float2 acc[kXcTile][kXcTile];
#pragma unroll
  for (int a = 0; a < kXcTile; a++)
#pragma unroll
    for (int b = 0; b < kXcTile; b++) acc[a][b] = make_float2(0.f, 0.f);
  const float2* xf = x + (int64_t)M * T * f;
  for (int64_t t = threadIdx.x; t < T; t += blockDim.x) {
    const float2* xt = xf + (int64_t)M * t;
    float2 xi[kXcTile], xj[kXcTile];
#pragma unroll
    for (int a = 0; a < kXcTile; a++) {
      xi[a] = (i0 + a < M) ? xt[i0 + a] : make_float2(0.f, 0.f);
      xj[a] = (j0 + a < M) ? xt[j0 + a] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int a = 0; a < kXcTile; a++)
#pragma unroll
      for (int b = 0; b < kXcTile; b++) {
        acc[a][b].x = fmaf(xi[a].x, xj[b].x, fmaf(xi[a].y, xj[b].y, acc[a][b].x));
        acc[a][b].y = fmaf(xi[a].y, xj[b].x, fmaf(-xi[a].x, xj[b].y, acc[a][b].y));
      }
  }
  // block reduction: warp shuffles then shared memory
  __shared__ float2 red[kXcThreads / 32][kXcTile * kXcTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < kXcTile; a++)
#pragma unroll
    for (int b = 0; b < kXcTile; b++) {
      float2 v = acc[a][b];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[warp][a * kXcTile + b] = v;
    }
  __syncthreads();
  if (threadIdx.x < kXcTile * kXcTile) {
    float2 s = make_float2(0.f, 0.f);
    for (int w = 0; w < kXcThreads / 32; w++) s = cadd(s, red[w][threadIdx.x]);
    int a = threadIdx.x / kXcTile, b = threadIdx.x % kXcTile;
    int i = i0 + a, j = j0 + b;
    if (i < M && j < M) out[i + (int64_t)M * (j + (int64_t)M * f)] = cscale(s, inv_t);
  }
}

// ---------------------------------------------------------------------------
// Streaming chain accumulation: Y[in][b][f] (c64); for blocks [b_lo, b_hi)
// vis[(i*M + j)*F + f] += scale * sum_b Y_i conj(Y_j), lower triangle mirrored.
// fault (or null): set by an earlier stage whose asynchronous copies did not
// arrive; the visibilities touched are then NaN.
__global__ void xcorr_accum_kernel(const float2* __restrict__ Y, int M, int64_t nb, int64_t F, int64_t b_lo,
                                   int64_t b_hi, float2* __restrict__ vis, float scale, const int* __restrict__ fault) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F) return;
  // pair index p -> (i, j), i <= j
  int p = blockIdx.y, i = 0;
  while (p >= M - i) {
    p -= M - i;
    i++;
  }
  const int j = i + p;
  float2 acc = make_float2(0.f, 0.f);
  const float2* yi = Y + (int64_t)i * nb * F + f;
  const float2* yj = Y + (int64_t)j * nb * F + f;
  for (int64_t b = b_lo; b < b_hi; b++) {
    float2 a = __ldg(&yi[b * F]), c = __ldg(&yj[b * F]);
    acc.x = fmaf(a.x, c.x, fmaf(a.y, c.y, acc.x));
    acc.y = fmaf(a.y, c.x, fmaf(-a.x, c.y, acc.y));
  }
  acc = cscale(acc, scale);
  if (fault && *fault) acc = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
  float2* v = vis + ((int64_t)i * M + j) * F + f;
  *v = cadd(*v, acc);
  if (i != j) {
    float2* w = vis + ((int64_t)j * M + i) * F + f;
    *w = cadd(*w, cconj(acc));
  }
}

// Small-M form: a CTA owns kXaF frequencies; its kXaG thread groups take
// blocks b_lo + g, b_lo + g + kXaG, ... and keep all M(M+1)/2 pair sums of
// their frequency in registers (each Y element is read once), then the groups
// are summed through shared memory in a fixed order (deterministic).
constexpr int kXaF = 32, kXaG = 8;

template <int M>
__global__ void __launch_bounds__(kXaF * kXaG)
    xcorr_accum_small_kernel(const float2* __restrict__ Y, int64_t nb, int64_t F, int64_t b_lo, int64_t b_hi,
                             float2* __restrict__ vis, float scale, const int* __restrict__ fault) {
  constexpr int NP = M * (M + 1) / 2;
  __shared__ float2 part[kXaG][NP][kXaF];
  const int fl = threadIdx.x % kXaF, g = threadIdx.x / kXaF;
  const int64_t f = (int64_t)blockIdx.x * kXaF + fl;
  float2 acc[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) acc[p] = make_float2(0.f, 0.f);
  if (f < F) {
    for (int64_t b = b_lo + g; b < b_hi; b += kXaG) {
      float2 y[M];
#pragma unroll
      for (int i = 0; i < M; i++) y[i] = __ldg(&Y[((int64_t)i * nb + b) * F + f]);
      int p = 0;
#pragma unroll
      for (int i = 0; i < M; i++) {
#pragma unroll
        for (int j = i; j < M; j++, p++) {  // y_i conj(y_j)
          acc[p].x = fmaf(y[i].x, y[j].x, fmaf(y[i].y, y[j].y, acc[p].x));
          acc[p].y = fmaf(y[i].y, y[j].x, fmaf(-y[i].x, y[j].y, acc[p].y));
        }
      }
    }
  }
#pragma unroll
  for (int p = 0; p < NP; p++) part[g][p][fl] = acc[p];
  __syncthreads();
  if (f >= F) return;
  const bool bad = fault && *fault;
  for (int p = g; p < NP; p += kXaG) {
    float2 t = part[0][p][fl];
    for (int q = 1; q < kXaG; q++) t = cadd(t, part[q][p][fl]);
    t = cscale(t, scale);
    if (bad) t = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    int i = 0, r = p;
    while (r >= M - i) {
      r -= M - i;
      i++;
    }
    const int j = i + r;
    float2* v = vis + ((int64_t)i * M + j) * F + f;
    *v = cadd(*v, t);
    if (i != j) {
      float2* w = vis + ((int64_t)j * M + i) * F + f;
      *w = cadd(*w, cconj(t));
    }
  }
}

int launch_xcorr_accum(const float2* Y, int M, int64_t nb, int64_t F, int64_t b_lo, int64_t b_hi, float2* vis,
                       float scale, cudaStream_t s, const int* fault) {
  if (b_hi <= b_lo) return AB_OK;
  const dim3 gs((unsigned)((F + kXaF - 1) / kXaF));
  switch (M) {
    case 2: xcorr_accum_small_kernel<2><<<gs, kXaF * kXaG, 0, s>>>(Y, nb, F, b_lo, b_hi, vis, scale, fault); break;
    case 4: xcorr_accum_small_kernel<4><<<gs, kXaF * kXaG, 0, s>>>(Y, nb, F, b_lo, b_hi, vis, scale, fault); break;
    case 6: xcorr_accum_small_kernel<6><<<gs, kXaF * kXaG, 0, s>>>(Y, nb, F, b_lo, b_hi, vis, scale, fault); break;
    default: {
      dim3 grid((unsigned)((F + 127) / 128), (unsigned)(M * (M + 1) / 2));
      xcorr_accum_kernel<<<grid, 128, 0, s>>>(Y, M, nb, F, b_lo, b_hi, vis, scale, fault);
    }
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

// ---------------------------------------------------------------------------
// Coarse integer correlator (tensor cores).
//
// Per channel, the int8 matrix A has one row per (antenna, pol, re|im):
// row 4a + 2p + 0 = Re x_{2a+p}, row 4a + 2p + 1 = Im x_{2a+p}; columns are
// time samples.  G = A A^T is accumulated with mma.sync m16n8k32 (A row-major
// fragment, B = A^T column-major, i.e. both read K-contiguous rows of A).
// Re V_ij = G[r_i, r_j] + G[m_i, m_j];  Im V_ij = G[m_i, r_j] - G[r_i, m_j].
constexpr int kCcThreads = 256;    // 8 warps
constexpr int kCcKT = 64;          // samples per shared-memory tile
constexpr int kCcPitch = kCcKT + 16;  // bytes per A row in smem (bank spread)

__device__ __forceinline__ int dec4i(unsigned v) { return (int)((v + 7u) & 15u) - 7; }

__device__ __forceinline__ void mma_s8(int (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int NT>  // NT = Rp / 8 n-tiles per warp
__global__ void __launch_bounds__(kCcThreads)
    coarse_xcorr_kernel(const uint8_t* __restrict__ raw, int64_t ant_stride, int64_t row_bytes, int nant,
                        int64_t rowstart, int64_t nrows, const int32_t* __restrict__ rows,
                        const int64_t* __restrict__ channels, int ncols, int64_t chunk_rows, int64_t slice,
                        int64_t slices_per_chunk, long long* __restrict__ G) {
  constexpr int Rp = NT * 8;
  constexpr int MT = Rp / 16;                 // m-tiles per channel
  constexpr int FC = (8 / MT) > 0 ? 8 / MT : 1;  // channels per CTA
  extern __shared__ __align__(16) uint8_t As[];  // [FC][Rp][kCcPitch]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int c0 = blockIdx.x * FC;
  const int64_t chunk = blockIdx.y / slices_per_chunk;
  const int64_t sl = blockIdx.y % slices_per_chunk;
  const int64_t k_begin = chunk * chunk_rows + sl * slice;
  int64_t k_end = k_begin + slice;
  const int64_t chunk_end = min((chunk + 1) * chunk_rows, nrows);
  if (k_end > chunk_end) k_end = chunk_end;
  // warp task: channel fc = warp / MT, m-tile mi = warp % MT
  const int fc = warp / MT, mi = warp % MT;
  const bool active = (warp < FC * MT) && (c0 + fc < ncols);
  int acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[j][q] = 0;
  // zero the padding rows once (rows >= 4*nant)
  for (int i = threadIdx.x; i < FC * Rp * kCcPitch; i += blockDim.x) As[i] = 0;
  __syncthreads();
  for (int64_t kt = k_begin; kt < k_end; kt += kCcKT) {
    // decode tile: (fc, a, t) triples
    const int total = FC * nant * kCcKT;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      int t = idx % kCcKT;
      int rest = idx / kCcKT;
      int a = rest % nant, f = rest / nant;
      int64_t k = kt + t;
      unsigned b0 = 0u, b1 = 0u;  // nibble 0 decodes to 0
      if (k < k_end && c0 + f < ncols) {
        int64_t r = rows ? (int64_t)rows[(int64_t)a * nrows + k] : rowstart + k;
        const uint8_t* p = raw + (int64_t)a * ant_stride + r * row_bytes + 2 * channels[c0 + f];
        uchar2 bb = *reinterpret_cast<const uchar2*>(p);
        b0 = bb.x;
        b1 = bb.y;
      }
      uint8_t* base = As + ((size_t)f * Rp + 4 * a) * kCcPitch + t;
      base[0] = (uint8_t)(int8_t)dec4i(b0 >> 4);
      base[kCcPitch] = (uint8_t)(int8_t)dec4i(b0 & 15u);
      base[2 * kCcPitch] = (uint8_t)(int8_t)dec4i(b1 >> 4);
      base[3 * kCcPitch] = (uint8_t)(int8_t)dec4i(b1 & 15u);
    }
    __syncthreads();
    if (active) {
      const uint8_t* Af = As + (size_t)fc * Rp * kCcPitch;
#pragma unroll
      for (int ks = 0; ks < kCcKT; ks += 32) {
        unsigned a[4];
        const uint8_t* ra = Af + (size_t)(mi * 16 + g) * kCcPitch + ks + tig * 4;
        a[0] = *reinterpret_cast<const unsigned*>(ra);
        a[1] = *reinterpret_cast<const unsigned*>(ra + 8 * kCcPitch);
        a[2] = *reinterpret_cast<const unsigned*>(ra + 16);
        a[3] = *reinterpret_cast<const unsigned*>(ra + 8 * kCcPitch + 16);
#pragma unroll
        for (int j = 0; j < NT; j++) {
          const uint8_t* rb = Af + (size_t)(j * 8 + g) * kCcPitch + ks + tig * 4;
          unsigned b0 = *reinterpret_cast<const unsigned*>(rb);
          unsigned b1 = *reinterpret_cast<const unsigned*>(rb + 16);
          mma_s8(acc[j], a, b0, b1);
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
  long long* Gc = G + (((int64_t)chunk * ncols + c0 + fc) * Rp) * Rp;
#pragma unroll
  for (int j = 0; j < NT; j++) {
    int row = mi * 16 + g, col = j * 8 + tig * 2;
    atomicAdd((unsigned long long*)&Gc[(int64_t)row * Rp + col], (unsigned long long)(long long)acc[j][0]);
    atomicAdd((unsigned long long*)&Gc[(int64_t)row * Rp + col + 1], (unsigned long long)(long long)acc[j][1]);
    atomicAdd((unsigned long long*)&Gc[(int64_t)(row + 8) * Rp + col], (unsigned long long)(long long)acc[j][2]);
    atomicAdd((unsigned long long*)&Gc[(int64_t)(row + 8) * Rp + col + 1], (unsigned long long)(long long)acc[j][3]);
  }
}

// FP16 form of the same Gram matrix.  The decoded values are integers in
// [-7, 8] (nibble 0x8 is +8), exact in fp16; mma.sync m16n8k16 multiplies them exactly and
// accumulates in fp32, which stays exact while |sum| < 2^24: a CTA slice of
// at most 4096 samples sums at most 4096 * 64 = 2^18.  The fp32 partials are
// converted to int64 exactly and flushed with int64 atomics, as in the int8
// form.  (The fp16 tensor path has a much higher rate than the int8 one on
// this part.)
__device__ __forceinline__ void mma_f16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kCcPitchH = kCcKT + 8;  // halves per A row in smem (conflict-free fragment loads)

template <int NT>
__global__ void __launch_bounds__(kCcThreads)
    coarse_xcorr_f16_kernel(const uint8_t* __restrict__ raw, int64_t ant_stride, int64_t row_bytes, int nant,
                            int64_t rowstart, int64_t nrows, const int32_t* __restrict__ rows,
                            const int64_t* __restrict__ channels, int ncols, int64_t chunk_rows, int64_t slice,
                            int64_t slices_per_chunk, long long* __restrict__ G) {
  constexpr int Rp = NT * 8;
  constexpr int MT = Rp / 16;
  constexpr int FC = (8 / MT) > 0 ? 8 / MT : 1;
  extern __shared__ __align__(16) unsigned short Ah[];  // fp16 bits, [FC][Rp][kCcPitchH]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int c0 = blockIdx.x * FC;
  const int64_t chunk = blockIdx.y / slices_per_chunk;
  const int64_t sl = blockIdx.y % slices_per_chunk;
  const int64_t k_begin = chunk * chunk_rows + sl * slice;
  int64_t k_end = k_begin + slice;
  const int64_t chunk_end = min((chunk + 1) * chunk_rows, nrows);
  if (k_end > chunk_end) k_end = chunk_end;
  const int fc = warp / MT, mi = warp % MT;
  const bool active = (warp < FC * MT) && (c0 + fc < ncols);
  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[j][q] = 0.f;
  for (int i = threadIdx.x; i < FC * Rp * kCcPitchH; i += blockDim.x) Ah[i] = 0;
  __syncthreads();
  auto h16 = [](int v) -> unsigned short { return __half_as_ushort(__int2half_rn(v)); };
  for (int64_t kt = k_begin; kt < k_end; kt += kCcKT) {
    const int total = FC * nant * kCcKT;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      int t = idx % kCcKT;
      int rest = idx / kCcKT;
      int a = rest % nant, f = rest / nant;
      int64_t k = kt + t;
      unsigned b0 = 0u, b1 = 0u;
      if (k < k_end && c0 + f < ncols) {
        int64_t r = rows ? (int64_t)rows[(int64_t)a * nrows + k] : rowstart + k;
        const uint8_t* p = raw + (int64_t)a * ant_stride + r * row_bytes + 2 * channels[c0 + f];
        uchar2 bb = *reinterpret_cast<const uchar2*>(p);
        b0 = bb.x;
        b1 = bb.y;
      }
      unsigned short* base = Ah + ((size_t)f * Rp + 4 * a) * kCcPitchH + t;
      base[0] = h16(dec4i(b0 >> 4));
      base[kCcPitchH] = h16(dec4i(b0 & 15u));
      base[2 * kCcPitchH] = h16(dec4i(b1 >> 4));
      base[3 * kCcPitchH] = h16(dec4i(b1 & 15u));
    }
    __syncthreads();
    if (active) {
      const unsigned short* Af = Ah + (size_t)fc * Rp * kCcPitchH;
#pragma unroll
      for (int ks = 0; ks < kCcKT; ks += 16) {
        unsigned a[4];
        const unsigned short* ra = Af + (size_t)(mi * 16 + g) * kCcPitchH + ks + tig * 2;
        a[0] = *reinterpret_cast<const unsigned*>(ra);
        a[1] = *reinterpret_cast<const unsigned*>(ra + 8 * kCcPitchH);
        a[2] = *reinterpret_cast<const unsigned*>(ra + 8);
        a[3] = *reinterpret_cast<const unsigned*>(ra + 8 * kCcPitchH + 8);
#pragma unroll
        for (int j = 0; j < NT; j++) {
          const unsigned short* rb = Af + (size_t)(j * 8 + g) * kCcPitchH + ks + tig * 2;
          mma_f16(acc[j], a, *reinterpret_cast<const unsigned*>(rb), *reinterpret_cast<const unsigned*>(rb + 8));
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
  long long* Gc = G + (((int64_t)chunk * ncols + c0 + fc) * Rp) * Rp;
#pragma unroll
  for (int j = 0; j < NT; j++) {
    int row = mi * 16 + g, col = j * 8 + tig * 2;
    atomicAdd((unsigned long long*)&Gc[(int64_t)row * Rp + col], (unsigned long long)__float2ll_rn(acc[j][0]));
    atomicAdd((unsigned long long*)&Gc[(int64_t)row * Rp + col + 1], (unsigned long long)__float2ll_rn(acc[j][1]));
    atomicAdd((unsigned long long*)&Gc[(int64_t)(row + 8) * Rp + col], (unsigned long long)__float2ll_rn(acc[j][2]));
    atomicAdd((unsigned long long*)&Gc[(int64_t)(row + 8) * Rp + col + 1],
              (unsigned long long)__float2ll_rn(acc[j][3]));
  }
}

// fault: the tensor-core form's fault word (or null); when set, every output
// of the call is INT64_MIN.
__global__ void coarse_finalize_kernel(const long long* __restrict__ G, int Rp, int M, int ncols, int64_t nchunks,
                                       int64_t* __restrict__ re, int64_t* __restrict__ im,
                                       const int* __restrict__ fault) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = nchunks * M * M * ncols;
  if (idx >= total) return;
  if (fault && *fault) {
    re[idx] = INT64_MIN;
    im[idx] = INT64_MIN;
    return;
  }
  int64_t k = idx % ncols;
  int64_t r = idx / ncols;
  int j = (int)(r % M);
  r /= M;
  int i = (int)(r % M);
  int64_t ch = r / M;
  const long long* Gc = G + ((ch * ncols + k) * Rp) * Rp;
  int ri = 2 * i, mi_ = 2 * i + 1, rj = 2 * j, mj = 2 * j + 1;  // row of (2a+p) re = 4a+2p = 2i
  re[idx] = Gc[(int64_t)ri * Rp + rj] + Gc[(int64_t)mi_ * Rp + mj];
  im[idx] = Gc[(int64_t)mi_ * Rp + rj] - Gc[(int64_t)ri * Rp + mj];
}

// ---------------------------------------------------------------------------
// Pairwise correlators on sortpols'd bytes.
__global__ void pairs4_kernel(const uint8_t* __restrict__ d0, const uint8_t* __restrict__ d1,
                              const int32_t* __restrict__ r0, const int32_t* __restrict__ r1, int64_t nmatch,
                              int64_t ncol, int64_t rows_per_block, long long* __restrict__ re,
                              long long* __restrict__ im) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ncol) return;
  int64_t lo = (int64_t)blockIdx.y * rows_per_block, hi = min(lo + rows_per_block, nmatch);
  int sr = 0, si = 0;
  for (int64_t m = lo; m < hi; m++) {
    int64_t a = r0 ? r0[m] : m, b = r1 ? r1[m] : m;
    unsigned x = d0[a * ncol + k], y = d1[b * ncol + k];
    int xr = dec4i(x >> 4), xi = dec4i(x & 15u), yr = dec4i(y >> 4), yi = dec4i(y & 15u);
    sr += xr * yr + xi * yi;
    si += yr * xi - xr * yi;
  }
  if (hi > lo) {
    atomicAdd((unsigned long long*)&re[k], (unsigned long long)(long long)sr);
    atomicAdd((unsigned long long*)&im[k], (unsigned long long)(long long)si);
  }
}

__global__ void pairs1_kernel(const uint8_t* __restrict__ d0, const uint8_t* __restrict__ d1,
                              const int32_t* __restrict__ r0, const int32_t* __restrict__ r1, int64_t nmatch,
                              int64_t ncol, int64_t nchan, int64_t rows_per_block, long long* __restrict__ sums) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchan) return;
  int64_t lo = (int64_t)blockIdx.y * rows_per_block, hi = min(lo + rows_per_block, nmatch);
  int s[6] = {0, 0, 0, 0, 0, 0};
  const int sh = 6 - 2 * (int)(c % 4);
  const int64_t byte = c / 4;
  for (int64_t m = lo; m < hi; m++) {
    int64_t a = r0 ? r0[m] : m, b = r1 ? r1[m] : m;
    unsigned x = d0[a * ncol + byte], y = d1[b * ncol + byte];
    int ar = (x >> (sh + 1)) & 1, ai = (x >> sh) & 1, br = (y >> (sh + 1)) & 1, bi = (y >> sh) & 1;
    s[0] += 2 - 2 * ((ar ^ br) + (ai ^ bi));
    s[1] += -2 * ((br ^ ai) - (ar ^ bi));
    s[2] += 1 - 2 * (ar ^ br);
    s[3] += 1 - 2 * (ai ^ bi);
    s[4] += 1 - 2 * (ar ^ bi);
    s[5] += 1 - 2 * (br ^ ai);
  }
  if (hi > lo)
    for (int q = 0; q < 6; q++) atomicAdd((unsigned long long*)&sums[q * nchan + c], (unsigned long long)(long long)s[q]);
}

}  // namespace ab

using namespace ab;

extern "C" int ab_avg_xcorr_all_ant(const float* x, int64_t nant, int64_t npol, int64_t ntime, int64_t nfreq,
                                    float* out, void* stream) {
  AB_CHECK_ARG(x && out, "ab_avg_xcorr_all_ant: NULL pointer");
  AB_CHECK_ARG(nant >= 1 && npol >= 1 && ntime >= 1 && nfreq >= 0, "ab_avg_xcorr_all_ant: bad sizes");
  int M = (int)(nant * npol);
  if (nfreq == 0) return AB_OK;
  AB_CHECK_ARG(nfreq <= 0x7fffffff, "ab_avg_xcorr_all_ant: nfreq too large");
  int ntile = (M + kXcTile - 1) / kXcTile;
  AB_CHECK_ARG(ntile * ntile <= 65535, "ab_avg_xcorr_all_ant: M=%d too large", M);
  dim3 grid((unsigned)nfreq, (unsigned)(ntile * ntile));
  xcorr_fine_kernel<<<grid, kXcThreads, 0, as_stream(stream)>>>((const float2*)x, M, ntime, nfreq, (float2*)out,
                                                               1.0f / (float)ntime);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

namespace ab {
int launch_coarse_tc(ab_ctx* ctx, const uint8_t* raw, int64_t ant_stride, int64_t nant, int64_t nchan,
                     int64_t rowstart, int64_t nrows, const int32_t* rows, const int64_t* channels, int64_t ncols,
                     int64_t chunk_rows, int Rp, long long* G, int* fault, cudaStream_t s);

// Largest channel count of one coarse-correlator call (grid x stays far below
// its limit, and the scratch size below cannot wrap).
constexpr int64_t kCoarseMaxCols = 1 << 20;

int coarse_xcorr_run(ab_ctx* ctx, const uint8_t* raw, int64_t ant_stride, int64_t nant, int64_t nchan,
                     int64_t rowstart, int64_t nrows, const int32_t* rows, const int64_t* channels, int64_t ncols,
                     int64_t chunk_rows, long long* G, int64_t* out_re, int64_t* out_im, cudaStream_t s) {
  const int R = (int)(4 * nant);
  const int Rp = ((R + 15) / 16) * 16;
  const int NT = Rp / 8;
  const int MT = Rp / 16;
  const int FC = (8 / MT) > 0 ? 8 / MT : 1;
  const int64_t nchunks = (nrows + chunk_rows - 1) / chunk_rows;
  int64_t slice = 4096;
  if (slice > chunk_rows) slice = ((chunk_rows + kCcKT - 1) / kCcKT) * kCcKT;
  const int64_t spc = (chunk_rows + slice - 1) / slice;
  size_t gbytes = sizeof(long long) * (size_t)(nchunks * ncols) * Rp * Rp;
  AB_CUDA(cudaMemsetAsync(G, 0, gbytes, s));
  const int M = (int)(2 * nant);
  // tensor-core (tcgen05) form: by default from 9 antennas up (where its
  // 128-row tiles are mostly filled), on request for any count up to 32;
  // only through a context (the allocation-free entry point keeps the
  // warp-level form)
  const int engine = ctx ? ctx->coarse_engine : 1;
  if (ctx && ctx->coarse_f16 && nant <= 32 && (engine == 2 || (engine == 0 && nant >= 9))) {
    void* fw = nullptr;
    AB_TRY(get_scratch(ctx, kScratchFault, 256, &fw));
    AB_CUDA(cudaMemsetAsync(fw, 0, sizeof(int), s));
    AB_TRY(launch_coarse_tc(ctx, raw, ant_stride, nant, nchan, rowstart, nrows, rows, channels, ncols, chunk_rows,
                            Rp, G, (int*)fw, s));
    const int64_t total = nchunks * M * M * ncols;
    coarse_finalize_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(G, Rp, M, (int)ncols, nchunks, out_re,
                                                                           out_im, (const int*)fw);
    AB_LAUNCH_CHECK();
    return AB_OK;
  }
  size_t smem = (size_t)FC * Rp * kCcPitch;
  AB_CHECK_ARG(nchunks * spc <= 0x7fffffff, "coarse xcorr: too many slices");
  dim3 grid((unsigned)((ncols + FC - 1) / FC), (unsigned)(nchunks * spc));
  AB_CHECK_ARG(grid.y <= 65535, "coarse xcorr: %u time slices exceed the grid limit; use larger chunks", grid.y);
  const bool f16 = !ctx || ctx->coarse_f16;
  const size_t smem16 = sizeof(unsigned short) * (size_t)FC * Rp * kCcPitchH;
#define AB_CC(NTV)                                                                                           \
  case NTV:                                                                                                  \
    if (f16) {                                                                                               \
      AB_CUDA(cudaFuncSetAttribute(coarse_xcorr_f16_kernel<NTV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                   (int)smem16));                                                            \
      coarse_xcorr_f16_kernel<NTV><<<grid, kCcThreads, smem16, s>>>(raw, ant_stride, 2 * nchan, (int)nant,     \
                                                                    rowstart, nrows, rows, channels,          \
                                                                    (int)ncols, chunk_rows, slice, spc, G);   \
    } else {                                                                                                 \
      AB_CUDA(cudaFuncSetAttribute(coarse_xcorr_kernel<NTV>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                   (int)smem));                                                              \
      coarse_xcorr_kernel<NTV><<<grid, kCcThreads, smem, s>>>(raw, ant_stride, 2 * nchan, (int)nant, rowstart, \
                                                              nrows, rows, channels, (int)ncols, chunk_rows,  \
                                                              slice, spc, G);                                 \
    }                                                                                                        \
    break;
  switch (NT) {
    AB_CC(2)
    AB_CC(4)
    AB_CC(6)
    AB_CC(8)
    AB_CC(10)
    AB_CC(12)
    AB_CC(14)
    AB_CC(16)
    default:
      set_error("coarse xcorr: nant=%lld unsupported (max 32)", (long long)nant);
      return AB_ERR_UNSUPPORTED;
  }
#undef AB_CC
  AB_LAUNCH_CHECK();
  int64_t total = nchunks * M * M * ncols;
  coarse_finalize_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(G, Rp, M, (int)ncols, nchunks, out_re,
                                                                         out_im, nullptr);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

// Bytes of int64 partial sums one call needs, or 0 when that count would not
// fit in 62 bits (absurd channel or chunk counts); callers reject 0.
size_t coarse_xcorr_scratch_bytes(int64_t nant, int64_t nrows, int64_t ncols, int64_t chunk_rows) {
  const int R = (int)(4 * nant);
  const int Rp = ((R + 15) / 16) * 16;
  if (nrows < 1 || chunk_rows < 1 || ncols < 1 || ncols > kCoarseMaxCols) return 0;
  const unsigned long long nchunks = (unsigned long long)((nrows + chunk_rows - 1) / chunk_rows);
  const unsigned long long per_chunk = sizeof(long long) * (unsigned long long)Rp * Rp * (unsigned long long)ncols;
  if (nchunks > (1ull << 62) / per_chunk) return 0;
  return (size_t)(per_chunk * nchunks);
}
}  // namespace ab

extern "C" int ab_xcorr_coarse_4bit(ab_ctx* ctx, const uint8_t* raw, int64_t ant_stride, int64_t nant, int64_t nspec,
                                    int64_t nchan, int64_t rowstart, int64_t nrows, const int32_t* rows,
                                    const int64_t* channels, int64_t ncols, int64_t chunk_rows, int64_t* out_re,
                                    int64_t* out_im, void* stream) {
  AB_CHECK_ARG(ctx && raw && channels && out_re && out_im, "ab_xcorr_coarse_4bit: NULL pointer");
  AB_CHECK_ARG(nant >= 1 && nant <= 32 && nchan >= 1 && ncols >= 1 && nrows >= 1,
               "ab_xcorr_coarse_4bit: bad sizes (1 <= nant <= 32)");
  AB_CHECK_ARG(rows || (rowstart >= 0 && rowstart + nrows <= nspec), "ab_xcorr_coarse_4bit: rows out of range");
  AB_CHECK_ARG(ant_stride >= nspec * 2 * nchan || nant == 1, "ab_xcorr_coarse_4bit: antenna stride too small");
  if (chunk_rows <= 0 || chunk_rows > nrows) chunk_rows = nrows;
  AB_CHECK_ARG(chunk_rows <= (1ll << 24), "ab_xcorr_coarse_4bit: chunk_rows must be <= 2^24 (int32 partials)");
  const size_t need = coarse_xcorr_scratch_bytes(nant, nrows, ncols, chunk_rows);
  AB_CHECK_ARG(need > 0, "ab_xcorr_coarse_4bit: %lld channels in %lld chunks is too large (at most %lld channels)",
               (long long)ncols, (long long)((nrows + chunk_rows - 1) / chunk_rows), (long long)kCoarseMaxCols);
  void* G = nullptr;
  AB_TRY(get_scratch(ctx, kScratchXcorrG, need, &G));
  return coarse_xcorr_run(ctx, raw, ant_stride, nant, nchan, rowstart, nrows, rows, channels, ncols, chunk_rows,
                          (long long*)G, out_re, out_im, as_stream(stream));
}

// ---------------------------------------------------------------------------
// Allocation-free coarse correlator.
//
// Some callers cannot allocate device memory while they run: a correlator
// service that reserves its whole device-memory budget at start-up and must
// not grow it, a host application whose own allocator owns the device memory
// and forbids raw cudaMalloc, or a latency-critical loop where an allocation
// (which can synchronise the device or fail under memory pressure) is not
// acceptable.  For them this entry point keeps its int64 partial sums in a
// fixed buffer compiled into the library instead of the context's scratch.
//
// The buffer is a file-scope __device__ array of kNoAllocScratchBytes (16 MiB);
// every GPU that loads this library holds it until the process exits.  In
// host code the array's name is only a host-side stand-in, so its device
// address is fetched with cudaGetSymbolAddress, with that device current, by
// every call made outside stream capture; a call made while its stream is
// being captured uses the address the last uncaptured call on that device
// found, so the first call on a device must come before any stream capture.
// All calls share the one buffer: the entry point clears it at the start of
// every call, and calls whose work overlaps on the GPU (different streams, or
// several host threads on one device) race on it.
constexpr size_t kNoAllocScratchBytes = 16u << 20;
static __device__ __align__(256) long long g_noalloc_scratch[kNoAllocScratchBytes / sizeof(long long)];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[128] = {nullptr};
}  // namespace

extern "C" int ab_xcorr_coarse_4bit_noalloc(const uint8_t* raw, int64_t ant_stride, int64_t nant, int64_t nspec,
                                            int64_t nchan, int64_t rowstart, int64_t nrows, const int32_t* rows,
                                            const int64_t* channels, int64_t ncols, int64_t chunk_rows,
                                            int64_t* out_re, int64_t* out_im, void* stream) {
  AB_CHECK_ARG(raw && channels && out_re && out_im, "ab_xcorr_coarse_4bit_noalloc: NULL pointer");
  AB_CHECK_ARG(nant >= 1 && nant <= 32 && nchan >= 1 && ncols >= 1 && nrows >= 1,
               "ab_xcorr_coarse_4bit_noalloc: bad sizes (1 <= nant <= 32)");
  AB_CHECK_ARG(rows || (rowstart >= 0 && rowstart + nrows <= nspec), "ab_xcorr_coarse_4bit_noalloc: rows out of range");
  AB_CHECK_ARG(ant_stride >= nspec * 2 * nchan || nant == 1, "ab_xcorr_coarse_4bit_noalloc: antenna stride too small");
  if (chunk_rows <= 0 || chunk_rows > nrows) chunk_rows = nrows;
  AB_CHECK_ARG(chunk_rows <= (1ll << 24), "ab_xcorr_coarse_4bit_noalloc: chunk_rows must be <= 2^24");
  const size_t need = coarse_xcorr_scratch_bytes(nant, nrows, ncols, chunk_rows);
  AB_CHECK_ARG(need > 0 && need <= kNoAllocScratchBytes,
               "ab_xcorr_coarse_4bit_noalloc: this call needs %zu bytes of scratch but the built-in buffer holds "
               "%zu; split it into calls with fewer channels or chunks, or use ab_xcorr_coarse_4bit",
               need, kNoAllocScratchBytes);
  int dev = 0;
  AB_CUDA(cudaGetDevice(&dev));
  AB_CHECK_ARG(dev >= 0 && dev < 128, "ab_xcorr_coarse_4bit_noalloc: device index %d out of range", dev);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  AB_CUDA(cudaStreamIsCapturing(as_stream(stream), &cap));
  void* G = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (cap == cudaStreamCaptureStatusNone) {
      // Outside capture the address is looked up on every call: after a
      // device reset, or with another context current on this device, the
      // module (and the buffer) may sit somewhere else than last time.
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        set_error("ab_xcorr_coarse_4bit_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return AB_ERR_CUDA;
      }
      g_noalloc_addr[dev] = p;
    } else if (!g_noalloc_addr[dev]) {
      set_error("ab_xcorr_coarse_4bit_noalloc: the first call on device %d must come before any stream capture", dev);
      return AB_ERR_ARG;
    }
    G = g_noalloc_addr[dev];
  }
  return coarse_xcorr_run(nullptr, raw, ant_stride, nant, nchan, rowstart, nrows, rows, channels, ncols, chunk_rows,
                          (long long*)G, out_re, out_im, as_stream(stream));
}

extern "C" int ab_avg_xcorr_4bit_pairs(const uint8_t* data0, const uint8_t* data1, const int32_t* rows0,
                                       const int32_t* rows1, int64_t nmatch, int64_t ncol, int64_t* re, int64_t* im,
                                       void* stream) {
  AB_CHECK_ARG(data0 && data1 && re && im && nmatch >= 0 && ncol >= 1, "ab_avg_xcorr_4bit_pairs: bad arguments");
  cudaStream_t s = as_stream(stream);
  AB_CUDA(cudaMemsetAsync(re, 0, sizeof(int64_t) * (size_t)ncol, s));
  AB_CUDA(cudaMemsetAsync(im, 0, sizeof(int64_t) * (size_t)ncol, s));
  if (nmatch == 0) return AB_OK;
  int64_t rpb = 2048;
  dim3 grid((unsigned)((ncol + 127) / 128), (unsigned)((nmatch + rpb - 1) / rpb));
  AB_CHECK_ARG(grid.y <= 65535, "ab_avg_xcorr_4bit_pairs: too many rows");
  pairs4_kernel<<<grid, 128, 0, s>>>(data0, data1, rows0, rows1, nmatch, ncol, rpb, (long long*)re, (long long*)im);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_avg_xcorr_1bit_pairs(const uint8_t* data0, const uint8_t* data1, const int32_t* rows0,
                                       const int32_t* rows1, int64_t nmatch, int64_t ncol, int64_t nchan, int64_t* sums,
                                       void* stream) {
  AB_CHECK_ARG(data0 && data1 && sums && nmatch >= 0 && ncol >= 1 && nchan >= 1 && nchan <= 4 * ncol,
               "ab_avg_xcorr_1bit_pairs: bad arguments");
  cudaStream_t s = as_stream(stream);
  AB_CUDA(cudaMemsetAsync(sums, 0, sizeof(int64_t) * 6 * (size_t)nchan, s));
  if (nmatch == 0) return AB_OK;
  int64_t rpb = 2048;
  dim3 grid((unsigned)((nchan + 127) / 128), (unsigned)((nmatch + rpb - 1) / rpb));
  AB_CHECK_ARG(grid.y <= 65535, "ab_avg_xcorr_1bit_pairs: too many rows");
  pairs1_kernel<<<grid, 128, 0, s>>>(data0, data1, rows0, rows1, nmatch, ncol, nchan, rpb, (long long*)sums);
  AB_LAUNCH_CHECK();
  return AB_OK;
}
