// fft_static.cuh -- compile-time-planned in-place FFT passes on shared memory.
//
// Same transform conventions as fft.cuh (dif: natural -> digit-reversed,
// dit: the adjoint), but the radix and span of every pass are template
// constants, so index arithmetic uses constant divisors and loop trip counts
// are known, and the twiddles of each pass are read from a "twiddle stream":
// a global table laid out in the order the pass consumes it,
//     stream_q[(k-1) * S_q + j] = exp(-2 pi i j k / (R_q S_q)),
// so that consecutive threads (consecutive j) read consecutive addresses.
// The streams are built on the host in double precision and rounded once.
#pragma once
#include "fft.cuh"

namespace ab {

// radix-16 DFT as 4 x 4 with the internal twiddles exp(-2 pi i a b / 16)
template <bool INV>
__device__ __forceinline__ void dft16(float2* x) {
  const float c1 = 0.9238795325112867f, s1 = 0.3826834323650898f, h = 0.7071067811865476f;
  // stage 1: 4 DFT4 over stride-4 subsequences x[a + 4 b]
  float2 y[16];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    float2 t[4] = {x[a], x[a + 4], x[a + 8], x[a + 12]};
    dft4<INV>(t);
#pragma unroll
    for (int k = 0; k < 4; k++) y[a * 4 + k] = t[k];  // y[a][k]
  }
  // twiddle y[a][k] by w16^(a k) (forward w16 = exp(-i pi / 8))
  auto tw = [&](float2 v, float c, float s) -> float2 {  // v * (c - i s) forward, (c + i s) inverse
    return INV ? make_float2(v.x * c - v.y * s, v.x * s + v.y * c) : make_float2(v.x * c + v.y * s, v.y * c - v.x * s);
  };
  y[1 * 4 + 1] = tw(y[5], c1, s1);
  y[1 * 4 + 2] = tw(y[6], h, h);
  y[1 * 4 + 3] = tw(y[7], s1, c1);
  y[2 * 4 + 1] = tw(y[9], h, h);
  y[2 * 4 + 2] = mul_mi<INV>(y[10]);
  y[2 * 4 + 3] = tw(y[11], -h, h);
  y[3 * 4 + 1] = tw(y[13], s1, c1);
  y[3 * 4 + 2] = tw(y[14], -h, h);
  y[3 * 4 + 3] = tw(y[15], -c1, -s1);
  // stage 2: DFT4 over a for each k; output index k + 4 k2
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float2 t[4] = {y[k], y[4 + k], y[8 + k], y[12 + k]};
    dft4<INV>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) x[k + 4 * k2] = t[k2];
  }
}

template <int R, bool INV>
__device__ __forceinline__ void dft_any(float2* x) {
  if constexpr (R == 16) dft16<INV>(x);
  else dft_small<R, INV>(x);
}

// compile-time plan: N points, radices Rs... applied in order
template <int N_, int... Rs>
struct SPlan {
  static constexpr int N = N_;
  static constexpr int NP = sizeof...(Rs);
  static constexpr int R[NP] = {Rs...};
  static constexpr int span(int q) {
    int prod = 1;
    for (int i = 0; i <= q; i++) prod *= R[i];
    return N / prod;
  }
  // offset of pass q's twiddle stream
  static constexpr int tw_off(int q) {
    int off = 0;
    for (int i = 0; i < q; i++) off += (R[i] - 1) * span(i);
    return off;
  }
  static constexpr int tw_len() { return tw_off(NP); }
  static constexpr bool valid() {
    int prod = 1;
    for (int i = 0; i < NP; i++) prod *= R[i];
    return prod == N;
  }
};

// TWS: the twiddle stream lies in shared memory (plain loads) instead of
// global memory (read-only cache loads)
template <int R, int S, int N, int NTHR, bool INV, bool TWS = false>
__device__ __forceinline__ void spass(float2* buf, const float2* __restrict__ tws, int tid) {
  constexpr int NBF = N / R;
#pragma unroll 1
  for (int bf = tid; bf < NBF; bf += NTHR) {
    const int blk = bf / S, j = bf - (bf / S) * S;
    const int base = blk * (R * S) + j;
    // padded addresses: pidx(base + r S) = pidx(base) + r (S + S/16) when 16 | S,
    // and pidx(base) + r when S = 1 and R | 16 (base is then a multiple of R)
    const int pb = pidx(base);
    auto addr = [&](int r) -> int {
      if constexpr (S % 16 == 0) return pb + r * (S + S / 16);
      else if constexpr (S == 1 && 16 % R == 0) return pb + r;
      else return pidx(base + r * S);
    };
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = buf[addr(r)];
    if constexpr (INV) {
      if (S > 1 && j) {
#pragma unroll
        for (int k = 1; k < R; k++) x[k] = cmulc(x[k], TWS ? tws[(k - 1) * S + j] : __ldg(&tws[(k - 1) * S + j]));
      }
      dft_any<R, true>(x);
    } else {
      dft_any<R, false>(x);
      if (S > 1 && j) {
#pragma unroll
        for (int k = 1; k < R; k++) x[k] = cmul(x[k], TWS ? tws[(k - 1) * S + j] : __ldg(&tws[(k - 1) * S + j]));
      }
    }
#pragma unroll
    for (int k = 0; k < R; k++) buf[addr(k)] = x[k];
  }
}

template <class PL, int NTHR, int q>
__device__ __forceinline__ void sdif_from(float2* buf, const float2* tw, int tid) {
  if constexpr (q < PL::NP) {
    spass<PL::R[q], PL::span(q), PL::N, NTHR, false>(buf, tw + PL::tw_off(q), tid);
    __syncthreads();
    sdif_from<PL, NTHR, q + 1>(buf, tw, tid);
  }
}

template <class PL, int NTHR, int q, bool TWS = false>
__device__ __forceinline__ void sdit_from(float2* buf, const float2* tw, int tid) {
  if constexpr (q >= 0) {
    spass<PL::R[q], PL::span(q), PL::N, NTHR, true, TWS>(buf, tw + PL::tw_off(q), tid);
    __syncthreads();
    sdit_from<PL, NTHR, q - 1, TWS>(buf, tw, tid);
  }
}

// forward (natural -> digit-reversed), padded buffer; caller syncs before
template <class PL, int NTHR>
__device__ __forceinline__ void sdif(float2* buf, const float2* tw, int tid) {
  sdif_from<PL, NTHR, 0>(buf, tw, tid);
}
// inverse unnormalised (digit-reversed -> natural)
template <class PL, int NTHR, bool TWS = false>
__device__ __forceinline__ void sdit(float2* buf, const float2* tw, int tid) {
  sdit_from<PL, NTHR, PL::NP - 1, TWS>(buf, tw, tid);
}

// position of frequency f after sdif
template <class PL, int q = 0>
__device__ __forceinline__ int spos(int f) {
  if constexpr (q < PL::NP) {
    constexpr int R = PL::R[q];
    return (f % R) * PL::span(q) + spos<PL, q + 1>(f / R);
  } else {
    return 0;
  }
}

// plans used by the hot kernels
using Plan4096 = SPlan<4096, 16, 16, 16>;
// radix orders chosen so every span is a multiple of 16 (or 1 with R | 16):
// constant padded offsets and conflict-free shared-memory access
using Plan16464 = SPlan<16464, 7, 7, 7, 3, 16>;  // nslice 32928 (acclen 2^15, cut 80)
using Plan16384 = SPlan<16384, 4, 16, 16, 16>;   // nslice 32768

}  // namespace ab
