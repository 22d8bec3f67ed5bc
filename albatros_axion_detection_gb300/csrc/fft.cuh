// fft.cuh -- in-place mixed-radix FFT passes on shared memory, and small
// register FFTs, for the IPFB / PFB kernels.
//
// Shared-memory transforms (one CTA owns one sequence of length n):
//   * dif_forward: natural-order input -> spectrum in digit-reversed order
//     (Sande-Tukey decimation in frequency, radices R_1..R_m applied in order);
//   * dit_inverse: the adjoint sequence of passes, digit-reversed input ->
//     natural-order output of the unnormalised inverse DFT.
// Running dif_forward, a pointwise operation addressed through
// fft_pos(), then dit_inverse needs no permutation pass at all.
//
// Position of frequency f after dif_forward: write f in mixed radix with R_1
// as the least significant digit, f = f_1 + R_1 f_2 + R_1 R_2 f_3 + ...; then
// pos(f) = sum_p f_p * S_p with S_p = n / (R_1 ... R_p).
//
// Twiddles come from a table tw[e] = exp(-2 pi i e / T) for e in [0, T)
// (T a multiple of n), computed on the host in double precision and rounded
// to float once.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ab {

constexpr int kMaxPasses = 12;

// A prime radix R run by Bluestein's method: the length-R DFT as a chirp
// multiply, a circular convolution of length L (7-smooth, L >= 2R - 1) by
// this library's FFT in shared memory, and a chirp multiply back:
//   X_k = c_k sum_r (x_r c_r) conj(c_(k-r)),  c_m = exp(-i pi m^2 / R).
struct BluesteinPass {
  int R, L;                   // the prime radix (0: none) and the convolution length
  int npass;                  // L's plan
  int radix[kMaxPasses];
  int span[kMaxPasses];
  const float2* chirp;        // c_(e) for e in [0, 2R): exp(-i pi e / R), indexed by m^2 mod 2R
  const float2* filt;         // FFT_L of conj(c) wrapped to length L, / L, at L's storage positions
  const float2* twL;          // exp(-2 pi i e / L), e < L
};

struct FftPlan {
  int n;                  // transform length (complex points)
  int npass;
  int radix[kMaxPasses];  // R_p
  int span[kMaxPasses];   // S_p = n / (R_1 .. R_p)
  // Radices other than 2, 3, 4, 5, 7, 8 (prime factors the register
  // butterflies do not cover) run as direct DFT passes, whose outputs go
  // through this global scratch: n complex per CTA, CTA (x, y) at
  // gscratch + (y * gridDim.x + x) * n.  Null for plans without them.
  float2* gscratch;
  // The prime radix bs.R (if any) runs as a Bluestein pass in a shared
  // scratch of padded_len(bs.L) float2 (the caller's sscratch).
  BluesteinPass bs;
};

// 32-byte store of 8 floats (one whole sector), p 32-byte aligned
__device__ __forceinline__ void st_global_v8(float* p, float a0, float a1, float a2, float a3, float a4, float a5,
                                             float a6, float a7) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};\n" ::"l"(p), "f"(a0), "f"(a1), "f"(a2),
               "f"(a3), "f"(a4), "f"(a5), "f"(a6), "f"(a7)
               : "memory");
}

// Asynchronous global -> shared copies (cp.async): 4 bytes through L1, 16
// bytes bypassing it; commit closes a group, wait<N> leaves at most N of this
// thread's groups in flight.
template <class T>
__device__ __forceinline__ void cp_async4(T* dst, const T* src) {
  static_assert(sizeof(T) == 4, "4-byte elements");
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---- small DFTs in registers, forward uses exp(-2 pi i rk / R) ----------
template <bool INV>
__device__ __forceinline__ void dft2(float2* x) {
  float2 a = x[0], b = x[1];
  x[0] = cadd(a, b);
  x[1] = csub(a, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2* x) {
  float2 s02 = cadd(x[0], x[2]), d02 = csub(x[0], x[2]);
  float2 s13 = cadd(x[1], x[3]), d13 = mul_mi<INV>(csub(x[1], x[3]));
  x[0] = cadd(s02, s13);
  x[2] = csub(s02, s13);
  x[1] = cadd(d02, d13);
  x[3] = csub(d02, d13);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2* x) {
  const float h = 0.7071067811865476f;
  float2 a[4] = {x[0], x[2], x[4], x[6]}, b[4] = {x[1], x[3], x[5], x[7]};
  dft4<INV>(a);
  dft4<INV>(b);
  // twiddles w8^k, k = 0..3 (forward w8 = exp(-i pi/4))
  float2 b1 = INV ? make_float2(h * (b[1].x - b[1].y), h * (b[1].x + b[1].y))
                  : make_float2(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));
  float2 b2 = mul_mi<INV>(b[2]);
  float2 b3 = INV ? make_float2(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y))
                  : make_float2(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));
  x[0] = cadd(a[0], b[0]);
  x[4] = csub(a[0], b[0]);
  x[1] = cadd(a[1], b1);
  x[5] = csub(a[1], b1);
  x[2] = cadd(a[2], b2);
  x[6] = csub(a[2], b2);
  x[3] = cadd(a[3], b3);
  x[7] = csub(a[3], b3);
}

// odd prime R: y_k = x0 + sum_r a_r cos(2pi rk/R) -/+ i sum_r b_r sin(2pi rk/R)
template <int R, bool INV>
__device__ __forceinline__ void dft_odd(float2* x, const float* cs, const float* sn) {
  constexpr int H = (R - 1) / 2;
  float2 a[H], b[H];
  float2 y0 = x[0];
#pragma unroll
  for (int r = 1; r <= H; r++) {
    a[r - 1] = cadd(x[r], x[R - r]);
    b[r - 1] = csub(x[r], x[R - r]);
    y0 = cadd(y0, a[r - 1]);
  }
  float2 out[R];
  out[0] = y0;
#pragma unroll
  for (int k = 1; k <= H; k++) {
    float2 t1 = x[0], t2 = make_float2(0.f, 0.f);
#pragma unroll
    for (int r = 1; r <= H; r++) {
      int idx = (r * k) % R;  // cos(2pi rk/R) = cos(2pi idx/R)
      float c = idx <= H ? cs[idx] : cs[R - idx];
      float s = idx <= H ? sn[idx] : -sn[R - idx];
      t1.x = fmaf(a[r - 1].x, c, t1.x);
      t1.y = fmaf(a[r - 1].y, c, t1.y);
      t2.x = fmaf(b[r - 1].x, s, t2.x);
      t2.y = fmaf(b[r - 1].y, s, t2.y);
    }
    float2 it2 = mul_mi<INV>(t2);  // -i t2 (forward)
    out[k] = cadd(t1, it2);
    out[R - k] = csub(t1, it2);
  }
#pragma unroll
  for (int k = 0; k < R; k++) x[k] = out[k];
}

template <bool INV>
__device__ __forceinline__ void dft3(float2* x) {
  const float cs[2] = {1.f, -0.5f}, sn[2] = {0.f, 0.8660254037844387f};
  dft_odd<3, INV>(x, cs, sn);
}
template <bool INV>
__device__ __forceinline__ void dft5(float2* x) {
  const float cs[3] = {1.f, 0.30901699437494745f, -0.8090169943749473f};
  const float sn[3] = {0.f, 0.9510565162951535f, 0.5877852522924732f};
  dft_odd<5, INV>(x, cs, sn);
}
template <bool INV>
__device__ __forceinline__ void dft7(float2* x) {
  const float cs[4] = {1.f, 0.6234898018587336f, -0.22252093395631434f, -0.900968867902419f};
  const float sn[4] = {0.f, 0.7818314824680298f, 0.9749279121818236f, 0.43388373911755823f};
  dft_odd<7, INV>(x, cs, sn);
}

template <int R, bool INV>
__device__ __forceinline__ void dft_small(float2* x) {
  if constexpr (R == 2) dft2<INV>(x);
  else if constexpr (R == 3) dft3<INV>(x);
  else if constexpr (R == 4) dft4<INV>(x);
  else if constexpr (R == 5) dft5<INV>(x);
  else if constexpr (R == 7) dft7<INV>(x);
  else if constexpr (R == 8) dft8<INV>(x);
}

// Padded shared-memory index: one float2 of padding after every 16 keeps the
// stride-R (R = 2, 4, 8) butterfly accesses of the last passes free of bank
// conflicts.  A buffer of n complex values occupies padded_len(n) float2.
__device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 4) + 1; }

// Twiddle source: exp(-2 pi i e / T) = hi[e >> 6] * lo[e & 63], two small
// shared-memory tables filled from the FP64-derived global table (exact
// float entries; the product adds at most ~1 ulp).
struct SmemTw {
  const float2* hi;  // ceil(T/64) entries: exp(-2 pi i 64 h / T)
  const float2* lo;  // 64 entries: exp(-2 pi i l / T)
  __device__ __forceinline__ float2 operator()(int e) const { return cmul(hi[e >> 6], lo[e & 63]); }
};
__host__ __device__ constexpr int smem_tw_len(int T) { return (T + 63) / 64 + 64; }

// Fill hi/lo (contiguous, smem_tw_len(T) float2 at `dst`) from the global
// table gtw of length T. Caller syncs afterwards.
__device__ __forceinline__ SmemTw load_smem_tw(float2* dst, const float2* __restrict__ gtw, int T, int tid,
                                               int nthr) {
  const int nhi = (T + 63) / 64;
  for (int i = tid; i < nhi; i += nthr) dst[i] = __ldg(&gtw[(int64_t)i * 64]);
  for (int i = tid; i < 64; i += nthr) dst[nhi + i] = i < T ? __ldg(&gtw[i]) : make_float2(1.f, 0.f);
  return SmemTw{dst, dst + nhi};
}

// One DIF pass of radix R over buf (padded indexing): butterfly, then twiddle
// exp(-2 pi i j k / (R S)) = tw(j * k * tstep), tstep = T / (R S).
template <int R, class TW>
__device__ __forceinline__ void dif_pass(float2* buf, int n, int S, const TW& tw, int T, int tid, int nthr) {
  const int nbf = n / R;
  const int tstep = T / (R * S);
  for (int bf = tid; bf < nbf; bf += nthr) {
    int blk = bf / S, j = bf - blk * S;
    int base = blk * R * S + j;
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = buf[pidx(base + r * S)];
    dft_small<R, false>(x);
    if (j) {
#pragma unroll
      for (int k = 1; k < R; k++) x[k] = cmul(x[k], tw(j * k * tstep));
    }
#pragma unroll
    for (int k = 0; k < R; k++) buf[pidx(base + k * S)] = x[k];
  }
}

// One DIT (adjoint) pass: conjugate twiddle, then inverse butterfly.
template <int R, class TW>
__device__ __forceinline__ void dit_pass(float2* buf, int n, int S, const TW& tw, int T, int tid, int nthr) {
  const int nbf = n / R;
  const int tstep = T / (R * S);
  for (int bf = tid; bf < nbf; bf += nthr) {
    int blk = bf / S, j = bf - blk * S;
    int base = blk * R * S + j;
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = buf[pidx(base + r * S)];
    if (j) {
#pragma unroll
      for (int k = 1; k < R; k++) x[k] = cmulc(x[k], tw(j * k * tstep));
    }
    dft_small<R, true>(x);
#pragma unroll
    for (int k = 0; k < R; k++) buf[pidx(base + k * S)] = x[k];
  }
}

// One pass of any radix R as a direct DFT (the prime factors without a
// register butterfly).  Output k of butterfly (blk, j) is
//   DIF: W_RS^(j k) sum_r x_r W_R^(r k)      DIT: sum_r conj(W_RS^(j r)) x_r conj(W_R)^(r k)
// with every twiddle an exact table entry (index (r k) mod R advanced by
// integer steps, no recurrences); the R terms are summed in blocks of 32
// before being added, which keeps fp32 rounding near that of an FFT.  All
// threads share the outputs; they go to the CTA's global scratch and are
// copied back after a barrier.  The caller syncs after the pass.
template <bool INV, class TW>
__device__ __noinline__ void generic_pass(float2* buf, int n, int R, int S, const TW& tw, int T, float2* scratch,
                                          int tid, int nthr) {
  const int tstep = T / (R * S), rstep = T / R;
  for (int o = tid; o < n; o += nthr) {
    const int bf = o / R, k = o - bf * R;
    const int blk = bf / S, j = bf - blk * S;
    const int base = blk * R * S + j;
    float2 acc = make_float2(0.f, 0.f), part = make_float2(0.f, 0.f);
    int e = 0;  // (r k) mod R
    for (int r = 0; r < R; r++) {
      float2 x = buf[pidx(base + r * S)];
      if (INV && j) x = cmulc(x, tw(j * r * tstep));
      const float2 w = tw(e * rstep);
      part = INV ? cadd(part, cmulc(x, w)) : cadd(part, cmul(x, w));
      e += k;
      if (e >= R) e -= R;
      if ((r & 31) == 31) {
        acc = cadd(acc, part);
        part = make_float2(0.f, 0.f);
      }
    }
    acc = cadd(acc, part);
    if (!INV && j) acc = cmul(acc, tw(j * k * tstep));
    scratch[base + k * S] = acc;
  }
  __syncthreads();
  for (int i = tid; i < n; i += nthr) buf[pidx(i)] = scratch[i];
}

// Twiddle source reading a global table directly.
struct GlobalTw {
  const float2* t;
  __device__ __forceinline__ float2 operator()(int e) const { return __ldg(&t[e]); }
};

template <bool INV, class TW, bool GEN = true>
__device__ __forceinline__ void run_pass(int R, float2* buf, int n, int S, const TW& tw, int T, int tid, int nthr,
                                         float2* gscratch = nullptr, const BluesteinPass* bs = nullptr,
                                         float2* sscratch = nullptr);

// A pass of the prime radix bs.R by Bluestein's method, butterfly by
// butterfly with all threads, through the shared scratch sc (padded_len(L)).
// DIF: y_k = W_RS^(j k) DFT(x)_k; DIT: y = IDFT(x_r conj(W_RS^(j r))), the
// inverse as conj(DFT(conj(.))).  Every chirp and twiddle is an exact table
// entry (chirp index m^2 mod 2R in integers).
template <bool INV, class TW>
__device__ __noinline__ void bluestein_pass(float2* buf, int n, int S, const TW& tw, int T, const BluesteinPass& bs,
                                            float2* sc, int tid, int nthr) {
  const int R = bs.R, L = bs.L, tstep = T / (R * S);
  const GlobalTw twl{bs.twL};
  const int nbf = n / R;
  for (int bf = 0; bf < nbf; bf++) {
    const int blk = bf / S, j = bf - blk * S;
    const int base = blk * R * S + j;
    for (int r = tid; r < L; r += nthr) {
      float2 a = make_float2(0.f, 0.f);
      if (r < R) {
        float2 x = buf[pidx(base + r * S)];
        if (INV) {
          if (j) x = cmulc(x, tw(j * r * tstep));
          x = cconj(x);
        }
        a = cmul(x, __ldg(&bs.chirp[(int)(((int64_t)r * r) % (2 * R))]));
      }
      sc[pidx(r)] = a;
    }
    __syncthreads();
    for (int q = 0; q < bs.npass; q++) {  // L's passes use register butterflies only (L is 7-smooth)
      run_pass<false, GlobalTw, false>(bs.radix[q], sc, L, bs.span[q], twl, L, tid, nthr);
      __syncthreads();
    }
    for (int i = tid; i < L; i += nthr) sc[pidx(i)] = cmul(sc[pidx(i)], __ldg(&bs.filt[i]));
    __syncthreads();
    for (int q = bs.npass - 1; q >= 0; q--) {
      run_pass<true, GlobalTw, false>(bs.radix[q], sc, L, bs.span[q], twl, L, tid, nthr);
      __syncthreads();
    }
    for (int k = tid; k < R; k += nthr) {
      float2 y = cmul(sc[pidx(k)], __ldg(&bs.chirp[(int)(((int64_t)k * k) % (2 * R))]));
      if (INV) y = cconj(y);
      else if (j) y = cmul(y, tw(j * k * tstep));
      buf[pidx(base + k * S)] = y;
    }
    __syncthreads();
  }
}

template <bool INV, class TW, bool GEN>
__device__ __forceinline__ void run_pass(int R, float2* buf, int n, int S, const TW& tw, int T, int tid, int nthr,
                                         float2* gscratch, const BluesteinPass* bs, float2* sscratch) {
  switch (R) {
    case 2: INV ? dit_pass<2>(buf, n, S, tw, T, tid, nthr) : dif_pass<2>(buf, n, S, tw, T, tid, nthr); break;
    case 3: INV ? dit_pass<3>(buf, n, S, tw, T, tid, nthr) : dif_pass<3>(buf, n, S, tw, T, tid, nthr); break;
    case 4: INV ? dit_pass<4>(buf, n, S, tw, T, tid, nthr) : dif_pass<4>(buf, n, S, tw, T, tid, nthr); break;
    case 5: INV ? dit_pass<5>(buf, n, S, tw, T, tid, nthr) : dif_pass<5>(buf, n, S, tw, T, tid, nthr); break;
    case 7: INV ? dit_pass<7>(buf, n, S, tw, T, tid, nthr) : dif_pass<7>(buf, n, S, tw, T, tid, nthr); break;
    case 8: INV ? dit_pass<8>(buf, n, S, tw, T, tid, nthr) : dif_pass<8>(buf, n, S, tw, T, tid, nthr); break;
    default:
      if constexpr (GEN) {
        if (bs && sscratch && bs->R == R)
          bluestein_pass<INV>(buf, n, S, tw, T, *bs, sscratch, tid, nthr);
        else if (gscratch)
          generic_pass<INV>(buf, n, R, S, tw, T, gscratch + (size_t)(blockIdx.y * gridDim.x + blockIdx.x) * n, tid,
                            nthr);
      }
      break;
  }
}

// Forward transform of the padded buffer, natural -> digit-reversed.
// The caller syncs before; this syncs after every pass.
template <class TW>
__device__ __forceinline__ void dif_forward(float2* buf, const FftPlan& p, const TW& tw, int T, int tid, int nthr,
                                            float2* sscratch = nullptr) {
  for (int q = 0; q < p.npass; q++) {
    run_pass<false>(p.radix[q], buf, p.n, p.span[q], tw, T, tid, nthr, p.gscratch, &p.bs, sscratch);
    __syncthreads();
  }
}

// Inverse (unnormalised) transform, digit-reversed -> natural.
template <class TW>
__device__ __forceinline__ void dit_inverse(float2* buf, const FftPlan& p, const TW& tw, int T, int tid, int nthr,
                                            float2* sscratch = nullptr) {
  for (int q = p.npass - 1; q >= 0; q--) {
    run_pass<true>(p.radix[q], buf, p.n, p.span[q], tw, T, tid, nthr, p.gscratch, &p.bs, sscratch);
    __syncthreads();
  }
}

// Storage position (logical, before pidx) of frequency f after dif_forward.
__device__ __forceinline__ int fft_pos(const FftPlan& p, int f) {
  int pos = 0;
  for (int q = 0; q < p.npass; q++) {
    int R = p.radix[q];
    int d = f % R;
    f /= R;
    pos += d * p.span[q];
  }
  return pos;
}

// ---- register FFT of compile-time power-of-two length N <= 64 ------------
// Forward, natural order in and out; twiddles from a constant table of
// exp(-2 pi i e / 64), e in [0, 64).
template <int N>
__device__ __forceinline__ void reg_fft_pow2(float2 (&x)[N], const float2* __restrict__ tw64) {
  static_assert(N >= 1 && N <= 64 && (N & (N - 1)) == 0, "N must be a power of two <= 64");
  if constexpr (N == 1) return;
  else {
    // bit reversal
#pragma unroll
    for (int i = 0; i < N; i++) {
      int j = 0;
#pragma unroll
      for (int b = 1, t = i; b < N; b <<= 1, t >>= 1) j = (j << 1) | (t & 1);
      if (i < j) {
        float2 t = x[i];
        x[i] = x[j];
        x[j] = t;
      }
    }
#pragma unroll
    for (int len = 2; len <= N; len <<= 1) {
#pragma unroll
      for (int i = 0; i < N; i += len) {
#pragma unroll
        for (int k = 0; k < len / 2; k++) {
          float2 w = tw64[k * (64 / len)];
          float2 u = x[i + k], v = cmul(x[i + k + len / 2], w);
          x[i + k] = cadd(u, v);
          x[i + k + len / 2] = csub(u, v);
        }
      }
    }
  }
}

}  // namespace ab
