// ipfb.cu -- inverse PFB: FP64 window-matrix spectrum and Wiener filter,
// row-stage inverse FFT (fused with 4-bit decode and channel placement for
// the streaming chain), and the time-axis Wiener deconvolution.
//
// Reference: cupy_ipfb (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91):
//   dd   = irfft(dat, axis=1)                 (nslice, P), /P
//   ddft = rfft(dd.T, axis=1)                 (P, nslice/2+1)
//   res  = irfft(ddft * filt, axis=1).T       /nslice
// Here stage 1 computes dd in the [n][t] layout (column n = sample phase,
// contiguous in t); stage 2 in its FFT form (this file) does rfft -> *filt ->
// irfft on each column inside one CTA's shared memory.  The IIR and FIR forms
// of stage 2, the streaming chain's default, are in fir.cu.
#include <math.h>

#include <type_traits>

#include "fft_static.cuh"
#include <algorithm>

#include "fold.cuh"
#include "ipfb.cuh"

namespace ab {

// ---------------------------------------------------------------------------
// FP64 window-matrix spectrum (get_matft, pfb_gpu_utils.py:123-137):
// matft[k, f] = sum_{t<ntap} w[t*P + k] exp(-2 pi i f t / nslice).
__global__ void matft_kernel(const double* __restrict__ win, int P, int ntap, int64_t nslice, int64_t nf,
                             float2* __restrict__ out, const double thresh, int mode) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)P * nf) return;
  int64_t k = idx / nf, f = idx - k * nf;
  double re = 0.0, im = 0.0;
  for (int t = 0; t < ntap; t++) {
    int64_t e = (f * t) % nslice;
    double s, c;
    sincospi(2.0 * (double)e / (double)nslice, &s, &c);
    double w = win[(int64_t)t * P + k];
    re = fma(w, c, re);
    im = fma(-w, s, im);
  }
  if (mode == 0) {
    out[idx] = make_float2((float)re, (float)im);
    return;
  }
  // Wiener filter (calculate_filter, pfb_gpu_utils.py:29-36):
  // 1/conj(m) * |m|^2/(t^2+|m|^2) * (1+t^2) = m (1+t^2) / (t^2+|m|^2)
  double a2 = re * re + im * im;
  double g = thresh > 0 ? (1.0 + thresh * thresh) / (thresh * thresh + a2) : 1.0 / a2;
  out[idx] = make_float2((float)(re * g), (float)(im * g));
}

__global__ void filter_kernel(const float2* __restrict__ m, float2* __restrict__ out, int64_t n, double thresh) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double re = m[i].x, im = m[i].y;
  double a2 = re * re + im * im;
  // 1/conj(m) = m/|m|^2
  double g = 1.0 / a2;
  if (thresh > 0) g *= a2 / (thresh * thresh + a2) * (1.0 + thresh * thresh);
  out[i] = make_float2((float)(re * g), (float)(im * g));
}

// host: sinc-Hamming window (pfb_utils.py:4-7) in double
void sinc_hamming_host(int ntap, int64_t lblock, std::vector<double>& w) {
  int64_t N = (int64_t)ntap * lblock;
  w.resize((size_t)N);
  const double pi = 3.14159265358979323846;
  for (int64_t i = 0; i < N; i++) {
    double ham = N > 1 ? 0.54 - 0.46 * cos(2.0 * pi * (double)i / (double)(N - 1)) : 1.0;
    double x = ((double)i - (double)N / 2.0) / (double)lblock;
    double sc = x == 0.0 ? 1.0 : sin(pi * x) / (pi * x);
    w[(size_t)i] = ham * sc;
  }
}

// ---------------------------------------------------------------------------
// Stage 1: row inverse FFT.  Two real rows share one complex P-point inverse
// FFT: Z = A + iB with A, B Hermitian-extended, z = IDFT(Z), rows = Re z,
// Im z.  The nonzero bins are scattered straight into digit-reversed
// positions so the DIT passes produce natural order.
constexpr int kRowFftsPerCta = 4;
constexpr int kRowThreadsPerFft = 256;

// shared memory of a row-stage CTA: kRowFftsPerCta padded P-point buffers,
// then the twiddle tables of T = P
__host__ __device__ inline size_t row_smem_bytes(int P, int fpc = kRowFftsPerCta) {
  return sizeof(float2) * ((size_t)padded_len(P) * fpc + smem_tw_len(P));
}

__device__ __forceinline__ float dec4f(unsigned v) { return (float)((int)((v + 7u) & 15u) - 7); }

struct NoPlan {};

// FFT policy helpers: a compile-time plan (twiddle stream `tws`) or the
// generic runtime plan (two-level shared-memory table `tw`).
template <class PL, int NTHR>
__device__ __forceinline__ void fft_inv(float2* buf, const FftPlan& plan, const SmemTw& tw, int T,
                                        const float2* tws, int tid, float2* sscratch = nullptr) {
  if constexpr (std::is_same<PL, NoPlan>::value) dit_inverse(buf, plan, tw, T, tid, NTHR, sscratch);
  else sdit<PL, NTHR>(buf, tws, tid);
}
template <class PL, int NTHR>
__device__ __forceinline__ void fft_fwd(float2* buf, const FftPlan& plan, const SmemTw& tw, int T,
                                        const float2* tws, int tid, float2* sscratch = nullptr) {
  if constexpr (std::is_same<PL, NoPlan>::value) dif_forward(buf, plan, tw, T, tid, NTHR, sscratch);
  else sdif<PL, NTHR>(buf, tws, tid);
}
template <class PL>
__device__ __forceinline__ int fpos(const FftPlan& plan, int f) {
  if constexpr (std::is_same<PL, NoPlan>::value) return fft_pos(plan, f);
  else return spos<PL>(f);
}

// value of bin k of a real spectrum pair into Z (k in [0, P/2]); padded buffer
template <class PL>
__device__ __forceinline__ void put_pair_t(float2* buf, const FftPlan& p, int P, int k, float2 A, float2 B) {
  if (k == 0 || 2 * k == P) {
    buf[pidx(fpos<PL>(p, k))] = make_float2(A.x, B.x);  // imag parts of DC / Nyquist ignored (irfft)
  } else {
    buf[pidx(fpos<PL>(p, k))] = make_float2(A.x - B.y, A.y + B.x);      // A + iB
    buf[pidx(fpos<PL>(p, P - k))] = make_float2(A.x + B.y, B.x - A.y);  // conj(A) + i conj(B)
  }
}

// grid: (ceil(nrows / FPC), nant); one FFT per spectrum row, both pols, FPC
// spectra per CTA (4: one 1024-thread CTA per SM; 2: two or three CTAs per SM
// whose phases interleave, with 8-byte instead of 16-byte column stores).
template <class PL, int FPC>
__global__ void __launch_bounds__(FPC* kRowThreadsPerFft, FPC == 4 ? 1 : 2)
    row_stage_packed4_kernel(Packed4Src src, int nrows, FftPlan plan, const float2* __restrict__ tw,
                             const float2* __restrict__ tws, float* __restrict__ out, int64_t ld) {
  extern __shared__ float2 smem[];
  const int P = plan.n, PL_ = padded_len(P);
  const int a = blockIdx.y;
  const int sub = threadIdx.x / kRowThreadsPerFft, ltid = threadIdx.x % kRowThreadsPerFft;
  const int t = blockIdx.x * FPC + sub;
  float2* buf = smem + (size_t)sub * PL_;
  SmemTw tws_s{nullptr, nullptr};
  if constexpr (std::is_same<PL, NoPlan>::value)
    tws_s = load_smem_tw(smem + (size_t)FPC * PL_, tw, P, threadIdx.x, blockDim.x);
  {
    float4* b4 = reinterpret_cast<float4*>(smem);  // zero all buffers (PL_ * FFTS float2, even count)
    const int n4 = (FPC * PL_) / 2;
    for (int i = threadIdx.x; i < n4; i += blockDim.x) b4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  int64_t rawrow = -1;
  if (t < nrows) {
    int64_t g = src.g0 + t;
    if (g >= 0) rawrow = src.spec_map ? (int64_t)src.spec_map[(int64_t)a * src.map_stride + g] : g;
  }
  if (rawrow >= 0) {
    const uint8_t* row = src.raw + (int64_t)a * src.ant_stride + rawrow * src.row_bytes;
    for (int k = ltid; k < src.nsel; k += kRowThreadsPerFft) {
      const int c = __ldg(&src.chan_cols[k]);
      float2 A, B;
      if (src.bits == 4) {
        uchar2 b = *reinterpret_cast<const uchar2*>(row + 2 * c);
        A = make_float2(dec4f(b.x >> 4), dec4f(b.x & 15u));
        B = make_float2(dec4f(b.y >> 4), dec4f(b.y & 15u));
      } else {
        // 1-bit (unpacking.c:207-246): a set bit is +1, a clear bit -1
        const unsigned v = (row[c >> 1] >> ((c & 1) ? 0 : 4)) & 15u;  // r0 i0 r1 i1
        A = make_float2((float)(((v >> 3) & 1u) * 2) - 1.f, (float)(((v >> 2) & 1u) * 2) - 1.f);
        B = make_float2((float)(((v >> 1) & 1u) * 2) - 1.f, (float)((v & 1u) * 2) - 1.f);
      }
      put_pair_t<PL>(buf, plan, P, __ldg(&src.chan_abs[k]), A, B);
    }
  }
  __syncthreads();
  fft_inv<PL, kRowThreadsPerFft>(buf, plan, tws_s, P, tws, ltid);
  // write: column n of input (2a+p) at rows t0..t0+3 (one 16-byte store per
  // column and pol when the rows are 16-byte aligned)
  const float inv = 1.0f / (float)P;
  const int nthr = FPC * kRowThreadsPerFft;
  const int64_t t0 = (int64_t)blockIdx.x * FPC;
  if (FPC == 4 && ld % 4 == 0 && t0 + 4 <= nrows && ((uintptr_t)out & 15) == 0) {
    for (int n = threadIdx.x; n < P; n += nthr) {
      float2 z0 = smem[pidx(n)], z1 = smem[(size_t)PL_ + pidx(n)];
      float2 z2 = smem[(size_t)2 * PL_ + pidx(n)], z3 = smem[(size_t)3 * PL_ + pidx(n)];
      *reinterpret_cast<float4*>(out + ((int64_t)(2 * a) * P + n) * ld + t0) =
          make_float4(z0.x * inv, z1.x * inv, z2.x * inv, z3.x * inv);
      *reinterpret_cast<float4*>(out + ((int64_t)(2 * a + 1) * P + n) * ld + t0) =
          make_float4(z0.y * inv, z1.y * inv, z2.y * inv, z3.y * inv);
    }
  } else if (FPC == 2 && ld % 2 == 0 && t0 + 2 <= nrows && ((uintptr_t)out & 7) == 0) {
    for (int n = threadIdx.x; n < P; n += nthr) {
      float2 z0 = smem[pidx(n)], z1 = smem[(size_t)PL_ + pidx(n)];
      *reinterpret_cast<float2*>(out + ((int64_t)(2 * a) * P + n) * ld + t0) = make_float2(z0.x * inv, z1.x * inv);
      *reinterpret_cast<float2*>(out + ((int64_t)(2 * a + 1) * P + n) * ld + t0) =
          make_float2(z0.y * inv, z1.y * inv);
    }
  } else {
    for (int i = threadIdx.x; i < FPC * P; i += nthr) {
      int n = i / FPC, f = i - n * FPC;
      int64_t tt = t0 + f;
      if (tt >= nrows) continue;
      float2 z = smem[(size_t)f * PL_ + pidx(n)];
      out[((int64_t)(2 * a) * P + n) * ld + tt] = z.x * inv;
      out[((int64_t)(2 * a + 1) * P + n) * ld + tt] = z.y * inv;
    }
  }
}

// dense c64 rows (nslice, P/2+1): one FFT for rows (2j, 2j+1)
template <class PL>
__global__ void __launch_bounds__(kRowFftsPerCta* kRowThreadsPerFft)
    row_stage_c64_kernel(const float2* __restrict__ dat, int64_t nslice, FftPlan plan,
                         const float2* __restrict__ tw, const float2* __restrict__ tws, float* __restrict__ out,
                         int64_t ld) {
  extern __shared__ float2 smem[];
  const int P = plan.n, nb = P / 2 + 1, PL_ = padded_len(P);
  const int sub = threadIdx.x / kRowThreadsPerFft, ltid = threadIdx.x % kRowThreadsPerFft;
  const int64_t ta = 2 * ((int64_t)blockIdx.x * kRowFftsPerCta + sub);
  float2* buf = smem + (size_t)sub * PL_;
  SmemTw tws_s{nullptr, nullptr};
  if constexpr (std::is_same<PL, NoPlan>::value)
    tws_s = load_smem_tw(smem + (size_t)kRowFftsPerCta * PL_, tw, P, threadIdx.x, blockDim.x);
  for (int i = ltid; i < PL_; i += kRowThreadsPerFft) buf[i] = make_float2(0.f, 0.f);
  __syncthreads();
  if (ta < nslice) {
    const float2* ra = dat + ta * nb;
    const float2* rb = ta + 1 < nslice ? dat + (ta + 1) * nb : nullptr;
    for (int k = ltid; k < nb; k += kRowThreadsPerFft) {
      float2 A = ra[k];
      float2 B = rb ? rb[k] : make_float2(0.f, 0.f);
      put_pair_t<PL>(buf, plan, P, k, A, B);
    }
  }
  __syncthreads();
  fft_inv<PL, kRowThreadsPerFft>(buf, plan, tws_s, P, tws, ltid);
  const float inv = 1.0f / (float)P;
  const int nthr = kRowFftsPerCta * kRowThreadsPerFft;
  const int64_t tbase = 2 * (int64_t)blockIdx.x * kRowFftsPerCta;
  for (int i = threadIdx.x; i < kRowFftsPerCta * 2 * P; i += nthr) {
    int n = i / (2 * kRowFftsPerCta), r = i - n * (2 * kRowFftsPerCta);
    int f = r >> 1, part = r & 1;
    int64_t tt = tbase + r;
    if (tt >= nslice) continue;
    float2 z = smem[(size_t)f * PL_ + pidx(n)];
    out[(int64_t)n * ld + tt] = (part ? z.y : z.x) * inv;
  }
}

// ---------------------------------------------------------------------------
// Stage 2: per column n, real FFT of length N via a complex FFT of M = N/2,
// multiply by the filter, inverse.  All in shared memory, one CTA per column.
constexpr int kTimeThreads = 1024;

__host__ __device__ inline size_t time_smem_bytes(int N) {
  return sizeof(float2) * ((size_t)padded_len(N / 2) + smem_tw_len(N));
}

// NTAP: number of window taps of the on-the-fly filter and of the fused PFB
// fold (compile time); 0 = runtime `ntap` (filter only, no fold).
template <class PL, bool TABLE, int NTHR, int FOLDG = 0, int NTAP = 0>
__global__ void __launch_bounds__(NTHR)
    time_stage_kernel(float* __restrict__ data, int64_t ld, int P, int N, FftPlan plan,
                      const float2* __restrict__ twN, const float2* __restrict__ tws,
                      const float2* __restrict__ table, const float* __restrict__ wtaps, int ntap, float thresh,
                      FoldArgs fa, const float2* __restrict__ tw64, const int2* __restrict__ pairs) {
  extern __shared__ float2 buf[];
  const int n = blockIdx.x, input = blockIdx.y;
  const int M = N / 2;
  const int tid = threadIdx.x;
  float* col = data + ((int64_t)input * P + n) * ld;
  const float2* col2 = reinterpret_cast<const float2*>(col);
  const SmemTw tw = load_smem_tw(buf + padded_len(M), twN, N, tid, NTHR);
  for (int m = tid; m < M; m += NTHR) buf[pidx(m)] = col2[m];
  // window taps of this column for the on-the-fly filter
  float w[8];
  if (!TABLE) {
#pragma unroll
    for (int t = 0; t < 8; t++) w[t] = t < ntap ? __ldg(&wtaps[(int64_t)t * P + n]) : 0.f;
  }
  // a Bluestein pass's scratch follows the twiddle tables (plans of ab_ipfb only)
  float2* bscr = plan.bs.R ? buf + padded_len(M) + smem_tw_len(N) : nullptr;
  __syncthreads();
  fft_fwd<PL, NTHR>(buf, plan, tw, N, tws, tid, bscr);

  const float scale = 0.5f / (float)N;  // irfft 1/N and the untangle's 1/2
  const float t2 = thresh * thresh;
  // filter at bin k from z = exp(-2 pi i k / N): m = sum_t w_t z^t (Horner),
  // H = m (1 + t^2) / (t^2 + |m|^2), or 1/conj(m) without threshold
  auto filt_z = [&](int k, float2 z) -> float2 {
    float2 h;
    if (TABLE) {
      h = __ldg(&table[(int64_t)n * (M + 1) + k]);
    } else {
      float2 m = make_float2(0.f, 0.f);
      if constexpr (NTAP > 0) {
        m.x = w[NTAP - 1];
#pragma unroll
        for (int t = NTAP - 2; t >= 0; t--) {
          m = cmul(m, z);
          m.x += w[t];
        }
      } else {
#pragma unroll
        for (int t = 7; t >= 0; t--) {
          if (t < ntap) {
            m = cmul(m, z);
            m.x += w[t];
          }
        }
      }
      float a2 = fmaf(m.x, m.x, m.y * m.y);
      float g = thresh > 0.f ? __fdividef(1.f + t2, t2 + a2) : __fdividef(1.f, a2);
      h = make_float2(m.x * g, m.y * g);
    }
    return cscale(h, scale);
  };

  for (int k = tid; k <= M / 2; k += NTHR) {
    if (k == 0) {
      float2 z = buf[0];
      float x0 = 2.f * (z.x + z.y), xm = 2.f * (z.x - z.y);  // 2 X[0], 2 X[M] (real)
      // z^0 = 1 and z^M = -1 (exp(-i pi))
      float y0 = x0 * filt_z(0, make_float2(1.f, 0.f)).x, ym = xm * filt_z(M, make_float2(-1.f, 0.f)).x;
      buf[0] = make_float2(y0 + ym, y0 - ym);  // real parts only (irfft)
      continue;
    }
    const int2 pp = __ldg(&pairs[k]);
    const int pk = pp.x, pc = pp.y;
    float2 zk = buf[pk], zc = buf[pc];
    float2 w1 = tw(k);                           // exp(-2 pi i k / N)
    const float2 w1c = make_float2(-w1.x, w1.y);  // exp(-2 pi i (M-k) / N) = -conj(w1)
    float2 E = cadd(zk, cconj(zc));              // 2 E_k
    float2 Od = csub(zk, cconj(zc));             // 2 i O_k
    float2 O = make_float2(Od.y, -Od.x);         // 2 O_k = (2 i O_k) / i
    float2 wO = cmul(w1, O);
    float2 Xk = cadd(E, wO);                     // 2 X_k
    float2 Xc = cconj(csub(E, wO));              // 2 X_{M-k}
    float2 Yk = cmul(Xk, filt_z(k, w1));
    float2 Yc = cmul(Xc, filt_z(M - k, w1c));
    float2 Et = cadd(Yk, cconj(Yc));
    float2 Ot = cmulc(csub(Yk, cconj(Yc)), w1);  // (Y_k - conj Y_{M-k}) conj(w)
    float2 iOt = make_float2(-Ot.y, Ot.x);
    buf[pk] = cadd(Et, iOt);
    if (pc != pk) buf[pc] = cadd(cconj(Et), make_float2(Ot.y, Ot.x));  // conj(Et) + i conj(Ot)
  }
  __syncthreads();
  fft_inv<PL, NTHR>(buf, plan, tw, N, tws, tid, bscr);
  if constexpr (FOLDG == 0) {
    float2* out2 = reinterpret_cast<float2*>(col);
    for (int m = tid; m < M; m += NTHR) out2[m] = buf[pidx(m)];
  } else {
    // fused PFB fold: previous tail rows -> shared memory, fold all blocks,
    // then store this chunk's last 4*O rows as the next chunk's tail
    constexpr int O = 2 * FOLDG;
    float* stail = reinterpret_cast<float*>(buf + padded_len(M) + smem_tw_len(N));
    float* st = fa.state + ((int64_t)input * P + n) * (4 * O);
    for (int i = tid; i < 4 * O; i += NTHR) stail[i] = st[i];
    __syncthreads();
    fold_blocks<FOLDG, NTAP, false>(buf, stail, fa, P, n, input, tw64, 0, (int)fa.nb);
    __syncthreads();
    const float* fbuf = reinterpret_cast<const float*>(buf);
    for (int i = tid; i < 4 * O; i += NTHR) {
      int64_t r = (int64_t)fa.acclen - 4 * O + i;
      float v = 0.f;
      if (r >= 0) {
        int t = (int)(fa.cut + r);
        v = fbuf[2 * pidx(t >> 1) + (t & 1)];
      } else {
        v = stail[r + 4 * O];  // acclen < 4*O: keep older rows
      }
      st[i] = v;
    }
  }
}

template <class K>
static int set_smem_attr(K kernel, size_t bytes) {
  AB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return AB_OK;
}

// Time-paired form: a CTA takes 8 consecutive spectra of ONE input (antenna
// a, pol p = blockIdx.y % 2) and transforms spectra (t, t+1) together as
// Z = A_t + i A_{t+1}.  Each column then receives 8 consecutive rows (32 bytes,
// one full sector) in one 32-byte store (two 16-byte stores by a lane pair
// when the column is only 16-byte aligned).  (Pairing the two pols of one spectrum instead
// leaves 16 bytes per column and input, half a sector per lane.)
template <class PL>
__global__ void __launch_bounds__(4 * kRowThreadsPerFft)
    row_stage_tpair_kernel(Packed4Src src, int nrows, FftPlan plan, const float2* __restrict__ tw,
                           const float2* __restrict__ tws, float* __restrict__ out, int64_t ld) {
  constexpr int FFTS = 4, ROWS = 2 * FFTS;
  extern __shared__ float2 smem[];
  const int P = plan.n, PL_ = padded_len(P);
  const int in = blockIdx.y, a = in >> 1, pol = in & 1;
  const int sub = threadIdx.x / kRowThreadsPerFft, ltid = threadIdx.x % kRowThreadsPerFft;
  const int64_t t0 = (int64_t)blockIdx.x * ROWS;
  float2* buf = smem + (size_t)sub * PL_;
  SmemTw tws_s{nullptr, nullptr};
  if constexpr (std::is_same<PL, NoPlan>::value)
    tws_s = load_smem_tw(smem + (size_t)FFTS * PL_, tw, P, threadIdx.x, blockDim.x);
  {
    float4* b4 = reinterpret_cast<float4*>(smem);  // zero all buffers (PL_ * FFTS float2, even count)
    const int n4 = (FFTS * PL_) / 2;
    for (int i = threadIdx.x; i < n4; i += blockDim.x) b4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  // raw rows of the two spectra of this FFT
  int64_t rawrow[2] = {-1, -1};
#pragma unroll
  for (int e = 0; e < 2; e++) {
    const int64_t t = t0 + 2 * sub + e;
    if (t < nrows) {
      const int64_t g = src.g0 + t;
      if (g >= 0) rawrow[e] = src.spec_map ? (int64_t)src.spec_map[(int64_t)a * src.map_stride + g] : g;
    }
  }
  if (rawrow[0] >= 0 || rawrow[1] >= 0) {
    const uint8_t* base = src.raw + (int64_t)a * src.ant_stride;
    for (int k = ltid; k < src.nsel; k += kRowThreadsPerFft) {
      const int c = __ldg(&src.chan_cols[k]);
      float2 v[2];
#pragma unroll
      for (int e = 0; e < 2; e++) {
        v[e] = make_float2(0.f, 0.f);
        if (rawrow[e] < 0) continue;
        const uint8_t* row = base + rawrow[e] * src.row_bytes;
        if (src.bits == 4) {
          const unsigned b = row[2 * c + pol];
          v[e] = make_float2(dec4f(b >> 4), dec4f(b & 15u));
        } else {
          // 1-bit (unpacking.c:207-246): r0 i0 r1 i1 per channel, set bit = +1
          const unsigned q = (row[c >> 1] >> ((c & 1) ? 0 : 4)) & 15u;
          const unsigned sh = pol ? 0u : 2u;
          v[e] = make_float2((float)(((q >> (sh + 1)) & 1u) * 2) - 1.f, (float)(((q >> sh) & 1u) * 2) - 1.f);
        }
      }
      put_pair_t<PL>(buf, plan, P, __ldg(&src.chan_abs[k]), v[0], v[1]);
    }
  }
  __syncthreads();
  fft_inv<PL, kRowThreadsPerFft>(buf, plan, tws_s, P, tws, ltid);
  // write: column n of this input gets rows t0 .. t0+7, one 32-byte store
  // (a whole sector) per column
  const float inv = 1.0f / (float)P;
  const int nthr = FFTS * kRowThreadsPerFft;
  float* ocol = out + (int64_t)in * P * ld + t0;
  if (ld % 8 == 0 && t0 + ROWS <= nrows && ((uintptr_t)out & 31) == 0) {
    for (int n = threadIdx.x; n < P; n += nthr) {
      const float2 z0 = smem[pidx(n)], z1 = smem[(size_t)PL_ + pidx(n)];
      const float2 z2 = smem[(size_t)2 * PL_ + pidx(n)], z3 = smem[(size_t)3 * PL_ + pidx(n)];
      st_global_v8(ocol + (int64_t)n * ld, z0.x * inv, z0.y * inv, z1.x * inv, z1.y * inv, z2.x * inv, z2.y * inv,
                   z3.x * inv, z3.y * inv);
    }
  } else if (ld % 4 == 0 && t0 + ROWS <= nrows && ((uintptr_t)out & 15) == 0) {
    // lane pair (2j, 2j+1) writes the two 16-byte halves of one column's 32 bytes
    for (int i = threadIdx.x; i < 2 * P; i += nthr) {
      const int n = i >> 1, h = i & 1;
      const float2 za = smem[(size_t)(2 * h) * PL_ + pidx(n)], zb = smem[(size_t)(2 * h + 1) * PL_ + pidx(n)];
      *reinterpret_cast<float4*>(ocol + (int64_t)n * ld + 4 * h) =
          make_float4(za.x * inv, za.y * inv, zb.x * inv, zb.y * inv);
    }
  } else {
    for (int i = threadIdx.x; i < ROWS * P; i += nthr) {
      const int n = i / ROWS, r = i - n * ROWS;
      if (t0 + r >= nrows) continue;
      const float2 z = smem[(size_t)(r >> 1) * PL_ + pidx(n)];
      ocol[(int64_t)n * ld + r] = ((r & 1) ? z.y : z.x) * inv;
    }
  }
}

// Persistent form of the time-paired row stage.  CTAs walk the tiles (8
// spectra of one input; tile = row block * inputs + input, so both pols of a
// spectrum follow each other) with a stride of gridDim.x.  A tile's global
// loads form a chain -- spectrum-map rows, then the packet words holding the
// selected bytes -- so they are issued with cp.async two tiles (map rows) and
// one tile (words) ahead into double-buffered shared slots and never stall
// the transform.  Needs nsel <= kRowThreadsPerFft (one selected channel per
// thread) and 4-byte-multiple packet rows and antenna strides (a word never
// leaves the packet buffer, and a byte's place in its word does not depend
// on the row).
constexpr int kRowPfRows = 8;
__host__ __device__ inline size_t row_pf_smem_bytes(int P, int tw_len = 0) {
  return row_smem_bytes(P, 4) + sizeof(int32_t) * 4 * kRowPfRows + sizeof(uint32_t) * 2 * kRowPfRows * kRowThreadsPerFft +
         sizeof(float2) * (size_t)tw_len;
}

// TWS (compile-time plans only): the plan's twiddle stream is copied into
// shared memory once per CTA and the FFT passes read it there.
template <class PL, bool TWS = false>
__global__ void __launch_bounds__(4 * kRowThreadsPerFft)
    row_stage_tpair_pf_kernel(Packed4Src src, int nrows, int nin, FftPlan plan, const float2* __restrict__ tw,
                              const float2* __restrict__ tws, float* __restrict__ out, int64_t ld) {
  constexpr int FFTS = 4, ROWS = kRowPfRows, T = kRowThreadsPerFft;
  static_assert(ROWS == 2 * FFTS, "two spectra per transform");
  extern __shared__ float2 smem[];
  const int P = plan.n, PL_ = padded_len(P);
  const int sub = threadIdx.x / T, ltid = threadIdx.x % T;
  float2* buf = smem + (size_t)sub * PL_;
  int32_t* st_map = reinterpret_cast<int32_t*>(smem + (size_t)FFTS * PL_ + smem_tw_len(P));  // [2][ROWS] raw rows
  int32_t* st_pres = st_map + 2 * ROWS;                                                         // [2][ROWS] present
  uint32_t* st_w = reinterpret_cast<uint32_t*>(st_pres + 2 * ROWS);                              // [2][ROWS][T] words
  SmemTw tws_s{nullptr, nullptr};
  if constexpr (std::is_same<PL, NoPlan>::value)
    tws_s = load_smem_tw(smem + (size_t)FFTS * PL_, tw, P, threadIdx.x, blockDim.x);
  const float2* twf = tws;  // FFT twiddle stream (global, or its copy in shared memory)
  if constexpr (TWS) {
    static_assert(!std::is_same<PL, NoPlan>::value, "shared twiddles need a compile-time plan");
    float2* tsh = reinterpret_cast<float2*>(st_w + 2 * ROWS * T);
    for (int q = threadIdx.x; q < PL::tw_len(); q += blockDim.x) tsh[q] = __ldg(&tws[q]);
    twf = tsh;  // visible after the first barrier of the loop
  }
  const int nrb = (nrows + ROWS - 1) / ROWS;
  const int ntiles = nrb * nin, G = gridDim.x;
  const bool has_k = ltid < src.nsel;
  const int col = has_k ? __ldg(&src.chan_cols[ltid]) : 0;
  const int kabs = has_k ? __ldg(&src.chan_abs[ltid]) : 0;
  // map rows of tile x into slot sl (threads 0..ROWS-1)
  auto issue_map = [&](int x, int sl) {
    if (x >= ntiles || threadIdx.x >= ROWS) return;
    const int rb = x / nin, a = (x % nin) >> 1;
    const int64_t t = (int64_t)rb * ROWS + threadIdx.x, g = src.g0 + t;
    int32_t* dst = st_map + sl * ROWS + threadIdx.x;
    if (t >= nrows || g < 0) *dst = -1;
    else if (src.spec_map) cp_async4(dst, src.spec_map + (int64_t)a * src.map_stride + g);
    else *dst = (int32_t)g;
  };
  // packet words of tile x (rows from map slot sl) into word slot sl
  auto issue_words = [&](int x, int sl) {
    if (x >= ntiles) return;
    const int in = x % nin, a = in >> 1, pol = in & 1;
    const int boff = src.bits == 4 ? 2 * col + pol : col >> 1;
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int r = 2 * sub + e;
      const int32_t row = st_map[sl * ROWS + r];
      if (ltid == 0) st_pres[sl * ROWS + r] = row >= 0;
      if (has_k && row >= 0) {
        const uint8_t* p = src.raw + (int64_t)a * src.ant_stride + (int64_t)row * src.row_bytes + (boff & ~3);
        cp_async4(st_w + ((size_t)sl * ROWS + r) * T + ltid, reinterpret_cast<const uint32_t*>(p));
      }
    }
  };
  int x = blockIdx.x;
  issue_map(x, 0);
  issue_map(x + G, 1);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  issue_words(x, 0);
  cp_async_commit();
  for (int i = 0; x < ntiles; x += G, i++) {
    const int sl = i & 1;
    cp_async_wait<0>();
    __syncthreads();  // words and presence of this tile, map rows of the next; buffers free
    issue_words(x + G, sl ^ 1);
    issue_map(x + 2 * G, sl);
    cp_async_commit();
    {
      float4* b4 = reinterpret_cast<float4*>(smem);  // zero all buffers (PL_ * FFTS float2, even count)
      const int n4 = (FFTS * PL_) / 2;
      for (int q = threadIdx.x; q < n4; q += blockDim.x) b4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int in = x % nin, pol = in & 1;
    const int r0 = 2 * sub;
    const bool p0 = st_pres[sl * ROWS + r0] != 0, p1 = st_pres[sl * ROWS + r0 + 1] != 0;
    if (has_k && (p0 || p1)) {
      const int boff = src.bits == 4 ? 2 * col + pol : col >> 1;
      const int sh = 8 * (boff & 3);
      float2 v[2];
#pragma unroll
      for (int e = 0; e < 2; e++) {
        v[e] = make_float2(0.f, 0.f);
        if (!(e ? p1 : p0)) continue;
        const unsigned b = (st_w[((size_t)sl * ROWS + r0 + e) * T + ltid] >> sh) & 0xffu;
        if (src.bits == 4) {
          v[e] = make_float2(dec4f(b >> 4), dec4f(b & 15u));
        } else {
          const unsigned q = (b >> ((col & 1) ? 0 : 4)) & 15u;
          const unsigned s2 = pol ? 0u : 2u;
          v[e] = make_float2((float)(((q >> (s2 + 1)) & 1u) * 2) - 1.f, (float)(((q >> s2) & 1u) * 2) - 1.f);
        }
      }
      put_pair_t<PL>(buf, plan, P, kabs, v[0], v[1]);
    }
    __syncthreads();
    if constexpr (TWS) sdit<PL, kRowThreadsPerFft, true>(buf, twf, ltid);
    else fft_inv<PL, kRowThreadsPerFft>(buf, plan, tws_s, P, tws, ltid);
    const float inv = 1.0f / (float)P;
    const int64_t t0 = (int64_t)(x / nin) * ROWS;
    float* ocol = out + (int64_t)in * P * ld + t0;
    if (t0 + ROWS <= nrows) {
      for (int n = threadIdx.x; n < P; n += blockDim.x) {
        const float2 z0 = smem[pidx(n)], z1 = smem[(size_t)PL_ + pidx(n)];
        const float2 z2 = smem[(size_t)2 * PL_ + pidx(n)], z3 = smem[(size_t)3 * PL_ + pidx(n)];
        st_global_v8(ocol + (int64_t)n * ld, z0.x * inv, z0.y * inv, z1.x * inv, z1.y * inv, z2.x * inv, z2.y * inv,
                     z3.x * inv, z3.y * inv);
      }
    } else {
      for (int q = threadIdx.x; q < ROWS * P; q += blockDim.x) {
        const int n = q / ROWS, r = q - n * ROWS;
        if (t0 + r >= nrows) continue;
        const float2 z = smem[(size_t)(r >> 1) * PL_ + pidx(n)];
        ocol[(int64_t)n * ld + r] = ((r & 1) ? z.y : z.x) * inv;
      }
    }
  }
  cp_async_wait<0>();  // nothing left in flight at exit
}

template <class PL, bool TWS = false>
static int launch_row_tpair_pf_t(ab_ctx* ctx, const Packed4Src& src, int nant, int nrows, int P, const FftPlan& plan,
                                 const float2* twP, const float2* tws, float* out, int64_t ld, cudaStream_t s) {
  size_t smem = row_pf_smem_bytes(P);
  if constexpr (TWS) smem = row_pf_smem_bytes(P, PL::tw_len());
  AB_CHECK_ARG(smem <= ctx->smem_optin, "row stage: %zu bytes of shared memory needed", smem);
  AB_TRY(set_smem_attr(row_stage_tpair_pf_kernel<PL, TWS>, smem));
  const int64_t ntiles = (int64_t)((nrows + kRowPfRows - 1) / kRowPfRows) * 2 * nant;
  AB_CHECK_ARG(ntiles < (1LL << 31), "row stage: too many tiles");
  const int grid = (int)std::min<int64_t>(ntiles, std::max(ctx->num_sms, 1));
  row_stage_tpair_pf_kernel<PL, TWS><<<grid, 4 * kRowThreadsPerFft, smem, s>>>(src, nrows, 2 * nant, plan, twP, tws, out,
                                                                              ld);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

template <class PL>
static int launch_row_tpair_t(ab_ctx* /*ctx*/, const Packed4Src& src, int nant, int nrows, int P, const FftPlan& plan,
                              const float2* twP, const float2* tws, float* out, int64_t ld, cudaStream_t s) {
  const size_t smem = row_smem_bytes(P, 4);
  AB_TRY(set_smem_attr(row_stage_tpair_kernel<PL>, smem));
  dim3 grid((unsigned)((nrows + 7) / 8), (unsigned)(2 * nant));
  row_stage_tpair_kernel<PL><<<grid, 4 * kRowThreadsPerFft, smem, s>>>(src, nrows, plan, twP, tws, out, ld);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

template <int FPC>
static int launch_row_packed4_t(ab_ctx* ctx, const Packed4Src& src, int nant, int nrows, int P, const FftPlan& plan,
                                const float2* twP, float* out, int64_t ld, cudaStream_t s) {
  size_t smem = row_smem_bytes(P, FPC);
  AB_CHECK_ARG(smem <= ctx->smem_optin, "row stage: lblock %d too large", P);
  dim3 grid((unsigned)((nrows + FPC - 1) / FPC), (unsigned)nant);
  bool tuned = false;
  { FftPlan tmp; ctx_plan(ctx, P, &tmp, &tuned); }
  if (P == Plan4096::N && !tuned) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    AB_TRY(set_smem_attr(row_stage_packed4_kernel<Plan4096, FPC>, smem));
    row_stage_packed4_kernel<Plan4096, FPC><<<grid, FPC * kRowThreadsPerFft, smem, s>>>(src, nrows, plan, twP, tws,
                                                                                         out, ld);
  } else {
    AB_TRY(set_smem_attr(row_stage_packed4_kernel<NoPlan, FPC>, smem));
    row_stage_packed4_kernel<NoPlan, FPC><<<grid, FPC * kRowThreadsPerFft, smem, s>>>(src, nrows, plan, twP, nullptr,
                                                                                       out, ld);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

int launch_row_stage_packed4(ab_ctx* ctx, const Packed4Src& src, int nant, int nrows, int P, const FftPlan& plan,
                             const float2* twP, float* out, int64_t ld, cudaStream_t s) {
  if (ctx->row_ffts_per_cta == 2) return launch_row_packed4_t<2>(ctx, src, nant, nrows, P, plan, twP, out, ld, s);
  if (ctx->row_ffts_per_cta == 4) return launch_row_packed4_t<4>(ctx, src, nant, nrows, P, plan, twP, out, ld, s);
  // default: time-paired spectra; the persistent prefetching form when its
  // conditions hold (ld % 8 for the 32-byte column stores, as the other)
  AB_CHECK_ARG(row_smem_bytes(P, 4) <= ctx->smem_optin, "row stage: lblock %d too large", P);
  bool tuned = false;
  { FftPlan tmp; ctx_plan(ctx, P, &tmp, &tuned); }
  const bool pf = ctx->row_prefetch && src.nsel <= kRowThreadsPerFft && src.row_bytes % 4 == 0 &&
                  src.ant_stride % 4 == 0 && ((uintptr_t)src.raw & 3) == 0 && ld % 8 == 0 &&
                  ((uintptr_t)out & 31) == 0 && row_pf_smem_bytes(P) <= ctx->smem_optin;
  if (P == Plan4096::N && !tuned) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    if (pf && ctx->row_prefetch == 2)
      return launch_row_tpair_pf_t<Plan4096, true>(ctx, src, nant, nrows, P, plan, twP, tws, out, ld, s);
    if (pf) return launch_row_tpair_pf_t<Plan4096>(ctx, src, nant, nrows, P, plan, twP, tws, out, ld, s);
    return launch_row_tpair_t<Plan4096>(ctx, src, nant, nrows, P, plan, twP, tws, out, ld, s);
  }
  if (pf) return launch_row_tpair_pf_t<NoPlan>(ctx, src, nant, nrows, P, plan, twP, nullptr, out, ld, s);
  return launch_row_tpair_t<NoPlan>(ctx, src, nant, nrows, P, plan, twP, nullptr, out, ld, s);
}

int launch_row_stage_c64(ab_ctx* ctx, const float2* dat, int64_t nslice, int P, const FftPlan& plan,
                         const float2* twP, float* out, int64_t ld, cudaStream_t s) {
  size_t smem = row_smem_bytes(P);
  AB_CHECK_ARG(smem <= ctx->smem_optin, "row stage: lblock %d too large", P);
  int64_t nfft = (nslice + 1) / 2;
  dim3 grid((unsigned)((nfft + kRowFftsPerCta - 1) / kRowFftsPerCta));
  bool tuned = false;
  { FftPlan tmp; ctx_plan(ctx, P, &tmp, &tuned); }
  if (P == Plan4096::N && !tuned) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    AB_TRY(set_smem_attr(row_stage_c64_kernel<Plan4096>, smem));
    row_stage_c64_kernel<Plan4096><<<grid, kRowFftsPerCta * kRowThreadsPerFft, smem, s>>>(dat, nslice, plan, twP,
                                                                                           tws, out, ld);
  } else {
    AB_TRY(set_smem_attr(row_stage_c64_kernel<NoPlan>, smem));
    row_stage_c64_kernel<NoPlan><<<grid, kRowFftsPerCta * kRowThreadsPerFft, smem, s>>>(dat, nslice, plan, twP,
                                                                                         nullptr, out, ld);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

template <class PL, int NTHR>
static int launch_time_t(ab_ctx* /*ctx*/, float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM,
                         const float2* twN, const float2* tws, const int2* pairs, const float2* table,
                         const float* wtaps, int ntap, float thresh, size_t smem, cudaStream_t s) {
  dim3 grid((unsigned)P, (unsigned)ninputs);
  if (table) {
    AB_TRY(set_smem_attr(time_stage_kernel<PL, true, NTHR>, smem));
    time_stage_kernel<PL, true, NTHR><<<grid, NTHR, smem, s>>>(buf, ld, P, N, planM, twN, tws, table, wtaps, ntap,
                                                              thresh, FoldArgs{}, nullptr, pairs);
  } else {
    AB_TRY(set_smem_attr(time_stage_kernel<PL, false, NTHR>, smem));
    time_stage_kernel<PL, false, NTHR><<<grid, NTHR, smem, s>>>(buf, ld, P, N, planM, twN, tws, table, wtaps, ntap,
                                                               thresh, FoldArgs{}, nullptr, pairs);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

int launch_time_stage(ab_ctx* ctx, float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM,
                      const float2* twN, const float2* table, const float* wtaps, int ntap, float thresh,
                      cudaStream_t s) {
  size_t smem = time_smem_bytes(N) + (planM.bs.R ? sizeof(float2) * (size_t)padded_len(planM.bs.L) : 0);
  AB_CHECK_ARG(smem <= ctx->smem_optin, "time stage: nslice %d needs %zu bytes of shared memory (max %zu)", N, smem,
               ctx->smem_optin);
  AB_CHECK_ARG(table || (wtaps && ntap >= 1 && ntap <= 8), "time stage: need a filter table or 1..8 window taps");
  const int M = N / 2;
  const float2* tws = nullptr;
  const int2* pairs = nullptr;
  FftPlan sp;
  bool tuned = false;
  { FftPlan tmp; ctx_plan(ctx, M, &tmp, &tuned); }
  if (M == Plan16464::N && !tuned) {
    AB_TRY(get_twiddle_stream(ctx, M, {7, 7, 7, 3, 16}, &tws));
    make_plan_from(M, {7, 7, 7, 3, 16}, &sp);
    AB_TRY(get_pair_table(ctx, sp, &pairs));
    return launch_time_t<Plan16464, 1024>(ctx, buf, ld, ninputs, P, N, planM, twN, tws, pairs, table, wtaps, ntap,
                                         thresh, smem, s);
  }
  if (M == Plan16384::N && !tuned) {
    AB_TRY(get_twiddle_stream(ctx, M, {4, 16, 16, 16}, &tws));
    make_plan_from(M, {4, 16, 16, 16}, &sp);
    AB_TRY(get_pair_table(ctx, sp, &pairs));
    return launch_time_t<Plan16384, 1024>(ctx, buf, ld, ninputs, P, N, planM, twN, tws, pairs, table, wtaps, ntap,
                                         thresh, smem, s);
  }
  AB_TRY(get_pair_table(ctx, planM, &pairs));
  return launch_time_t<NoPlan, kTimeThreads>(ctx, buf, ld, ninputs, P, N, planM, twN, nullptr, pairs, table, wtaps,
                                             ntap, thresh, smem, s);
}

template <class PL, int NTHR, int G>
static int launch_fold_t(float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM, const float2* twN,
                         const float2* tws, const int2* pairs, const float* wtaps, int ntap, float thresh,
                         const FoldArgs& fa, const float2* tw64, size_t smem, cudaStream_t s) {
  dim3 grid((unsigned)P, (unsigned)ninputs);
  AB_TRY(set_smem_attr(time_stage_kernel<PL, false, NTHR, G, 4>, smem));
  time_stage_kernel<PL, false, NTHR, G, 4><<<grid, NTHR, smem, s>>>(buf, ld, P, N, planM, twN, tws, nullptr, wtaps,
                                                                    ntap, thresh, fa, tw64, pairs);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

template <class PL, int NTHR>
static int launch_fold_o(float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM, const float2* twN,
                         const float2* tws, const int2* pairs, const float* wtaps, int ntap, float thresh,
                         const FoldArgs& fa, const float2* tw64, size_t smem, cudaStream_t s) {
#define AB_FOLD_CASE(OO, GG) \
  case OO:                 \
    return launch_fold_t<PL, NTHR, GG>(buf, ld, ninputs, P, N, planM, twN, tws, pairs, wtaps, ntap, thresh, fa, tw64, smem, s);
  switch (fa.O) {
    AB_FOLD_CASE(4, 2)
    AB_FOLD_CASE(8, 4)
    AB_FOLD_CASE(16, 8)
    AB_FOLD_CASE(32, 16)
    AB_FOLD_CASE(64, 32)
    default:
      set_error("fused fold: osamp %d not supported (4..64)", fa.O);
      return AB_ERR_UNSUPPORTED;
  }
#undef AB_FOLD_CASE
}

int launch_time_fold(ab_ctx* ctx, float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM,
                     const float2* twN, const float* wtaps, int ntap, float thresh, const FoldArgs& fa,
                     const float2* tw64, cudaStream_t s) {
  size_t smem = time_smem_bytes(N) + sizeof(float) * 4 * 64;
  AB_CHECK_ARG(smem <= ctx->smem_optin, "time stage: nslice %d needs %zu bytes of shared memory (max %zu)", N, smem,
               ctx->smem_optin);
  AB_CHECK_ARG(wtaps && ntap == 4 && fa.ntap == 4, "fused fold: needs ntap = 4");
  const int M = N / 2;
  const float2* tws = nullptr;
  const int2* pairs = nullptr;
  FftPlan sp;
  bool tuned = false;
  { FftPlan tmp; ctx_plan(ctx, M, &tmp, &tuned); }
  if (M == Plan16464::N && !tuned) {
    AB_TRY(get_twiddle_stream(ctx, M, {7, 7, 7, 3, 16}, &tws));
    make_plan_from(M, {7, 7, 7, 3, 16}, &sp);
    AB_TRY(get_pair_table(ctx, sp, &pairs));
    return launch_fold_o<Plan16464, 1024>(buf, ld, ninputs, P, N, planM, twN, tws, pairs, wtaps, ntap, thresh, fa,
                                          tw64, smem, s);
  }
  if (M == Plan16384::N && !tuned) {
    AB_TRY(get_twiddle_stream(ctx, M, {4, 16, 16, 16}, &tws));
    make_plan_from(M, {4, 16, 16, 16}, &sp);
    AB_TRY(get_pair_table(ctx, sp, &pairs));
    return launch_fold_o<Plan16384, 1024>(buf, ld, ninputs, P, N, planM, twN, tws, pairs, wtaps, ntap, thresh, fa,
                                          tw64, smem, s);
  }
  AB_TRY(get_pair_table(ctx, planM, &pairs));
  return launch_fold_o<NoPlan, kTimeThreads>(buf, ld, ninputs, P, N, planM, twN, nullptr, pairs, wtaps, ntap, thresh,
                                             fa, tw64, smem, s);
}

}  // namespace ab

using namespace ab;

extern "C" int ab_get_matft(ab_ctx* ctx, float* matft, int64_t nslice, int64_t nchan, int64_t ntap, void* stream) {
  AB_CHECK_ARG(ctx && matft, "ab_get_matft: NULL pointer");
  AB_CHECK_ARG(nslice >= 1 && nchan >= 2 && ntap >= 1, "ab_get_matft: bad sizes");
  int64_t P = 2 * (nchan - 1), nf = nslice / 2 + 1;
  std::vector<double> w;
  sinc_hamming_host((int)ntap, P, w);
  double* dw = nullptr;
  AB_CUDA(cudaMalloc(&dw, sizeof(double) * w.size()));
  cudaStream_t s = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(dw, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    int64_t total = P * nf;
    matft_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(dw, (int)P, (int)ntap, nslice, nf,
                                                                 (float2*)matft, 0.0, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dw);
  if (e != cudaSuccess) {
    set_error("ab_get_matft: %s", cudaGetErrorString(e));
    return AB_ERR_CUDA;
  }
  return AB_OK;
}

// Fused FP64 matft + filter, used by the Python layer when both are wanted.
extern "C" int ab_build_filter(ab_ctx* ctx, float* filt, int64_t nslice, int64_t nchan, int64_t ntap,
                               double thresh, void* stream) {
  AB_CHECK_ARG(ctx && filt, "ab_build_filter: NULL pointer");
  AB_CHECK_ARG(nslice >= 1 && nchan >= 2 && ntap >= 1, "ab_build_filter: bad sizes");
  int64_t P = 2 * (nchan - 1), nf = nslice / 2 + 1;
  std::vector<double> w;
  sinc_hamming_host((int)ntap, P, w);
  double* dw = nullptr;
  AB_CUDA(cudaMalloc(&dw, sizeof(double) * w.size()));
  cudaStream_t s = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(dw, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    int64_t total = P * nf;
    matft_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(dw, (int)P, (int)ntap, nslice, nf,
                                                                 (float2*)filt, thresh, 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dw);
  if (e != cudaSuccess) {
    set_error("ab_build_filter: %s", cudaGetErrorString(e));
    return AB_ERR_CUDA;
  }
  return AB_OK;
}

extern "C" int ab_calculate_filter(const float* matft, float* filt, int64_t n, double thresh, void* stream) {
  AB_CHECK_ARG(matft && filt && n >= 0, "ab_calculate_filter: bad arguments");
  if (n == 0) return AB_OK;
  filter_kernel<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>((const float2*)matft, (float2*)filt, n,
                                                                            thresh);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_ipfb(ab_ctx* ctx, const float* dat, const float* filt, float* out, int64_t nslice, int64_t nchan,
                       void* stream) {
  AB_CHECK_ARG(ctx && dat && filt && out, "ab_ipfb: NULL pointer");
  AB_CHECK_ARG(nslice >= 2 && nslice % 2 == 0, "ab_ipfb: nslice must be even and >= 2 (got %lld)", (long long)nslice);
  AB_CHECK_ARG(nchan >= 3, "ab_ipfb: nchan must be >= 3");
  AB_CHECK_ARG(((uintptr_t)out & 7) == 0, "ab_ipfb: out must be 8-byte aligned");
  int P = (int)(2 * (nchan - 1));
  FftPlan planP, planM;
  if (!ctx_plan(ctx, P, &planP)) {
    set_error("ab_ipfb: lblock %d does not factor into 2,3,5,7", P);
    return AB_ERR_UNSUPPORTED;
  }
  if (!ctx_plan(ctx, (int)(nslice / 2), &planM) && !make_plan_any((int)(nslice / 2), &planM)) {
    set_error("ab_ipfb: no FFT plan for nslice/2 = %lld", (long long)(nslice / 2));
    return AB_ERR_UNSUPPORTED;
  }
  if (plan_has_generic(planM)) {
    // prime factors above 7: the largest by Bluestein's method when its
    // convolution fits in shared memory beside the column, the others (and
    // that one otherwise) as direct DFT passes through a scratch column per CTA
    int rmax = 0;
    for (int q = 0; q < planM.npass; q++) rmax = std::max(rmax, planM.radix[q]);
    if (rmax >= 32) {
      BluesteinPass bs{};
      AB_TRY(get_bluestein(ctx, rmax, &bs));
      if (time_smem_bytes((int)nslice) + sizeof(float2) * (size_t)padded_len(bs.L) <= ctx->smem_optin) planM.bs = bs;
    }
    bool direct = false;
    for (int q = 0; q < planM.npass; q++) {
      const int r = planM.radix[q];
      direct |= r != 2 && r != 3 && r != 4 && r != 5 && r != 7 && r != 8 && r != planM.bs.R;
    }
    if (direct) {
      void* g = nullptr;
      AB_TRY(get_scratch(ctx, kScratchDftPass, sizeof(float2) * (size_t)P * (size_t)planM.n, &g));
      planM.gscratch = (float2*)g;
    }
  }
  const float2 *twP, *twN;
  AB_TRY(get_twiddles(ctx, P, &twP));
  AB_TRY(get_twiddles(ctx, nslice, &twN));
  cudaStream_t s = as_stream(stream);
  AB_TRY(launch_row_stage_c64(ctx, (const float2*)dat, nslice, P, planP, twP, out, nslice, s));
  AB_TRY(launch_time_stage(ctx, out, nslice, 1, P, (int)nslice, planM, twN, (const float2*)filt, nullptr, 0, 0.f, s));
  return AB_OK;
}
