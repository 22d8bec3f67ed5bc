// ipfb.cu -- inverse PFB: FP64 window-matrix spectrum and Wiener filter,
// row-stage inverse FFT (fused with 4-bit decode and channel placement for
// the streaming chain), and the time-axis Wiener deconvolution.
//
// Reference: cupy_ipfb (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91):
//   dd   = irfft(dat, axis=1)                 (nslice, P), /P
//   ddft = rfft(dd.T, axis=1)                 (P, nslice/2+1)
//   res  = irfft(ddft * filt, axis=1).T       /nslice
// Here stage 1 computes dd in the [n][t] layout (column n = sample phase,
// contiguous in t), stage 2 does rfft -> *filt -> irfft on each column inside
// one CTA's shared memory.
#include <math.h>

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
constexpr int kRowFftsPerCta = 2;
constexpr int kRowThreadsPerFft = 256;

// value of bin k of a real spectrum pair into Z (k in [0, P/2])
__device__ __forceinline__ void put_pair(float2* buf, const FftPlan& p, int P, int k, float2 A, float2 B) {
  if (k == 0 || 2 * k == P) {
    buf[fft_pos(p, k)] = make_float2(A.x, B.x);  // imag parts of DC / Nyquist ignored (irfft)
  } else {
    buf[fft_pos(p, k)] = make_float2(A.x - B.y, A.y + B.x);          // A + iB
    buf[fft_pos(p, P - k)] = make_float2(A.x + B.y, B.x - A.y);      // conj(A) + i conj(B)
  }
}

__device__ __forceinline__ void row_dit(float2* buf, const FftPlan& p, const float2* tw, int T, int tid, int nthr) {
  for (int q = p.npass - 1; q >= 0; q--) {
    run_pass<true>(p.radix[q], buf, p.n, p.span[q], tw, T, tid, nthr);
    __syncthreads();
  }
}

__device__ __forceinline__ float dec4f(unsigned v) { return (float)((int)((v + 7u) & 15u) - 7); }

// grid: (ceil(nrows / kRowFftsPerCta), nant); one FFT per spectrum row, both pols.
__global__ void __launch_bounds__(kRowFftsPerCta* kRowThreadsPerFft)
    row_stage_packed4_kernel(Packed4Src src, int nrows, FftPlan plan, const float2* __restrict__ tw,
                             float* __restrict__ out, int64_t ld) {
  extern __shared__ float2 smem[];
  const int P = plan.n;
  const int a = blockIdx.y;
  const int sub = threadIdx.x / kRowThreadsPerFft, ltid = threadIdx.x % kRowThreadsPerFft;
  const int t = blockIdx.x * kRowFftsPerCta + sub;
  float2* buf = smem + (size_t)sub * P;
  for (int i = ltid; i < P; i += kRowThreadsPerFft) buf[i] = make_float2(0.f, 0.f);
  __syncthreads();
  int64_t rawrow = -1;
  if (t < nrows) {
    int64_t g = src.g0 + t;
    if (g >= 0) rawrow = src.spec_map ? (int64_t)src.spec_map[(int64_t)a * src.map_stride + g] : g;
  }
  if (rawrow >= 0) {
    const uint8_t* row = src.raw + (int64_t)a * src.ant_stride + rawrow * src.row_bytes;
    for (int k = ltid; k < src.nsel; k += kRowThreadsPerFft) {
      uchar2 b = *reinterpret_cast<const uchar2*>(row + 2 * __ldg(&src.chan_cols[k]));
      float2 A = make_float2(dec4f(b.x >> 4), dec4f(b.x & 15u));
      float2 B = make_float2(dec4f(b.y >> 4), dec4f(b.y & 15u));
      put_pair(buf, plan, P, __ldg(&src.chan_abs[k]), A, B);
    }
  }
  __syncthreads();
  row_dit(smem + (size_t)sub * P, plan, tw, P, ltid, kRowThreadsPerFft);
  // write: column n of input (2a+p) at row t; threads of a warp take
  // consecutive rows of the same n where possible
  const float inv = 1.0f / (float)P;
  const int nthr = kRowFftsPerCta * kRowThreadsPerFft;
  const int64_t t0 = (int64_t)blockIdx.x * kRowFftsPerCta;
  for (int i = threadIdx.x; i < kRowFftsPerCta * P; i += nthr) {
    int n = i / kRowFftsPerCta, f = i - n * kRowFftsPerCta;
    int64_t tt = t0 + f;
    if (tt >= nrows) continue;
    float2 z = smem[(size_t)f * P + n];
    out[((int64_t)(2 * a) * P + n) * ld + tt] = z.x * inv;
    out[((int64_t)(2 * a + 1) * P + n) * ld + tt] = z.y * inv;
  }
}

// dense c64 rows (nslice, P/2+1): one FFT for rows (2j, 2j+1)
__global__ void __launch_bounds__(kRowFftsPerCta* kRowThreadsPerFft)
    row_stage_c64_kernel(const float2* __restrict__ dat, int64_t nslice, FftPlan plan,
                         const float2* __restrict__ tw, float* __restrict__ out, int64_t ld) {
  extern __shared__ float2 smem[];
  const int P = plan.n, nb = P / 2 + 1;
  const int sub = threadIdx.x / kRowThreadsPerFft, ltid = threadIdx.x % kRowThreadsPerFft;
  const int64_t ta = 2 * ((int64_t)blockIdx.x * kRowFftsPerCta + sub);
  float2* buf = smem + (size_t)sub * P;
  for (int i = ltid; i < P; i += kRowThreadsPerFft) buf[i] = make_float2(0.f, 0.f);
  __syncthreads();
  if (ta < nslice) {
    const float2* ra = dat + ta * nb;
    const float2* rb = ta + 1 < nslice ? dat + (ta + 1) * nb : nullptr;
    for (int k = ltid; k < nb; k += kRowThreadsPerFft) {
      float2 A = ra[k];
      float2 B = rb ? rb[k] : make_float2(0.f, 0.f);
      put_pair(buf, plan, P, k, A, B);
    }
  }
  __syncthreads();
  row_dit(buf, plan, tw, P, ltid, kRowThreadsPerFft);
  const float inv = 1.0f / (float)P;
  const int nthr = kRowFftsPerCta * kRowThreadsPerFft;
  const int64_t tbase = 2 * (int64_t)blockIdx.x * kRowFftsPerCta;
  for (int i = threadIdx.x; i < kRowFftsPerCta * 2 * P; i += nthr) {
    int n = i / (2 * kRowFftsPerCta), r = i - n * (2 * kRowFftsPerCta);
    int f = r >> 1, part = r & 1;
    int64_t tt = tbase + r;
    if (tt >= nslice) continue;
    float2 z = smem[(size_t)f * P + n];
    out[(int64_t)n * ld + tt] = (part ? z.y : z.x) * inv;
  }
}

// ---------------------------------------------------------------------------
// Stage 2: per column n, real FFT of length N via a complex FFT of M = N/2,
// multiply by the filter, inverse.  All in shared memory, one CTA per column.
constexpr int kTimeThreads = 1024;

template <bool TABLE>
__global__ void __launch_bounds__(kTimeThreads)
    time_stage_kernel(float* __restrict__ data, int64_t ld, int P, int N, FftPlan plan,
                      const float2* __restrict__ twN, const float2* __restrict__ table,
                      const float* __restrict__ wtaps, int ntap, float thresh) {
  extern __shared__ float2 buf[];
  const int n = blockIdx.x, input = blockIdx.y;
  const int M = N / 2;
  float* col = data + ((int64_t)input * P + n) * ld;
  const float2* col2 = reinterpret_cast<const float2*>(col);
  for (int m = threadIdx.x; m < M; m += blockDim.x) buf[m] = col2[m];
  // window taps of this column for the on-the-fly filter
  float w[8];
  if (!TABLE) {
#pragma unroll
    for (int t = 0; t < 8; t++) w[t] = t < ntap ? __ldg(&wtaps[(int64_t)t * P + n]) : 0.f;
  }
  __syncthreads();
  dif_forward(buf, plan, twN, N);

  const float scale = 0.5f / (float)N;  // irfft 1/N and the untangle's 1/2
  const float t2 = thresh * thresh;
  auto filt = [&](int k) -> float2 {
    float2 h;
    if (TABLE) {
      h = __ldg(&table[(int64_t)n * (M + 1) + k]);
    } else {
      float2 m = make_float2(0.f, 0.f);
      for (int t = 0; t < ntap; t++) {
        int e = (int)(((int64_t)t * k) % N);
        float2 z = __ldg(&twN[e]);
        m.x = fmaf(w[t], z.x, m.x);
        m.y = fmaf(w[t], z.y, m.y);
      }
      float a2 = fmaf(m.x, m.x, m.y * m.y);
      float g = thresh > 0.f ? (1.f + t2) / (t2 + a2) : 1.f / a2;
      h = make_float2(m.x * g, m.y * g);
    }
    return cscale(h, scale);
  };

  for (int k = threadIdx.x; k <= M / 2; k += blockDim.x) {
    if (k == 0) {
      float2 z = buf[0];
      float x0 = 2.f * (z.x + z.y), xm = 2.f * (z.x - z.y);  // 2 X[0], 2 X[M] (real)
      float y0 = x0 * filt(0).x, ym = xm * filt(M).x;          // real parts only (irfft)
      buf[0] = make_float2(y0 + ym, y0 - ym);
      continue;
    }
    int pk = fft_pos(plan, k), pc = fft_pos(plan, M - k);
    float2 zk = buf[pk], zc = buf[pc];
    float2 w1 = __ldg(&twN[k]);                  // exp(-2 pi i k / N)
    float2 E = cadd(zk, cconj(zc));              // 2 E_k
    float2 Od = csub(zk, cconj(zc));             // 2 i O_k
    float2 O = make_float2(Od.y, -Od.x);         // 2 O_k = (2 i O_k) / i
    float2 wO = cmul(w1, O);
    float2 Xk = cadd(E, wO);                     // 2 X_k
    float2 Xc = cconj(csub(E, wO));              // 2 X_{M-k}
    float2 Yk = cmul(Xk, filt(k));
    float2 Yc = cmul(Xc, filt(M - k));
    float2 Et = cadd(Yk, cconj(Yc));
    float2 Ot = cmulc(csub(Yk, cconj(Yc)), w1);  // (Y_k - conj Y_{M-k}) conj(w)
    float2 iOt = make_float2(-Ot.y, Ot.x);
    buf[pk] = cadd(Et, iOt);
    if (pc != pk) buf[pc] = cadd(cconj(Et), make_float2(Ot.y, Ot.x));  // conj(Et) + i conj(Ot)
  }
  __syncthreads();
  dit_inverse(buf, plan, twN, N);
  float2* out2 = reinterpret_cast<float2*>(col);
  for (int m = threadIdx.x; m < M; m += blockDim.x) out2[m] = buf[m];
}

int launch_row_stage_packed4(const Packed4Src& src, int nant, int nrows, int P, const FftPlan& plan,
                             const float2* twP, float* out, int64_t ld, cudaStream_t s) {
  size_t smem = sizeof(float2) * (size_t)P * kRowFftsPerCta;
  static bool attr_set = false;
  if (!attr_set) {
    AB_CUDA(cudaFuncSetAttribute(row_stage_packed4_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    attr_set = true;
  }
  AB_CHECK_ARG(smem <= 96 * 1024, "row stage: lblock %d too large", P);
  dim3 grid((unsigned)((nrows + kRowFftsPerCta - 1) / kRowFftsPerCta), (unsigned)nant);
  row_stage_packed4_kernel<<<grid, kRowFftsPerCta * kRowThreadsPerFft, smem, s>>>(src, nrows, plan, twP, out, ld);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

int launch_row_stage_c64(const float2* dat, int64_t nslice, int P, const FftPlan& plan, const float2* twP,
                         float* out, int64_t ld, cudaStream_t s) {
  size_t smem = sizeof(float2) * (size_t)P * kRowFftsPerCta;
  static bool attr_set = false;
  if (!attr_set) {
    AB_CUDA(cudaFuncSetAttribute(row_stage_c64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    attr_set = true;
  }
  AB_CHECK_ARG(smem <= 96 * 1024, "row stage: lblock %d too large", P);
  int64_t nfft = (nslice + 1) / 2;
  dim3 grid((unsigned)((nfft + kRowFftsPerCta - 1) / kRowFftsPerCta));
  row_stage_c64_kernel<<<grid, kRowFftsPerCta * kRowThreadsPerFft, smem, s>>>(dat, nslice, plan, twP, out, ld);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

int launch_time_stage(float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM,
                      const float2* twN, const float2* table, const float* wtaps, int ntap, float thresh,
                      size_t smem_optin, cudaStream_t s) {
  size_t smem = sizeof(float2) * (size_t)(N / 2);
  AB_CHECK_ARG(smem <= smem_optin, "time stage: nslice %d needs %zu bytes of shared memory (max %zu)", N, smem,
               smem_optin);
  AB_CHECK_ARG(table || (wtaps && ntap >= 1 && ntap <= 8), "time stage: need a filter table or 1..8 window taps");
  dim3 grid((unsigned)P, (unsigned)ninputs);
  if (table) {
    AB_CUDA(cudaFuncSetAttribute(time_stage_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_optin));
    time_stage_kernel<true><<<grid, kTimeThreads, smem, s>>>(buf, ld, P, N, planM, twN, table, wtaps, ntap, thresh);
  } else {
    AB_CUDA(cudaFuncSetAttribute(time_stage_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_optin));
    time_stage_kernel<false><<<grid, kTimeThreads, smem, s>>>(buf, ld, P, N, planM, twN, table, wtaps, ntap, thresh);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
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
  if (!make_plan(P, &planP)) {
    set_error("ab_ipfb: lblock %d does not factor into 2,3,5,7", P);
    return AB_ERR_UNSUPPORTED;
  }
  if (!make_plan((int)(nslice / 2), &planM)) {
    set_error("ab_ipfb: nslice/2 = %lld does not factor into 2,3,5,7", (long long)(nslice / 2));
    return AB_ERR_UNSUPPORTED;
  }
  const float2 *twP, *twN;
  AB_TRY(get_twiddles(ctx, P, &twP));
  AB_TRY(get_twiddles(ctx, nslice, &twN));
  cudaStream_t s = as_stream(stream);
  AB_TRY(launch_row_stage_c64((const float2*)dat, nslice, P, planP, twP, out, nslice, s));
  AB_TRY(launch_time_stage(out, nslice, 1, P, (int)nslice, planM, twN, (const float2*)filt, nullptr, 0, 0.f,
                           ctx->smem_optin, s));
  return AB_OK;
}
