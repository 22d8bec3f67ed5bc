// fir.cu -- the IPFB time-axis Wiener deconvolution as a short two-sided FIR,
// fused with the forward-PFB fold, for the streaming chain.
//
// Reference (cupy_ipfb, albatros_analysis/src/utils/pfb_gpu_utils.py:56-91):
// per sample phase n the column x[t] (t < nslice) is transformed along time,
// multiplied by filt[n, f] and transformed back, i.e. circularly convolved with
//   h_n = irfft(filt[n, :]),  filt = m (1+t^2) / (t^2 + |m|^2),
//   m[n, f] = sum_{k<ntap} w[k*P + n] exp(-2 pi i f k / nslice)
// (get_matft :123-137, calculate_filter :29-36).  filt is a rational function
// of exp(-2 pi i f / nslice) whose poles stay away from the unit circle while
// the Wiener threshold is not small, so h_n decays geometrically: with the
// default threshold 0.45 and the 4-tap sinc-Hamming window, the taps beyond
// |j| = 32 carry 2e-9 of the filter's energy.  The time stage here evaluates
//   y[t] = sum_{|j| <= J} h_n[j] x[(t - j) mod nslice]
// for the kept rows t in [cut, cut + acclen) only, with the taps h_n computed
// once in FP64 from the reference's filter at the same nslice DFT bins (so the
// circular wrap of the reference is reproduced for cut < J) and J chosen per
// filter so that the dropped tail is below 1e-7 of the filter norm (else the
// FFT time stage runs).  This replaces two nslice-point FFTs per column with
// 2J+1 FMAs per kept sample.
//
// Kernel layout: one CTA per (segment of a column, column n, input).  A
// segment owns the fine blocks whose last row falls in its kept rows
// [s0, s0 + S); it recomputes the 4*O rows before s0 (segment 0 reads them
// from the previous chunk's tail state instead), folds and DFTs its blocks
// into W, and the last segment writes this chunk's last 4*O rows to the other
// half of the double-buffered tail state.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "fold.cuh"
#include "ipfb.cuh"

namespace ab {

// ---------------------------------------------------------------------------
// FP64 taps.  For column n: h[n][j + JM] = (1/N) sum_{f=0}^{N-1} H(f) e^{2 pi i f j / N}
// for |j| <= JM, with H the Hermitian filter of the reference (the sum over
// f <= N/2 with weight 2 for the interior bins), and energy[n] = sum over all
// j of h^2 (Parseval).  T[k] = e^{2 pi i k / N} in double.
constexpr int kFirJMax = 96;
constexpr int kFirTapsThreads = 256;

__global__ void __launch_bounds__(kFirTapsThreads)
    fir_taps_kernel(const double* __restrict__ w, int ntap, int P, int N, double thresh,
                    const double2* __restrict__ T, double* __restrict__ h, double* __restrict__ energy) {
  constexpr int NJ = 2 * kFirJMax + 1, TILE = kFirTapsThreads;
  __shared__ double2 Hs[TILE];
  __shared__ double red[kFirTapsThreads];
  const int n = blockIdx.x, tid = threadIdx.x;
  const int j = tid - kFirJMax;
  const int nf = N / 2 + 1;
  const double t2 = thresh * thresh;
  double acc = 0.0, eacc = 0.0;
  double2 step = make_double2(1.0, 0.0);
  if (tid < NJ) {
    const int a = j >= 0 ? j : -j;
    step = T[a % N];
    if (j < 0) step.y = -step.y;  // e^{2 pi i j / N}
  }
  for (int f0 = 0; f0 < nf; f0 += TILE) {
    const int f = f0 + tid;
    if (f < nf) {
      const double2 zc = T[f];  // e^{+2 pi i f / N}; z = conj
      const double zr = zc.x, zi = -zc.y;
      double mr = w[(int64_t)(ntap - 1) * P + n], mi = 0.0;
      for (int k = ntap - 2; k >= 0; k--) {  // Horner in z = e^{-2 pi i f / N}
        const double r = mr * zr - mi * zi, i = mr * zi + mi * zr;
        mr = r + w[(int64_t)k * P + n];
        mi = i;
      }
      const double a2 = mr * mr + mi * mi;
      const double g = thresh > 0 ? (1.0 + t2) / (t2 + a2) : 1.0 / a2;
      const double c = (f == 0 || 2 * f == N) ? 1.0 : 2.0;
      const double hr = mr * g, hi = mi * g;
      Hs[tid] = make_double2(c * hr, c * hi);
      eacc += c * (hr * hr + hi * hi);
    } else {
      Hs[tid] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    if (tid < NJ) {
      long long k = ((long long)f0 * j) % N;
      if (k < 0) k += N;
      double2 p = T[k];  // e^{2 pi i f0 j / N}, then advanced by `step`
      const int cnt = min(TILE, nf - f0);
      for (int q = 0; q < cnt; q++) {
        const double2 H = Hs[q];
        acc = fma(H.x, p.x, fma(-H.y, p.y, acc));
        const double pr = p.x * step.x - p.y * step.y;
        p.y = p.x * step.y + p.y * step.x;
        p.x = pr;
      }
    }
    __syncthreads();
  }
  red[tid] = eacc;
  __syncthreads();
  for (int s = kFirTapsThreads / 2; s > 0; s >>= 1) {
    if (tid < s) red[tid] += red[tid + s];
    __syncthreads();
  }
  if (tid == 0) energy[n] = red[0] / (double)N;
  if (tid < NJ) h[(int64_t)n * NJ + tid] = acc / (double)N;
}

// Choose J and build the float taps (P, 2J+1), cached in the context.
int get_fir_taps(ab_ctx* ctx, int P, int N, int ntap, float thresh, int* J_out, const float** taps_out) {
  *J_out = 0;
  *taps_out = nullptr;
  uint32_t tb;
  memcpy(&tb, &thresh, sizeof(tb));
  std::vector<int64_t> key = {P, N, ntap, (int64_t)tb};
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->fir_taps.find(key);
    if (it != ctx->fir_taps.end()) {
      *J_out = it->second.first;
      *taps_out = it->second.second;
      return AB_OK;
    }
  }
  constexpr int JM = kFirJMax, NJ = 2 * JM + 1;
  std::vector<double> w;
  sinc_hamming_host(ntap, P, w);
  std::vector<double2> T(N);
  for (int k = 0; k < N; k++) {
    const double a = 2.0 * M_PI * (double)k / (double)N;
    T[k] = make_double2(std::cos(a), std::sin(a));
  }
  double *dw = nullptr, *dh = nullptr, *de = nullptr;
  double2* dT = nullptr;
  auto release = [&]() {
    cudaFree(dw);
    cudaFree(dh);
    cudaFree(de);
    cudaFree(dT);
  };
  if (cudaMalloc(&dw, sizeof(double) * w.size()) != cudaSuccess ||
      cudaMalloc(&dT, sizeof(double2) * T.size()) != cudaSuccess ||
      cudaMalloc(&dh, sizeof(double) * (size_t)P * NJ) != cudaSuccess ||
      cudaMalloc(&de, sizeof(double) * (size_t)P) != cudaSuccess) {
    release();
    set_error("FIR taps: device allocation failed");
    return AB_ERR_NOMEM;
  }
  std::vector<double> h((size_t)P * NJ), e(P);
  cudaError_t err = cudaMemcpy(dw, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(dT, T.data(), sizeof(double2) * T.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    fir_taps_kernel<<<P, kFirTapsThreads>>>(dw, ntap, P, N, (double)thresh, dT, dh, de);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpy(h.data(), dh, sizeof(double) * h.size(), cudaMemcpyDeviceToHost);
  if (err == cudaSuccess) err = cudaMemcpy(e.data(), de, sizeof(double) * e.size(), cudaMemcpyDeviceToHost);
  release();
  if (err != cudaSuccess) {
    set_error("FIR taps: %s", cudaGetErrorString(err));
    return AB_ERR_CUDA;
  }
  // smallest J in {32, 64} whose dropped tail is below 1e-7 of the filter's
  // L2 norm in every column.  The tail is measured directly on the computed
  // taps (no cancellation): the energy in J < |j| <= JM, doubled for J = 64 to
  // cover |j| > JM (the taps decay geometrically, so the part beyond JM is
  // smaller than the part just inside it).  A filter that decays slowly, or
  // an nslice so short that the taps alias (2*JM + 1 > N), fails the test.
  int J = 0;
  for (int cand : {32, 64}) {
    if (2 * JM + 1 > N) break;
    double worst = 0.0;
    bool finite = true;
    for (int n = 0; n < P && finite; n++) {
      const double* hn = &h[(size_t)n * NJ];
      double tail = 0.0;
      for (int q = 0; q < NJ; q++) {
        const int j = q - JM;
        if (j < -cand || j > cand) tail += hn[q] * hn[q];
      }
      if (cand == 64) tail *= 2.0;
      finite = std::isfinite(tail) && std::isfinite(e[n]) && e[n] > 0;
      worst = std::max(worst, std::sqrt(tail / e[n]));
    }
    if (finite && worst <= 1e-7) {
      J = cand;
      break;
    }
  }
  float* dtaps = nullptr;
  if (J > 0) {
    const int K = 2 * J + 1;
    std::vector<float> hf((size_t)P * K);
    for (int n = 0; n < P; n++)
      for (int k = 0; k < K; k++) hf[(size_t)n * K + k] = (float)h[(size_t)n * NJ + (k - J + JM)];
    if (cudaMalloc(&dtaps, sizeof(float) * hf.size()) != cudaSuccess) {
      set_error("FIR taps: device allocation failed");
      return AB_ERR_NOMEM;
    }
    if (cudaMemcpy(dtaps, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(dtaps);
      set_error("FIR taps: upload failed");
      return AB_ERR_CUDA;
    }
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->fir_taps.find(key);
  if (it != ctx->fir_taps.end()) {  // another thread got there first
    cudaFree(dtaps);
  } else {
    it = ctx->fir_taps.emplace(key, std::make_pair(J, (const float*)dtaps)).first;
  }
  *J_out = it->second.first;
  *taps_out = it->second.second;
  return AB_OK;
}

// ---------------------------------------------------------------------------
// FIR + fold.  U kept rows per thread (one unit), NTHR threads: a CTA computes
// up to R = U*NTHR rows, S = R - 4*O of them new (the rest re-create the fine
// blocks' overlap).  Shared memory: the x window (padded one float per U) and
// the y rows in the pidx float2 layout the fold reads.
constexpr int kFirThreads = 256;

__host__ __device__ constexpr int fir_xpad(int n, int U) { return n + n / U + 1; }

template <int J, int U, int G>
__global__ void __launch_bounds__(kFirThreads, J <= 32 ? 2 : 1)
    fir_fold_kernel(const float* __restrict__ data, int64_t ld, int P, int nslice, int cut, int acclen, int S,
                    const float* __restrict__ taps, FoldArgs fa, const float* __restrict__ state_in,
                    float* __restrict__ state_out, const float2* __restrict__ tw64) {
  constexpr int O = 2 * G, K = 2 * J + 1, R = U * kFirThreads;
  extern __shared__ float2 smem2[];
  float* xs = reinterpret_cast<float*>(smem2);
  float2* ys2 = smem2 + (fir_xpad(R + 2 * J + U, U) + 1) / 2;  // float2-aligned
  float* ys = reinterpret_cast<float*>(ys2);
  const int seg = blockIdx.x, n = blockIdx.y, in = blockIdx.z, tid = threadIdx.x;
  const int s0 = seg * S;
  const int s1 = min(s0 + S, acclen);
  const bool first = seg == 0, last = s0 + S >= acclen;
  const int ylo = first ? 0 : s0 - 4 * O;  // first row computed here
  const int nrows = s1 - ylo;              // <= R
  const int yoff = ylo - s0 + 4 * O;       // ys row of computed row ylo
  const float* col = data + ((int64_t)in * P + n) * ld;
  // x window: xs[e] = x[(cut + ylo - J + e) mod nslice], e < nrows + 2J (+ slack)
  const int xbase = cut + ylo - J;
  const int nx = nrows + 2 * J;
  for (int e = tid; e < nx + U; e += kFirThreads) {
    float v = 0.f;
    if (e < nx) {
      int t = xbase + e;
      if (t < 0 || t >= nslice) t = ((t % nslice) + nslice) % nslice;
      v = __ldg(col + t);
    }
    xs[e + e / U] = v;
  }
  const float* st_in = state_in + ((int64_t)in * P + n) * (4 * O);
  if (first) {
    for (int i = tid; i < 4 * O; i += kFirThreads) ys[2 * pidx(i >> 1) + (i & 1)] = st_in[i];
  }
  float h[K];
#pragma unroll
  for (int k = 0; k < K; k++) h[k] = __ldg(&taps[(int64_t)n * K + k]);
  __syncthreads();
  // y[ylo + i] = sum_j h[j + J] x[cut + ylo + i - j] = sum_{k} h[k] xs[i + 2J - k]
  if (tid * U < nrows) {
    float acc[U];
#pragma unroll
    for (int g = 0; g < U; g++) acc[g] = 0.f;
    const float* xu = xs + tid * (U + 1);  // xs index of e = tid*U (one pad float per U)
#pragma unroll
    for (int ep = 0; ep < U + 2 * J; ep++) {
      const float v = xu[ep + ep / U];
#pragma unroll
      for (int g = 0; g < U; g++) {
        const int k = g + 2 * J - ep;
        if (k >= 0 && k < K) acc[g] = fmaf(h[k], v, acc[g]);
      }
    }
    const int t0 = yoff + tid * U;  // even
#pragma unroll
    for (int q = 0; q < U / 2; q++) ys2[pidx((t0 >> 1) + q)] = make_float2(acc[2 * q], acc[2 * q + 1]);
  }
  __syncthreads();
  // blocks whose last row lies in [s0, s0 + S) (the last segment: >= s0)
  const int row0 = (int)fa.row0, nb = (int)fa.nb;
  auto first_block_ending_at_or_after = [&](int r) -> int {  // min b with row0 + b*O + 4O - 1 >= r
    const int num = r - 4 * O + 1 - row0;
    int b = num <= 0 ? 0 : (num + O - 1) / O;
    return min(b, nb);
  };
  const int b0 = first ? 0 : first_block_ending_at_or_after(s0);
  const int b1 = last ? nb : first_block_ending_at_or_after(s0 + S);
  if (b1 > b0) {
    FoldArgs f2 = fa;
    f2.cut = 4 * O - s0;  // ys row of chunk row rr is 4O - s0 + rr
    f2.acclen = s1;       // rows >= s1 are zero (only past the end of the stream)
    fold_blocks<G, 4, true>(ys2, nullptr, f2, P, n, in, tw64, b0, b1);
  }
  if (last) {
    float* st = state_out + ((int64_t)in * P + n) * (4 * O);
    for (int i = tid; i < 4 * O; i += kFirThreads) {
      const int t = 4 * O - s0 + (acclen - 4 * O + i);
      st[i] = ys[2 * pidx(t >> 1) + (t & 1)];
    }
  }
}

template <int J, int U>
static size_t fir_smem_bytes(int O) {
  constexpr int R = U * kFirThreads;
  const size_t xs2 = (size_t)(fir_xpad(R + 2 * J + U, U) + 1) / 2;
  return sizeof(float2) * (xs2 + (size_t)padded_len((R + 4 * O + U) / 2 + 1));
}

template <int J, int U, int G>
static int launch_fir_t(const FirArgs& a, const FoldArgs& fa, cudaStream_t s) {
  constexpr int O = 2 * G, R = U * kFirThreads;
  const int S = R - 4 * O;
  const int nseg = std::max(1, (a.acclen + S - 1) / S);
  const size_t smem = fir_smem_bytes<J, U>(O);
  AB_CUDA(cudaFuncSetAttribute(fir_fold_kernel<J, U, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)nseg, (unsigned)a.P, (unsigned)a.ninputs);
  fir_fold_kernel<J, U, G><<<grid, kFirThreads, smem, s>>>(a.data, a.ld, a.P, a.nslice, a.cut, a.acclen, S, a.taps,
                                                           fa, a.state_in, a.state_out, a.tw64);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

template <int J, int U>
static int launch_fir_o(const FirArgs& a, const FoldArgs& fa, cudaStream_t s) {
  switch (fa.O) {
    case 4: return launch_fir_t<J, U, 2>(a, fa, s);
    case 8: return launch_fir_t<J, U, 4>(a, fa, s);
    case 16: return launch_fir_t<J, U, 8>(a, fa, s);
    case 32: return launch_fir_t<J, U, 16>(a, fa, s);
    case 64: return launch_fir_t<J, U, 32>(a, fa, s);
    default:
      set_error("FIR time stage: osamp %d not supported (4..64)", fa.O);
      return AB_ERR_UNSUPPORTED;
  }
}

int launch_fir_fold(const FirArgs& a, const FoldArgs& fa, cudaStream_t s) {
  AB_CHECK_ARG(fa.ntap == 4, "FIR time stage: needs ntap = 4");
  AB_CHECK_ARG(a.P <= 65535 && a.ninputs <= 65535, "FIR time stage: grid too large");
  AB_CHECK_ARG(a.row_tile == 16 || a.row_tile == 32, "FIR time stage: row tile must be 16 or 32");
  AB_CHECK_ARG(a.row_tile * kFirThreads > 4 * fa.O, "FIR time stage: row tile too small for osamp %d", fa.O);
  if (a.J == 32) return a.row_tile == 32 ? launch_fir_o<32, 32>(a, fa, s) : launch_fir_o<32, 16>(a, fa, s);
  if (a.J == 64) return a.row_tile == 32 ? launch_fir_o<64, 32>(a, fa, s) : launch_fir_o<64, 16>(a, fa, s);
  set_error("FIR time stage: J = %d not supported", a.J);
  return AB_ERR_UNSUPPORTED;
}

}  // namespace ab
