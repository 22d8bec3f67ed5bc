// fir.cu -- the IPFB time-axis Wiener deconvolution as a short filter, fused
// with the forward-PFB fold, for the streaming chain: as a (2J+1)-tap FIR
// (this header) or as its IIR factorisation (from "IIR time stage" on), which
// the chain tries first.
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
// Kernel layout: persistent CTAs (two per SM; one for the 129-tap FIR) walk the items
// (segment of a column, column n, input), staging the next item's rows with
// cp.async while they compute the current one.  A
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
// IIR form of the same filter.  With W(z) = sum_{k<4} w_k z^-k (the column's
// window taps, m = W(exp(2 pi i f / nslice))), the reference's filter is
//   H(z) = W(z) (1 + t^2) / D(z),  D(z) = t^2 + W(z) W(1/z),
// and D, positive on the unit circle, factors as D(z) = B(z) B(1/z) with
// B(z) = b_0 + b_1 z^-1 + b_2 z^-2 + b_3 z^-3 minimum-phase (Wilson's
// iteration: Newton's method on B(z)B(1/z) = D(z), started from a constant).
// So y = g W(z) / (A(z) A(1/z)) x with A = B / b_0 and g = (1 + t^2) / b_0^2:
// a 4-tap FIR, a causal 3-pole recursion and an anti-causal 3-pole recursion,
// 11 FMAs per sample.  Applied to the periodic column it reproduces the
// circular convolution.  The threads of a CTA run the recursions over
// consecutive row ranges and pass their end states on (iir_fold_kernel); a
// state is carried over at least IW rows, after which 1/A's impulse response
// is below 1e-10 of its peak, and the rest of its effect is dropped.
// Per-column IIR coefficients: g w0..g w3, a1..a3, 0, then 1/A's impulse
// response h[U-5..U-1] for the three row tiles' U (state advance over one
// thread's rows), each padded to 8 floats.
constexpr int kIirU64 = 67, kIirU32 = 41, kIirU16 = 21, kIirCoef = 32;
__host__ __device__ constexpr int iir_hh_offset(int U) { return U == kIirU64 ? 24 : U == kIirU32 ? 8 : 16; }

static bool iir_factor(const double* w, double t, double coef[kIirCoef], int* carry) {
  const int m = 3;
  double d[4];
  for (int k = 0; k <= m; k++) {
    d[k] = 0.0;
    for (int i = 0; i + k <= m; i++) d[k] += w[i] * w[i + k];
  }
  d[0] += t * t;
  if (!(d[0] > 0.0)) return false;
  double b[4] = {std::sqrt(d[0]), 0.0, 0.0, 0.0};
  for (int it = 0; it < 200; it++) {
    // B X* + X B* = D + B B*, lags 0..m
    double M[4][5];
    for (int k = 0; k <= m; k++) {
      double rhs = d[k];
      for (int j = 0; j + k <= m; j++) rhs += b[j] * b[j + k];
      for (int i = 0; i <= m; i++) M[k][i] = (i >= k ? b[i - k] : 0.0) + (i + k <= m ? b[i + k] : 0.0);
      M[k][4] = rhs;
    }
    for (int c = 0; c <= m; c++) {  // Gaussian elimination with partial pivoting
      int pv = c;
      for (int r = c + 1; r <= m; r++)
        if (std::fabs(M[r][c]) > std::fabs(M[pv][c])) pv = r;
      if (std::fabs(M[pv][c]) < 1e-300) return false;
      if (pv != c)
        for (int q = 0; q < 5; q++) std::swap(M[c][q], M[pv][q]);
      for (int r = 0; r <= m; r++) {
        if (r == c) continue;
        const double f = M[r][c] / M[c][c];
        for (int q = c; q < 5; q++) M[r][q] -= f * M[c][q];
      }
    }
    double delta = 0.0, norm = 0.0;
    for (int i = 0; i <= m; i++) {
      const double x = M[i][4] / M[i][i];
      delta = std::max(delta, std::fabs(x - b[i]));
      norm = std::max(norm, std::fabs(x));
      b[i] = x;
    }
    if (!std::isfinite(norm)) return false;
    if (delta <= 1e-15 * norm) break;
  }
  // check B(z) B(1/z) = D(z) on the unit circle
  for (int q = 0; q < 64; q++) {
    const double om = M_PI * q / 63.0;
    double br = 0, bi = 0;
    for (int k = 0; k <= m; k++) {
      br += b[k] * std::cos(om * k);
      bi -= b[k] * std::sin(om * k);
    }
    double dd = d[0];
    for (int k = 1; k <= m; k++) dd += 2.0 * d[k] * std::cos(om * k);
    if (std::fabs(br * br + bi * bi - dd) > 1e-11 * dd) return false;
  }
  const double a1 = b[1] / b[0], a2 = b[2] / b[0], a3 = b[3] / b[0];
  // decay of 1/A: rows over which a recursion state must be carried
  double h[600] = {1.0};
  double peak = 1.0;
  int last = 0;
  for (int k = 1; k < 600; k++) {
    h[k] = -(a1 * h[k - 1] + (k >= 2 ? a2 * h[k - 2] : 0.0) + (k >= 3 ? a3 * h[k - 3] : 0.0));
    peak = std::max(peak, std::fabs(h[k]));
    if (std::fabs(h[k]) > 1e-10 * peak) last = k;
  }
  if (last >= 590 || peak > 1e6) return false;
  *carry = last + 1;  // rows after which 1/A's impulse response stays below 1e-10 of its peak
  const double g = (1.0 + t * t) / (b[0] * b[0]);  // folded into the FIR taps
  coef[0] = g * w[0];
  coef[1] = g * w[1];
  coef[2] = g * w[2];
  coef[3] = g * w[3];
  coef[4] = a1;
  coef[5] = a2;
  coef[6] = a3;
  for (int k = 7; k < kIirCoef; k++) coef[k] = 0.0;
  for (int i = 0; i < 5; i++) {
    coef[iir_hh_offset(kIirU32) + i] = h[kIirU32 - 5 + i];
    coef[iir_hh_offset(kIirU16) + i] = h[kIirU16 - 5 + i];
    coef[iir_hh_offset(kIirU64) + i] = h[kIirU64 - 5 + i];
  }
  return true;
}

// Per-column IIR coefficients as float (P, kIirCoef) and the state-carry
// length IW in {40, 80} rows (0 when no factorisation or a longer carry is
// needed), cached in the context per (P, ntap, thresh).
int get_iir_coeffs(ab_ctx* ctx, int P, int ntap, float thresh, int* W_out, const float** coef_out) {
  *W_out = 0;
  *coef_out = nullptr;
  if (ntap != 4) return AB_OK;
  uint32_t tb;
  memcpy(&tb, &thresh, sizeof(tb));
  std::vector<int64_t> key = {-1, P, ntap, (int64_t)tb};
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->fir_taps.find(key);
    if (it != ctx->fir_taps.end()) {
      *W_out = it->second.first;
      *coef_out = it->second.second;
      return AB_OK;
    }
  }
  std::vector<double> w;
  sinc_hamming_host(ntap, P, w);
  std::vector<float> cf((size_t)P * kIirCoef);
  int carry = 0;
  bool ok = thresh > 0.f;
  for (int n = 0; n < P && ok; n++) {
    double wn[4], c[kIirCoef];
    for (int k = 0; k < 4; k++) wn[k] = w[(size_t)k * P + n];
    int wm = 0;
    ok = iir_factor(wn, (double)thresh, c, &wm);
    carry = std::max(carry, wm);
    for (int k = 0; k < kIirCoef; k++) cf[(size_t)n * kIirCoef + k] = (float)c[k];
  }
  const int IW = !ok ? 0 : carry <= 40 ? 40 : carry <= 80 ? 80 : 0;
  float* dc = nullptr;
  if (IW > 0) {
    if (cudaMalloc(&dc, sizeof(float) * cf.size()) != cudaSuccess) {
      set_error("IIR coefficients: device allocation failed");
      return AB_ERR_NOMEM;
    }
    if (cudaMemcpy(dc, cf.data(), sizeof(float) * cf.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(dc);
      set_error("IIR coefficients: upload failed");
      return AB_ERR_CUDA;
    }
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->fir_taps.find(key);
  if (it != ctx->fir_taps.end()) {
    cudaFree(dc);
  } else {
    it = ctx->fir_taps.emplace(key, std::make_pair(IW, (const float*)dc)).first;
  }
  *W_out = it->second.first;
  *coef_out = it->second.second;
  return AB_OK;
}

// ---------------------------------------------------------------------------
// FIR + fold.  U kept rows per thread (U odd, so that lanes reading rows U
// apart hit distinct shared-memory banks), kFirThreads threads: a work item
// (segment seg of column n of input in) computes up to R = U*kFirThreads rows,
// S = R - 4*O of them new (the rest re-create the fine blocks' overlap).
// CTAs are persistent and walk the items with a stride of gridDim.x; while
// one item is filtered and folded, the next item's x window, taps, window
// coefficients and (for a first segment) tail rows are copied into the other
// staging buffer with cp.async, so the global-memory latency overlaps the FMAs.
// The fold gives each fine block to one thread: it folds the 4 taps into O
// samples and takes their real DFT in registers (compile-time radix-2 FFT of
// O/2 points plus the real-input untangle), then writes the O packed floats
// of W with 32-byte stores.
constexpr int kFirThreads = 256;
constexpr int kYPad = 2;  // pad floats per O rows of the y buffer (yidx); even, for the fold's pair loads

__constant__ float2 c_fir_tw[64];  // exp(-2 pi i k / 64)

int fir_init_device() {
  float2 tw[64];
  for (int k = 0; k < 64; k++) {
    const double a = -2.0 * M_PI * (double)k / 64.0;
    tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  AB_CUDA(cudaMemcpyToSymbol(c_fir_tw, tw, sizeof(tw)));
  return AB_OK;
}

// FIR layout: U rows per thread, R = U*kFirThreads computed rows per item,
// halo J rows each side, y rows in their own buffer.
template <int J, int U, int O>
struct FirLayout {
  static constexpr int R = U * kFirThreads;
  static constexpr int HL = J;
  static constexpr int HR = J;
  static constexpr int K = 2 * J + 1;
  static constexpr int XS = (R + HL + HR + U + 3) & ~3;  // x window (floats, unpadded)
  static constexpr int TAPS = (K + 3) & ~3;
  static constexpr int ST = 4 * O;                      // tail rows of the previous chunk
  static constexpr int WT = 4 * O;                      // window coefficients, float4 per t'
  static constexpr int STAGE = XS + TAPS + ST + WT;     // floats per staging buffer (multiple of 4)
  static constexpr int YROWS = R + 8 * O + U;           // y rows held (incl. zeros past the end)
  static constexpr int YS = YROWS + kYPad * (YROWS / O + 1) + 4;  // kYPad pad floats per O rows
  static constexpr size_t bytes() { return sizeof(float) * (2 * (size_t)STAGE + (size_t)YS); }
};

// IIR layout: thread k runs the recursions over window rows [k U, k U + U);
// window row D*U is the item's first computed row, so threads 0..D-1 (and
// the D threads after the last computed row) only run the recursions into
// the computed rows.  R = (kFirThreads - 2D) U computed rows per item.  y
// rows are written over the x window once it is dead (XS holds both), and
// each thread's end-of-range states go to two exchange arrays.
template <int U, int O, int D>
struct IirLayout {
  static constexpr int R = (kFirThreads - 2 * D) * U;
  static constexpr int XW = kFirThreads * U + 6;  // all threads' rows, 3 before, up to 3 of alignment shift
  static constexpr int YROWS = R + 8 * O;
  static constexpr int YS = YROWS + kYPad * (YROWS / O + 1) + 4;
  static constexpr int XS = ((XW > YS ? XW : YS) + 3) & ~3;
  static constexpr int TAPS = kIirCoef;
  static constexpr int STAGE = XS + TAPS + 4 * O + 4 * O;
  static constexpr int XCH = 6 * kFirThreads;  // forward and backward states, 3 floats each
  static constexpr size_t bytes() { return sizeof(float) * (2 * (size_t)STAGE + XCH); }
};


// d * exp(-2 pi i e / N) for a compile-time e
template <int N>
__device__ __forceinline__ float2 tw_mul(float2 d, int e) {
  if (e == 0) return d;
  if (4 * e == N) return make_float2(d.y, -d.x);  // * (-i)
  return cmul(d, c_fir_tw[e * (64 / N)]);
}

// In-place radix-2 DIF FFT of N points in registers (forward, exp(-2 pi i/N));
// output in bit-reversed order.  Fully unrolled: indices and twiddles are
// compile-time.
template <int N>
__device__ __forceinline__ void reg_fft_dif(float2 (&a)[N]) {
#pragma unroll
  for (int span = N / 2; span >= 1; span >>= 1) {
#pragma unroll
    for (int base = 0; base < N; base += 2 * span) {
#pragma unroll
      for (int j = 0; j < span; j++) {
        const float2 u = a[base + j], v = a[base + j + span];
        a[base + j] = cadd(u, v);
        a[base + j + span] = tw_mul<N>(csub(u, v), j * (N / (2 * span)));
      }
    }
  }
}

__host__ __device__ constexpr int bitrev(int k, int bits) {
  int r = 0;
  for (int i = 0; i < bits; i++) r |= ((k >> i) & 1) << (bits - 1 - i);
  return r;
}
__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

struct FirItem {
  int seg, n, in;
  int s0, s1, ylo, nrows;
  bool first, last;
};

// Work item -> (input, segment, column): item = (in * nseg + seg) * P + n, so
// that CTAs working side by side take neighbouring columns (whose 32-byte W
// groups share lines).  P is a power of two (pshift = log2 P); r / nseg is
// taken as a 64-bit product with mseg = ceil(2^32 / nseg), exact for
// r < 2^32 / nseg (r = in * nseg + seg is far below that).
struct ItemDecode {
  int nseg, pshift;
  uint64_t mseg;
};
__device__ __forceinline__ ItemDecode item_decode(int nseg, int P) {
  return ItemDecode{nseg, __ffs(P) - 1, ((1ull << 32) + (uint64_t)nseg - 1) / (uint64_t)nseg};
}
__device__ __forceinline__ FirItem fir_item(int item, const ItemDecode& dc, int S, int acclen, int O) {
  FirItem it;
  const uint32_t r = (uint32_t)item >> dc.pshift;
  const uint32_t q = (uint32_t)(((uint64_t)r * dc.mseg) >> 32);
  it.n = item & ((1 << dc.pshift) - 1);
  it.in = (int)q;
  it.seg = (int)(r - q * (uint32_t)dc.nseg);
  it.s0 = it.seg * S;
  it.s1 = min(it.s0 + S, acclen);
  it.first = it.seg == 0;
  it.last = it.s0 + S >= acclen;
  it.ylo = it.first ? 0 : it.s0 - 4 * O;  // first row computed here
  it.nrows = it.s1 - it.ylo;              // <= R
  return it;
}

// Shift (0..3 floats) at which the x window lands in shared memory so that
// it can be copied with 16-byte cp.async from the 16-byte boundary at or
// below col + xbase; -1 when the window wraps around the column or that
// boundary lies before the column (4-byte copies, no shift).
__device__ __forceinline__ int window_shift(const float* col, int xbase, int nx, int nslice) {
  const int xo = (int)((((uintptr_t)(col + xbase)) >> 2) & 3);
  return (xbase - xo < 0 || xbase + nx > nslice) ? -1 : xo;
}

// stage[sh + e] = column[(xbase + e) mod nslice] for e < nx, sh = max(shift, 0);
// an aligned shift also copies the shift floats before xbase into stage[0, sh).
__device__ __forceinline__ void prefetch_window(float* stage, const float* col, int xbase, int nx, int nslice,
                                                int shift, int tid) {
  if (shift >= 0) {
    const float* src = col + xbase - shift;
    const int tot = shift + nx, n4 = tot >> 2;
    for (int q = tid; q < n4; q += kFirThreads) cp_async16(stage + 4 * q, src + 4 * q);
    for (int e = 4 * n4 + tid; e < tot; e += kFirThreads) cp_async4(stage + e, src + e);
  } else {
    for (int e = tid; e < nx; e += kFirThreads) {
      int t = xbase + e;
      if (t < 0 || t >= nslice) t = ((t % nslice) + nslice) % nslice;
      cp_async4(stage + e, col + t);
    }
  }
}

// The item's other inputs, after its x window: the column's K taps or
// coefficients (TAPS floats reserved), the previous chunk's last 4*O rows
// (first segment only) and the 4*O fine-window coefficients of column n as
// a float4 per t' ([t'][i] = win[(i*O + t')*P + n]).
template <int O>
__device__ __forceinline__ void prefetch_item_extras(float* st_taps, int K, int TAPS, const float* taps,
                                                     const FirItem& it, int P, const float* win,
                                                     const float* state_in, int tid) {
  for (int k = tid; k < K; k += kFirThreads) cp_async4(st_taps + k, taps + (int64_t)it.n * K + k);
  float* st_tail = st_taps + TAPS;
  if (it.first) {
    const float* st = state_in + ((int64_t)it.in * P + it.n) * (4 * O);
    for (int q = tid; q < O; q += kFirThreads) cp_async16(st_tail + 4 * q, st + 4 * q);
  }
  float* st_win = st_tail + 4 * O;
  for (int q = tid; q < 4 * O; q += kFirThreads) {
    const int tp = q >> 2, i = q & 3;
    cp_async4(st_win + q, win + (int64_t)(i * O + tp) * P + it.n);
  }
}

// y rows are padded kYPad floats per O rows, with the pads at the fine
// blocks' first rows (y row phi + k*O): a block's 4*O rows then sit at
// base + c + kYPad*(c/O) for compile-time c.  The kernels index the y
// buffer from a base shifted by phi & 1 floats, so every block starts on an
// 8-byte boundary and the fold reads rows in pairs; blocks O + 2 floats (an
// odd number of 8-byte units) apart fall in distinct banks (one lane per
// block), and the filter's stores of lanes U rows apart meet at most 2-way
// conflicts at osamp 64 for U = 21 and 41 (a 1-float pad gives 3-way at
// U = 41, 11-way at U = 21).  Pair loads halve the fold's shared loads
// against a 3-float pad read one float at a time, with the same FMAs in the
// same order.  (Two lanes per block, each
// taking half the FFT, removed the fold's idle threads but met 2-way
// conflicts on every y load and cost more than it saved.)
template <int O>
__device__ __forceinline__ int yidx(int q, int phi) {  // q >= 0, 0 <= phi < O
  return q + kYPad * (int)((unsigned)(q - phi + O) / (unsigned)O);
}
template <int O>
__device__ __forceinline__ int y_phase(const FirItem& it, const FoldArgs& fa) {
  return (((4 * O - it.s0 + (int)fa.row0) % O) + O) % O;
}

// Fine blocks an item folds: those whose last row lies in [s0, s0 + S) (the
// last segment: >= s0), as [b0, b1).
template <int O>
__device__ __forceinline__ void fold_block_range(const FirItem& it, const FoldArgs& fa, int S, int* b0, int* b1) {
  const int row0 = (int)fa.row0, nb = (int)fa.nb;
  auto first_block_ending_at_or_after = [&](int r) -> int {  // min b with row0 + b*O + 4O - 1 >= r
    const int num = r - 4 * O + 1 - row0;
    const int b = num <= 0 ? 0 : (num + O - 1) / O;
    return min(b, nb);
  };
  *b0 = it.first ? 0 : first_block_ending_at_or_after(it.s0);
  *b1 = it.last ? nb : first_block_ending_at_or_after(it.s0 + S);
}

// Fold + real DFT of fine block b of an item from its y rows (y row q = kept
// row q - 4*O + s0), by one thread: the 4 taps fold into O samples, whose
// real DFT is a compile-time radix-2 FFT of O/2 points plus the real-input
// untangle, written as O packed floats of W with 32-byte stores.
template <int O>
__device__ __forceinline__ void fold_one_block(const float* ys, int phi, const float4* wt, const FirItem& it,
                                               const FoldArgs& fa, int P, int b) {
  constexpr int NC = O / 2, LOGNC = ilog2(NC);
  constexpr int GW = O < 8 ? O : 8;
  const int rfirst = (int)fa.row0 + b * O;
  float* wb = fa.W + (int64_t)it.in * fa.nb * ((int64_t)O * P) + (int64_t)it.n * GW + (int64_t)b * ((int64_t)O * P);
  if (rfirst >= it.s1) {  // entirely past the end of the stream
#pragma unroll
    for (int p = 0; p < O; p += GW) {
      float* dst = wb + (int64_t)(p / GW) * P * GW;
      if constexpr (GW == 8) st_global_v8(dst, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
      else *reinterpret_cast<float4*>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return;
  }
  const int q0 = 4 * O - it.s0 + rfirst;  // y row of the block's first row (= phi mod O)
  // rows q0 + c at yb[c + kYPad*(c/O)]; yb is 8-byte aligned (ys is shifted
  // by phi & 1), so the rows 2m, 2m+1 of each tap come as one float2
  const float2* yb = reinterpret_cast<const float2*>(ys + yidx<O>(q0, phi));
  float2 a[NC];
#pragma unroll
  for (int m = 0; m < NC; m++) {
    const float2 y0 = yb[m], y1 = yb[m + (O + kYPad) / 2], y2 = yb[m + (O + kYPad)],
                 y3 = yb[m + 3 * (O + kYPad) / 2];
    const float4 wa = wt[2 * m], wb4 = wt[2 * m + 1];
    a[m] = make_float2(fmaf(wa.x, y0.x, fmaf(wa.y, y1.x, fmaf(wa.z, y2.x, wa.w * y3.x))),
                       fmaf(wb4.x, y0.y, fmaf(wb4.y, y1.y, fmaf(wb4.z, y2.y, wb4.w * y3.y))));
  }
  reg_fft_dif<NC>(a);
  // untangle the real input: W_k = (Z_k + conj Z_{NC-k})/2 + w^k (Z_k - conj Z_{NC-k})/(2i);
  // packed floats p = 2k, 2k+1 ((W_0, W_{O/2}) at p = 0, 1), one group of
  // GW floats per store (a whole 32-byte sector when GW = 8)
#pragma unroll
  for (int p = 0; p < O; p += GW) {
    float2 o[GW / 2];
#pragma unroll
    for (int h = 0; h < GW / 2; h++) {
      const int k = p / 2 + h;
      if (k == 0) {
        o[h] = make_float2(a[0].x + a[0].y, a[0].x - a[0].y);
      } else {
        const float2 z = a[bitrev(k, LOGNC)], c = cconj(a[bitrev(NC - k, LOGNC)]);
        const float2 E = cscale(cadd(z, c), 0.5f);
        const float2 Dd = csub(z, c);
        const float2 Od = make_float2(0.5f * Dd.y, -0.5f * Dd.x);
        o[h] = cadd(E, cmul(c_fir_tw[k * (64 / O)], Od));
      }
    }
    float* dst = wb + (int64_t)(p / GW) * P * GW;
    if constexpr (GW == 8) st_global_v8(dst, o[0].x, o[0].y, o[1].x, o[1].y, o[2].x, o[2].y, o[3].x, o[3].y);
    else *reinterpret_cast<float4*>(dst) = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
  }
}

// The last segment keeps the chunk's last 4*O rows as the next chunk's tail.
template <int O>
__device__ __forceinline__ void fold_tail_state(const float* ys, int phi, const FirItem& it, int P, int acclen,
                                                float* __restrict__ state_out, int tid) {
  float* st = state_out + ((int64_t)it.in * P + it.n) * (4 * O);
  for (int i = tid; i < 4 * O; i += kFirThreads) st[i] = ys[yidx<O>(4 * O - it.s0 + (acclen - 4 * O + i), phi)];
}

// All of an item's fine blocks, one per thread, then its tail state.
template <int O>
__device__ __forceinline__ void fold_item_blocks(const float* ys, int phi, const float4* wt, const FirItem& it,
                                                 const FoldArgs& fa, int P, int S, int acclen,
                                                 float* __restrict__ state_out, int tid) {
  int b0, b1;
  fold_block_range<O>(it, fa, S, &b0, &b1);
  for (int b = b0 + tid; b < b1; b += kFirThreads) fold_one_block<O>(ys, phi, wt, it, fa, P, b);
  if (it.last) fold_tail_state<O>(ys, phi, it, P, acclen, state_out, tid);
}

// y rows that do not come from the filter: the previous chunk's tail (first
// segment, y rows [0, 4*O)) and zeros past the end of the stream (last
// segment; zero-padded final blocks).
template <int O>
__device__ __forceinline__ void y_edges(float* ys, int phi, const float* tail, const FirItem& it, int yoff, int tid) {
  if (it.first)
    for (int i = tid; i < 4 * O; i += kFirThreads) ys[yidx<O>(i, phi)] = tail[i];
  if (it.last)
    for (int q = yoff + it.nrows + tid; q < yoff + it.nrows + 4 * O; q += kFirThreads) ys[yidx<O>(q, phi)] = 0.f;
}

// ---------------------------------------------------------------------------
// FIR time stage + fold.
template <int J, int U, int G>
__global__ void __launch_bounds__(kFirThreads, J <= 32 ? 2 : 1)
    fir_fold_kernel(const float* __restrict__ data, int64_t ld, int P, int nslice, int cut, int acclen, int S,
                    int nseg, int nitems, const float* __restrict__ taps, FoldArgs fa,
                    const float* __restrict__ state_in, float* __restrict__ state_out) {
  constexpr int O = 2 * G;
  using Lay = FirLayout<J, U, O>;
  constexpr int K = Lay::K;
  extern __shared__ float4 smem4[];
  float* stage0 = reinterpret_cast<float*>(smem4);
  float* ys = stage0 + 2 * Lay::STAGE;
  const int tid = threadIdx.x;
  const ItemDecode dc = item_decode(nseg, P);

  auto prefetch = [&](int item, float* stage) {
    const FirItem it = fir_item(item, dc, S, acclen, O);
    const float* col = data + ((int64_t)it.in * P + it.n) * ld;
    // x window: stage[e] = x[(cut + ylo - J + e) mod nslice], e < nrows + 2J
    const int xbase = cut + it.ylo - J, nx = it.nrows + 2 * J;
    prefetch_window(stage, col, xbase, nx, nslice, window_shift(col, xbase, nx, nslice) == 0 ? 0 : -1, tid);
    for (int e = nx + tid; e < nx + U; e += kFirThreads) stage[e] = 0.f;
    prefetch_item_extras<O>(stage + Lay::XS, K, Lay::TAPS, taps, it, P, fa.win, state_in, tid);
    cp_async_commit();
  };

  // Unlike the IIR form, the next item's prefetch goes out before the wait for
  // this item's inputs, which costs a barrier at the end of each item: with
  // the FIR form's shorter items the earlier prefetch measured faster.
  int item = blockIdx.x, buf = 0;
  if (item < nitems) prefetch(item, stage0);
  for (; item < nitems; item += gridDim.x, buf ^= 1) {
    float* stage = stage0 + buf * Lay::STAGE;
    const int next = item + gridDim.x;
    if (next < nitems) {
      prefetch(next, stage0 + (buf ^ 1) * Lay::STAGE);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const FirItem it = fir_item(item, dc, S, acclen, O);
    const int yoff = it.ylo - it.s0 + 4 * O;  // y row of computed row ylo
    const int phi = y_phase<O>(it, fa);
    float* ysb = ys + (phi & 1);  // blocks start on 8-byte boundaries (yidx)
    y_edges<O>(ysb, phi, stage + Lay::XS + Lay::TAPS, it, yoff, tid);
    // y[ylo + i] = sum_j h[j + J] x[cut + ylo + i - j] = sum_k h[k] xs[i + 2J - k]
    if (tid * U < it.nrows) {
      float h[K];
#pragma unroll
      for (int k = 0; k < K; k++) h[k] = stage[Lay::XS + k];
      float acc[U];
#pragma unroll
      for (int g = 0; g < U; g++) acc[g] = 0.f;
      const float* xu = stage + tid * U;
#pragma unroll
      for (int ep = 0; ep < U + 2 * J; ep++) {
        const float v = xu[ep];
#pragma unroll
        for (int g = 0; g < U; g++) {
          const int k = g + 2 * J - ep;
          if (k >= 0 && k < K) acc[g] = fmaf(h[k], v, acc[g]);
        }
      }
      const int t0 = yoff + tid * U;
      const int nv = it.nrows - tid * U;
#pragma unroll
      for (int g = 0; g < U; g++) ysb[g < nv ? yidx<O>(t0 + g, phi) : Lay::YS - 2] = acc[g];  // spare slot past nrows
    }
    __syncthreads();
    fold_item_blocks<O>(ysb, phi, reinterpret_cast<const float4*>(stage + Lay::XS + Lay::TAPS + Lay::ST), it, fa, P,
                        S, acclen, state_out, tid);
    __syncthreads();  // ys and this staging buffer are reused next
  }
}

// ---------------------------------------------------------------------------
// IIR time stage + fold.  Per item each thread
//  1. runs u = W x and the causal recursion v = u / A over its U rows from
//     zero state, keeping u and the end state zf (v at its last 3 rows);
//  2. takes the true state at its start, T(k-1) = zf(k-1) + Phi T(k-2),
//     as the D-term sum zf(k-1) + Phi zf(k-2) + ... + Phi^(D-1) zf(k-D)
//     (Phi: U rows of the homogeneous recursion; the dropped Phi^D term is
//     1/A's impulse response after D*U >= IW rows, below 1e-10 of its peak),
//     and re-runs v from it;
//  3. the same for the anti-causal recursion y = v / A(1/z) from its top row
//     (zero-state pass, states exchanged with the D threads above), writing
//     the computed rows of y.
// 16 FMAs per row against 7 (U + 2 IW) / U + 3 (U + IW) / U for per-thread
// warm-ups of IW rows.

struct Iir3 {
  float p1, p2, p3;  // outputs at the nearest, second and third rows
};

// State after U more rows of the homogeneous recursion from s: the start
// acts as the input u'_0 = -(a1 p1 + a2 p2 + a3 p3), u'_1 = -(a2 p1 + a3 p2),
// u'_2 = -a3 p1 to the zero-state recursion, whose outputs at rows U-1, U-2,
// U-3 are those inputs convolved with 1/A's impulse response, hh[i] = h[U-5+i].
__device__ __forceinline__ Iir3 iir_advance(Iir3 s, float a1, float a2, float a3, const float* hh) {
  const float u0 = -fmaf(a1, s.p1, fmaf(a2, s.p2, a3 * s.p3));
  const float u1 = -fmaf(a2, s.p1, a3 * s.p2);
  const float u2 = -a3 * s.p1;
  Iir3 r;
  r.p1 = fmaf(hh[4], u0, fmaf(hh[3], u1, hh[2] * u2));
  r.p2 = fmaf(hh[3], u0, fmaf(hh[2], u1, hh[1] * u2));
  r.p3 = fmaf(hh[2], u0, fmaf(hh[1], u1, hh[0] * u2));
  return r;
}

// sum over d = 1..D of Phi^(d-1) z(k + dir*d), terms outside [0, nthr) omitted
template <int D>
__device__ __forceinline__ Iir3 iir_incoming(const float* z, int k, int dir, int nthr, float a1, float a2, float a3,
                                             const float* hh) {
  Iir3 s = {0.f, 0.f, 0.f};
#pragma unroll
  for (int d = D; d >= 1; d--) {
    if (d < D) s = iir_advance(s, a1, a2, a3, hh);
    const int j = k + dir * d;
    if (j >= 0 && j < nthr) {
      s.p1 += z[j];
      s.p2 += z[kFirThreads + j];
      s.p3 += z[2 * kFirThreads + j];
    }
  }
  return s;
}

// CTAs per SM: two for the 21- and 41-row tiles, one for the 67-row tile
// (its two staging buffers take 150-210 KB of shared memory).
__host__ __device__ constexpr int iir_ctas_per_sm(int U) { return U > kIirU32 ? 1 : 2; }

template <int U, int G, int D>
__global__ void __launch_bounds__(kFirThreads, iir_ctas_per_sm(U))
    iir_fold_kernel(const float* __restrict__ data, int64_t ld, int P, int nslice, int cut, int acclen, int S,
                    int nseg, int nitems, const float* __restrict__ coef, FoldArgs fa,
                    const float* __restrict__ state_in, float* __restrict__ state_out) {
  constexpr int O = 2 * G;
  using Lay = IirLayout<U, O, D>;
  static_assert(U >= 5, "the state advance needs U >= 5");
  extern __shared__ float4 smem4[];
  float* stage0 = reinterpret_cast<float*>(smem4);
  float* zf = stage0 + 2 * Lay::STAGE;  // [3][kFirThreads] forward end states
  float* zb = zf + 3 * kFirThreads;     // [3][kFirThreads] backward end states
  const int tid = threadIdx.x;
  const ItemDecode dc = item_decode(nseg, P);
  // threads that run: up to D past the one holding the last computed row
  auto threads_of = [](const FirItem& it) { return min(kFirThreads, (D * U + it.nrows - 1) / U + D + 1); };

  auto prefetch = [&](int item, float* stage) {
    const FirItem it = fir_item(item, dc, S, acclen, O);
    const float* col = data + ((int64_t)it.in * P + it.n) * ld;
    const int xbase = cut + it.ylo - D * U - 3, nx = threads_of(it) * U + 3;
    prefetch_window(stage, col, xbase, nx, nslice, window_shift(col, xbase, nx, nslice), tid);
    prefetch_item_extras<O>(stage + Lay::XS, kIirCoef, Lay::TAPS, coef, it, P, fa.win, state_in, tid);
    cp_async_commit();
  };

  // The next item's inputs are fetched into the other staging buffer right
  // after this item's opening barrier: every thread has then finished the
  // previous item, whose buffer that is, so no barrier is needed at the end
  // of an item.
  int item = blockIdx.x, buf = 0;
  if (item < nitems) prefetch(item, stage0);
  for (; item < nitems; item += gridDim.x, buf ^= 1) {
    float* stage = stage0 + buf * Lay::STAGE;
    const int next = item + gridDim.x;
    cp_async_wait<0>();  // this item's inputs: the only copies in flight
    __syncthreads();
    if (next < nitems) prefetch(next, stage0 + (buf ^ 1) * Lay::STAGE);
    const FirItem it = fir_item(item, dc, S, acclen, O);
    const int nthr = threads_of(it);
    const float* cf = stage + Lay::XS;
    const float w0 = cf[0], w1 = cf[1], w2 = cf[2], w3 = cf[3];
    const float a1 = cf[4], a2 = cf[5], a3 = cf[6];
    const float* hh = cf + iir_hh_offset(U);
    float u[U];
    Iir3 s = {0.f, 0.f, 0.f};
    if (tid < nthr) {
      const float* col = data + ((int64_t)it.in * P + it.n) * ld;
      const int xbase = cut + it.ylo - D * U - 3;
      const int sh = max(window_shift(col, xbase, nthr * U + 3, nslice), 0);
      const float* xk = stage + sh + tid * U;  // x of window row tid*U + m at xk[m + 3]
      float x0 = xk[0], x1 = xk[1], x2 = xk[2];
#pragma unroll
      for (int m = 0; m < U; m++) {
        const float x3 = xk[m + 3];
        const float ut = fmaf(w0, x3, fmaf(w1, x2, fmaf(w2, x1, w3 * x0)));
        x0 = x1;
        x1 = x2;
        x2 = x3;
        const float vt = fmaf(-a1, s.p1, fmaf(-a2, s.p2, fmaf(-a3, s.p3, ut)));
        s.p3 = s.p2;
        s.p2 = s.p1;
        s.p1 = vt;
        u[m] = ut;
      }
    }
    zf[tid] = s.p1;
    zf[kFirThreads + tid] = s.p2;
    zf[2 * kFirThreads + tid] = s.p3;
    __syncthreads();
    // the x window is dead: y rows go over it
    const int yoff = it.ylo - it.s0 + 4 * O;  // y row of computed row ylo
    const int phi = y_phase<O>(it, fa);
    float* ys = stage + (phi & 1);  // blocks start on 8-byte boundaries (yidx)
    y_edges<O>(ys, phi, stage + Lay::XS + Lay::TAPS, it, yoff, tid);
    Iir3 q = {0.f, 0.f, 0.f};
    if (tid < nthr) {
      s = iir_incoming<D>(zf, tid, -1, nthr, a1, a2, a3, hh);
#pragma unroll
      for (int m = 0; m < U; m++) {
        const float vt = fmaf(-a1, s.p1, fmaf(-a2, s.p2, fmaf(-a3, s.p3, u[m])));
        s.p3 = s.p2;
        s.p2 = s.p1;
        s.p1 = vt;
        u[m] = vt;
      }
#pragma unroll
      for (int m = U - 1; m >= 0; m--) {
        const float yt = fmaf(-a1, q.p1, fmaf(-a2, q.p2, fmaf(-a3, q.p3, u[m])));
        q.p3 = q.p2;
        q.p2 = q.p1;
        q.p1 = yt;
      }
    }
    zb[tid] = q.p1;
    zb[kFirThreads + tid] = q.p2;
    zb[2 * kFirThreads + tid] = q.p3;
    __syncthreads();
    if (tid >= D && tid < nthr) {
      q = iir_incoming<D>(zb, tid, 1, nthr, a1, a2, a3, hh);
      const int r0 = (tid - D) * U;  // computed row of this thread's first row
#pragma unroll
      for (int m = U - 1; m >= 0; m--) {
        const float yt = fmaf(-a1, q.p1, fmaf(-a2, q.p2, fmaf(-a3, q.p3, u[m])));
        q.p3 = q.p2;
        q.p2 = q.p1;
        q.p1 = yt;
        if (r0 + m < it.nrows) ys[yidx<O>(yoff + r0 + m, phi)] = yt;
      }
    }
    __syncthreads();
    fold_item_blocks<O>(ys, phi, reinterpret_cast<const float4*>(stage + Lay::XS + Lay::TAPS + 4 * O), it, fa, P, S,
                        acclen, state_out, tid);
  }
}

template <int S_, int O>
static int64_t fir_items(const FirArgs& a, int* nseg) {
  *nseg = std::max(1, (a.acclen + S_ - 1) / S_);
  return (int64_t)*nseg * a.P * a.ninputs;
}

template <int J, int U, int G>
static int launch_fir_t(const FirArgs& a, const FoldArgs& fa, cudaStream_t s) {
  constexpr int O = 2 * G;
  using Lay = FirLayout<J, U, O>;
  constexpr int S = Lay::R - 4 * O;
  int nseg;
  const int64_t nitems = fir_items<S, O>(a, &nseg);
  AB_CHECK_ARG(nitems < (1LL << 31), "FIR time stage: too many work items");
  const size_t smem = Lay::bytes();
  AB_CUDA(cudaFuncSetAttribute(fir_fold_kernel<J, U, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int per_sm = J <= 32 ? 2 : 1;
  const int64_t grid = std::min<int64_t>(nitems, (int64_t)per_sm * std::max(a.num_sms, 1));
  fir_fold_kernel<J, U, G><<<(unsigned)grid, kFirThreads, smem, s>>>(a.data, a.ld, a.P, a.nslice, a.cut, a.acclen, S,
                                                                     nseg, (int)nitems, a.taps, fa, a.state_in,
                                                                     a.state_out);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

template <int U, int G, int D>
static int launch_iir_t(const FirArgs& a, const FoldArgs& fa, cudaStream_t s) {
  constexpr int O = 2 * G;
  using Lay = IirLayout<U, O, D>;
  // new rows per item: a whole number of fold rounds (one block per thread
  // per round) when at least one fits
  constexpr int SMAX = Lay::R - 4 * O, ROUND = kFirThreads * O;
  constexpr int S = SMAX >= ROUND ? SMAX / ROUND * ROUND : SMAX;
  static_assert(S > 0, "IIR tile too small for this osamp");
  int nseg;
  const int64_t nitems = fir_items<S, O>(a, &nseg);
  AB_CHECK_ARG(nitems < (1LL << 31), "IIR time stage: too many work items");
  const size_t smem = Lay::bytes();
  AB_CUDA(cudaFuncSetAttribute(iir_fold_kernel<U, G, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = std::min<int64_t>(nitems, iir_ctas_per_sm(U) * (int64_t)std::max(a.num_sms, 1));
  iir_fold_kernel<U, G, D><<<(unsigned)grid, kFirThreads, smem, s>>>(a.data, a.ld, a.P, a.nslice, a.cut, a.acclen, S,
                                                                     nseg, (int)nitems, a.taps, fa, a.state_in,
                                                                     a.state_out);
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

template <int U, int D>
static int launch_iir_o(const FirArgs& a, const FoldArgs& fa, cudaStream_t s) {
  switch (fa.O) {
    case 4: return launch_iir_t<U, 2, D>(a, fa, s);
    case 8: return launch_iir_t<U, 4, D>(a, fa, s);
    case 16: return launch_iir_t<U, 8, D>(a, fa, s);
    case 32: return launch_iir_t<U, 16, D>(a, fa, s);
    case 64: return launch_iir_t<U, 32, D>(a, fa, s);
    default:
      set_error("IIR time stage: osamp %d not supported (4..64)", fa.O);
      return AB_ERR_UNSUPPORTED;
  }
}

int launch_fir_fold(const FirArgs& a, const FoldArgs& fa, cudaStream_t s) {
  AB_CHECK_ARG(fa.ntap == 4, "FIR time stage: needs ntap = 4");
  AB_CHECK_ARG(a.P <= 65535 && a.ninputs <= 65535, "FIR time stage: grid too large");
  AB_CHECK_ARG(a.P > 0 && (a.P & (a.P - 1)) == 0, "FIR time stage: P = %d must be a power of two", a.P);
  AB_CHECK_ARG(a.row_tile == 16 || a.row_tile == 32 || a.row_tile == 64,
               "FIR time stage: row tile must be 16, 32 or 64");
  AB_CHECK_ARG(a.num_sms > 0, "FIR time stage: SM count unknown");
  AB_CHECK_ARG(a.row_tile * kFirThreads > 4 * fa.O, "FIR time stage: row tile too small for osamp %d", fa.O);
  AB_CHECK_ARG(((uintptr_t)fa.W & 31) == 0 && (a.P % 4) == 0, "FIR time stage: W must be 32-byte aligned");
  // odd rows per thread keep the shared loads of lanes U rows apart
  // conflict-free without padding.  IIR: D = ceil(IW / U) exchanged states.
  if (a.iir_w > 0) {
    const int U = a.row_tile == 64 ? kIirU64 : a.row_tile == 32 ? kIirU32 : kIirU16;
    const int D = (a.iir_w + U - 1) / U;
    if (U == kIirU64 && D == 1) return launch_iir_o<kIirU64, 1>(a, fa, s);
    if (U == kIirU64 && D == 2) return launch_iir_o<kIirU64, 2>(a, fa, s);
    if (U == kIirU32 && D == 1) return launch_iir_o<kIirU32, 1>(a, fa, s);
    if (U == kIirU32 && D == 2) return launch_iir_o<kIirU32, 2>(a, fa, s);
    if (U == kIirU16 && D == 2) return launch_iir_o<kIirU16, 2>(a, fa, s);
    if (U == kIirU16 && D == 4) return launch_iir_o<kIirU16, 4>(a, fa, s);
  } else {
    // the FIR form has two row tiles; 64 takes the larger
    if (a.J == 32) return a.row_tile >= 32 ? launch_fir_o<32, 33>(a, fa, s) : launch_fir_o<32, 17>(a, fa, s);
    if (a.J == 64) return a.row_tile >= 32 ? launch_fir_o<64, 33>(a, fa, s) : launch_fir_o<64, 17>(a, fa, s);
  }
  set_error("FIR time stage: J = %d / IW = %d not supported", a.J, a.iir_w);
  return AB_ERR_UNSUPPORTED;
}

}  // namespace ab
