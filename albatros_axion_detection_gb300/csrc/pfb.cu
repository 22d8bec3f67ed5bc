// pfb.cu -- forward PFB (cupy_pfb, albatros_analysis/src/utils/pfb_gpu_utils.py:105-121):
//   y[b, k] = sum_{i<ntap} ts[(b+i) L + k] win[i L + k];  out[b] = rfft(y[b])
// computed as stage A (tap fold + O-point real DFT over t', k = n + P t')
// and stage B (twiddle + P-point DFT over n), see pfb.cuh.
#include <algorithm>
#include <type_traits>

#include "async.cuh"
#include "fft_static.cuh"
#include "pfb.cuh"

namespace ab {

constexpr int kFoldCols = 32;   // sample phases per CTA (one warp lane each)
constexpr int kFoldBlocks = 16; // output blocks per CTA (one warp each)

// shared memory of a stage-A CTA: data tile [kFoldCols][pitch] + window [ntap*O][kFoldCols]
__host__ __device__ inline size_t stage_a_smem(int O, int ntap) {
  return sizeof(float) * ((size_t)kFoldCols * ((kFoldBlocks + ntap - 1) * O + 1) + (size_t)ntap * O * kFoldCols);
}

template <int O>
__global__ void __launch_bounds__(kFoldCols* kFoldBlocks)
    pfb_stage_a_kernel(TsSrc src, int P, int ntap, int64_t row0, int64_t nb, const float* __restrict__ win,
                       float* __restrict__ W, const float2* __restrict__ tw64, int vec4) {
  extern __shared__ float tile[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n0 = blockIdx.y * kFoldCols;
  const int64_t b0 = (int64_t)blockIdx.x * kFoldBlocks;
  const int in = blockIdx.z;
  const int RW = (kFoldBlocks + ntap - 1) * O;  // rows in the tile
  const int pitch = RW + 1;                     // odd pitch: conflict-free columns
  float* wsm = tile + (size_t)kFoldCols * pitch;  // window [ntap*O][kFoldCols]
  const int64_t rbase = row0 + b0 * O;          // first tile row (timestream row)
  // ---- window slice of these sample phases
  for (int k = warp; k < ntap * O; k += kFoldBlocks) wsm[k * kFoldCols + lane] = __ldg(&win[(int64_t)k * P + n0 + lane]);
  // ---- load tile[n][r] = ts(rbase + r, n0 + n) ----
  if (src.natural) {
    for (int r = warp; r < RW; r += kFoldBlocks) {
      int64_t rr = rbase + r;
      float v = 0.f;
      if (rr >= 0 && rr < src.nrows_valid) v = __ldg(&src.cur[rr * P + n0 + lane]);
      tile[lane * pitch + r] = v;
    }
  } else if (vec4) {
    // column layout, 16-byte aligned rows: float4 loads along t
    const int RW4 = RW / 4;
    for (int c = warp; c < kFoldCols; c += kFoldBlocks) {
      const int64_t colbase = ((int64_t)in * P + n0 + c) * src.ld;
      for (int q = lane; q < RW4; q += 32) {
        int64_t rr = rbase + 4 * q;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (rr + 3 < src.nrows_valid && rr >= 0) {
          v = __ldg(reinterpret_cast<const float4*>(src.cur + colbase + src.off + rr));
        } else if (rr + 3 < 0) {
          if (src.prev) v = __ldg(reinterpret_cast<const float4*>(src.prev + colbase + src.prev_off + rr));
        } else {
          float e[4];
          for (int u = 0; u < 4; u++) {
            int64_t r1 = rr + u;
            e[u] = 0.f;
            if (r1 < src.nrows_valid) {
              if (r1 >= 0) e[u] = src.cur[colbase + src.off + r1];
              else if (src.prev) e[u] = src.prev[colbase + src.prev_off + r1];
            }
          }
          v = make_float4(e[0], e[1], e[2], e[3]);
        }
        float* d = tile + c * pitch + 4 * q;
        d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
      }
    }
  } else {
    for (int c = warp; c < kFoldCols; c += kFoldBlocks) {
      const int64_t colbase = ((int64_t)in * P + n0 + c) * src.ld;
      for (int r = lane; r < RW; r += 32) {
        int64_t rr = rbase + r;
        float v = 0.f;
        if (rr < src.nrows_valid) {
          if (rr >= 0) v = __ldg(&src.cur[colbase + src.off + rr]);
          else if (src.prev) v = __ldg(&src.prev[colbase + src.prev_off + rr]);
        }
        tile[c * pitch + r] = v;
      }
    }
  }
  __syncthreads();
  const int64_t b = b0 + warp;
  if (b >= nb) return;
  const int n = n0 + lane;
  const float* col = tile + lane * pitch + warp * O;
  // tap fold: y[t'] = sum_i ts((b+i) O + t') win[(i O + t') P + n]
  constexpr int H = O > 1 ? O / 2 : 1;
  float2 z[H];
#pragma unroll
  for (int m = 0; m < H; m++) z[m] = make_float2(0.f, 0.f);
  for (int i = 0; i < ntap; i++) {
    const float* wrow = wsm + i * O * kFoldCols + lane;
#pragma unroll
    for (int tp = 0; tp < O; tp++) {
      float v = col[i * O + tp] * wrow[tp * kFoldCols];
      if (O == 1) z[0].x += v;
      else if (tp & 1) z[tp >> 1].y += v;
      else z[tp >> 1].x += v;
    }
  }
  const int GW = O < 8 ? O : 8;
  const int NG = O / GW;
  float* Wb = W + (((int64_t)in * nb + b) * NG * P) * GW;
  if constexpr (O == 1) {
    Wb[n] = z[0].x;
  } else {
    reg_fft_pow2<H>(z, tw64);
    float out[O];
    out[0] = z[0].x + z[0].y;  // W_0
    out[1] = z[0].x - z[0].y;  // W_{O/2}
#pragma unroll
    for (int k = 1; k < H; k++) {
      float2 zk = z[k], zc = cconj(z[H - k]);
      float2 E = cscale(cadd(zk, zc), 0.5f);
      float2 Dd = csub(zk, zc);                            // 2 i O_k
      float2 Od = make_float2(0.5f * Dd.y, -0.5f * Dd.x);  // O_k
      float2 w = tw64[k * (64 / O)];                       // exp(-2 pi i k / O)
      float2 Wk = cadd(E, cmul(w, Od));
      out[2 * k] = Wk.x;
      out[2 * k + 1] = Wk.y;
    }
#pragma unroll
    for (int g = 0; g < NG; g++) {
      float* dst = Wb + ((int64_t)g * P + n) * GW;
      if constexpr (O >= 4) {
#pragma unroll
        for (int e = 0; e < GW; e += 4)
          *reinterpret_cast<float4*>(dst + e) =
              make_float4(out[g * GW + e], out[g * GW + e + 1], out[g * GW + e + 2], out[g * GW + e + 3]);
      } else {
#pragma unroll
        for (int e = 0; e < GW; e++) dst[e] = out[g * GW + e];
      }
    }
  }
}

// Stage B: one CTA per (group g, block b, input).  Loads the group's P x GW
// floats, then for each fine offset s carried by the group forms
// V_s[n] = W_s[n] exp(-2 pi i s n / L) and its P-point DFT.
constexpr int kStageBThreads = 512;
struct NoPlanB {};

template <class PL>
__global__ void __launch_bounds__(kStageBThreads)
    pfb_stage_b_kernel(const float* __restrict__ W, int P, int O, int64_t nb, FftPlan plan,
                       const float2* __restrict__ twL, const float2* __restrict__ tws, int u0, int u1,
                       float2* __restrict__ out) {
  constexpr bool kStatic = !std::is_same<PL, NoPlanB>::value;
  extern __shared__ float4 smem4[];
  const int GW = O < 8 ? O : 8, NG = O / GW;
  const int g = blockIdx.y;
  const int64_t b = blockIdx.x;
  const int in = blockIdx.z;
  const int64_t L = (int64_t)P * O;
  float* wt = reinterpret_cast<float*>(smem4);                   // P * GW floats
  float2* buf = reinterpret_cast<float2*>(wt + (size_t)P * GW);  // padded P complex
  const SmemTw tw = load_smem_tw(buf + padded_len(P), twL, (int)L, threadIdx.x, blockDim.x);
  const float* src = W + ((((int64_t)in * nb + b) * NG + g) * P) * GW;
  if (GW >= 4) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
    for (int i = threadIdx.x; i < P * GW / 4; i += blockDim.x) smem4[i] = __ldg(&s4[i]);
  } else {
    for (int i = threadIdx.x; i < P * GW; i += blockDim.x) wt[i] = __ldg(&src[i]);
  }
  __syncthreads();
  const bool full = u1 < 0;
  const int64_t nq = full ? L / 2 + 1 : (int64_t)(u1 - u0) * O;
  float2* ob = out + ((int64_t)in * nb + b) * nq;
  // slots of this group: pairs of floats (e, e+1), e even
  for (int e = 0; e < GW; e += (GW == 1 ? 1 : 2)) {
    const int c = (g * GW + e) / 2;  // complex slot index (0 holds W_0 / W_{O/2})
    const int nv = (GW == 1) ? 1 : 2;
    for (int v = 0; v < nv; v++) {
      int s;
      if (c == 0) s = (v == 0) ? 0 : O / 2;
      else s = (v == 0) ? c : O - c;
      // build V
      for (int n = threadIdx.x; n < P; n += blockDim.x) {
        float2 x;
        if (GW == 1) x = make_float2(wt[n], 0.f);
        else if (c == 0) x = make_float2(wt[n * GW + e + v], 0.f);
        else {
          x = make_float2(wt[n * GW + e], wt[n * GW + e + 1]);
          if (v) x.y = -x.y;
        }
        if (s) x = cmul(x, tw(s * n));
        buf[pidx(n)] = x;
      }
      __syncthreads();
      if constexpr (kStatic) sdif<PL, kStageBThreads>(buf, tws, threadIdx.x);
      else dif_forward(buf, plan, tw, (int)L, threadIdx.x, blockDim.x);
      auto pos = [&](int u) -> int {
        if constexpr (kStatic) return spos<PL>(u);
        else return fft_pos(plan, u);
      };
      // extract
      if (full) {
        int umax = (s == 0) ? P / 2 : P / 2 - 1;
        for (int u = threadIdx.x; u <= umax; u += blockDim.x) ob[(int64_t)u * O + s] = buf[pidx(pos(u))];
      } else {
        for (int u = u0 + threadIdx.x; u < u1; u += blockDim.x)
          ob[(int64_t)(u - u0) * O + s] = buf[pidx(pos(u))];
      }
      __syncthreads();
    }
  }
}

// Stage B specialised for P = 4096 and osamp >= 8 (8 floats per group): the
// group's W tile is stored transposed ([float][n]) so the V build reads
// consecutive n, and the CTA's two halves (256 threads each) transform two
// fine offsets at once: s = c and s = O - c of the same complex slot c.
constexpr int kB2Threads = 512;
__host__ __device__ inline size_t stage_b2_smem() {
  return sizeof(float) * 8 * 4096 + sizeof(float2) * (2 * (size_t)padded_len(4096) + 1024);
}

__global__ void __launch_bounds__(kB2Threads)
    pfb_stage_b4096_kernel(const float* __restrict__ W, int O, int64_t nb, const float2* __restrict__ twL,
                           const float2* __restrict__ tws, int u0, int u1, float2* __restrict__ out) {
  constexpr int P = 4096, GW = 8, PLN = padded_len(4096);
  extern __shared__ float4 smem4[];
  const int NG = O / GW;
  const int g = blockIdx.y;
  const int64_t b = blockIdx.x;
  const int in = blockIdx.z;
  const int L = P * O;
  const int tid = threadIdx.x, half = tid >> 8, ltid = tid & 255;
  float* wt = reinterpret_cast<float*>(smem4);                  // [8][4096]
  float2* bufs = reinterpret_cast<float2*>(wt + 8 * P);          // 2 padded buffers
  float2* vtw = bufs + 2 * PLN;                                  // hi[512], lo[512]: exp(-2 pi i e / L)
  const int nhi = (L + 511) / 512;
  for (int i = tid; i < nhi; i += kB2Threads) vtw[i] = __ldg(&twL[(int64_t)i * 512]);
  for (int i = tid; i < 512; i += kB2Threads) vtw[512 + i] = i < L ? __ldg(&twL[i]) : make_float2(1.f, 0.f);
  const float4* s4 = reinterpret_cast<const float4*>(W + ((((int64_t)in * nb + b) * NG + g) * P) * GW);
  for (int i = tid; i < P * GW / 4; i += kB2Threads) {
    float4 v = __ldg(&s4[i]);
    int n = i >> 1, e0 = (i & 1) * 4;
    wt[(e0 + 0) * P + n] = v.x;
    wt[(e0 + 1) * P + n] = v.y;
    wt[(e0 + 2) * P + n] = v.z;
    wt[(e0 + 3) * P + n] = v.w;
  }
  __syncthreads();
  const bool full = u1 < 0;
  const int64_t nq = full ? L / 2 + 1 : (int64_t)(u1 - u0) * O;
  float2* ob = out + ((int64_t)in * nb + b) * nq;
  float2* buf = bufs + half * PLN;
  for (int e = 0; e < GW; e += 2) {
    const int c = (g * GW + e) / 2;
    int s;
    if (c == 0) s = half == 0 ? 0 : O / 2;
    else s = half == 0 ? c : O - c;
    const float* wr = wt + e * P;
    const float* wi = wt + (e + 1) * P;
    for (int n = ltid; n < P; n += 256) {
      float2 x;
      if (c == 0) x = make_float2(half == 0 ? wr[n] : wi[n], 0.f);
      else x = make_float2(wr[n], half == 0 ? wi[n] : -wi[n]);
      if (s) {
        int ex = s * n;
        x = cmul(x, cmul(vtw[ex >> 9], vtw[512 + (ex & 511)]));
      }
      buf[pidx(n)] = x;
    }
    __syncthreads();
    sdif<Plan4096, 256>(buf, tws, ltid);
    if (full) {
      int umax = (s == 0) ? P / 2 : P / 2 - 1;
      for (int u = ltid; u <= umax; u += 256) ob[(int64_t)u * O + s] = buf[pidx(spos<Plan4096>(u))];
    } else {
      for (int u = u0 + ltid; u < u1; u += 256) ob[(int64_t)(u - u0) * O + s] = buf[pidx(spos<Plan4096>(u))];
    }
    __syncthreads();
  }
}

// Stage B, one CTA per (complex slot c, block, input) for P = 4096: the two
// fine offsets carried by slot c (s = c and O - c; for c = 0 the real W_0 and
// W_{O/2}) are transformed at once by the CTA's two 256-thread halves.  Each
// thread keeps W_c of 8 sample phases in registers while building V, so the
// CTA needs only the two FFT buffers in shared memory (two CTAs per SM).
constexpr int kBSThreads = 512;
__host__ __device__ inline size_t stage_bslot_smem() {
  return sizeof(float2) * (2 * (size_t)padded_len(4096) + 1024);
}

__global__ void __launch_bounds__(kBSThreads, 2)
    pfb_stage_bslot_kernel(const float* __restrict__ W, int O, int64_t nb, const float2* __restrict__ twL,
                           const float2* __restrict__ tws, int u0, int u1, float2* __restrict__ out) {
  constexpr int P = 4096, PLN = padded_len(4096), PER = P / kBSThreads;
  extern __shared__ float2 sm2[];
  const int GW = O < 8 ? O : 8, NG = O / GW;
  const int c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const int in = blockIdx.z;
  const int L = P * O;
  const int tid = threadIdx.x, half = tid >> 8, ltid = tid & 255;
  float2* bufs = sm2;
  float2* vtw = bufs + 2 * PLN;  // hi[512], lo[512]: exp(-2 pi i e / L)
  const int nhi = (L + 511) / 512;
  for (int i = tid; i < nhi; i += kBSThreads) vtw[i] = __ldg(&twL[(int64_t)i * 512]);
  for (int i = tid; i < 512; i += kBSThreads) vtw[512 + i] = i < L ? __ldg(&twL[i]) : make_float2(1.f, 0.f);
  // W_c of sample phases n = tid + 512 q
  const int g = (2 * c) / GW, e = (2 * c) % GW;
  const float* src = W + ((((int64_t)in * nb + b) * NG + g) * P) * GW + e;
  float2 wv[PER];
#pragma unroll
  for (int q = 0; q < PER; q++) wv[q] = __ldg(reinterpret_cast<const float2*>(src + (size_t)(tid + q * kBSThreads) * GW));
  const int s0 = c, s1 = (c == 0) ? O / 2 : O - c;
  __syncthreads();
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int s = h ? s1 : s0;
    float2* buf = bufs + h * PLN;
#pragma unroll
    for (int q = 0; q < PER; q++) {
      const int n = tid + q * kBSThreads;
      float2 x;
      if (c == 0) x = make_float2(h ? wv[q].y : wv[q].x, 0.f);
      else x = h ? cconj(wv[q]) : wv[q];
      if (s) {
        const int ex = s * n;
        x = cmul(x, cmul(vtw[ex >> 9], vtw[512 + (ex & 511)]));
      }
      buf[pidx(n)] = x;
    }
  }
  __syncthreads();
  float2* buf = bufs + half * PLN;
  sdif<Plan4096, 256>(buf, tws, ltid);
  const int s = half ? s1 : s0;
  const bool full = u1 < 0;
  const int64_t nq = full ? L / 2 + 1 : (int64_t)(u1 - u0) * O;
  float2* ob = out + ((int64_t)in * nb + b) * nq;
  if (full) {
    int umax = (s == 0) ? P / 2 : P / 2 - 1;
    for (int u = ltid; u <= umax; u += 256) ob[(int64_t)u * O + s] = buf[pidx(spos<Plan4096>(u))];
  } else {
    for (int u = u0 + ltid; u < u1; u += 256) ob[(int64_t)(u - u0) * O + s] = buf[pidx(spos<Plan4096>(u))];
  }
}

// Stage B for a band [u0, u1) of coarse channels (P = 4096, O >= 2): one CTA
// per (slot c, block, input), one transform per slot for c >= 1.  With
// z[n] = W_c[n] w_L^{c n} (w_L = exp(-2 pi i / L)), the input of the fine
// offset O - c is conj(W_c[n]) w_L^{(O-c) n} = conj(z[n]) w_P^{n}, whose DFT is
// conj(Z[P - 1 - u]): so Y[O u + c] = Z[u] and Y[O u + O - c] = conj(Z[P-1-u]),
// the band and its mirror image taken from the same transform (the spectrum
// of the real PFB block is Hermitian).  Slot 0 carries the real W_0 and
// W_{O/2} and takes two transforms.  Only the needed outputs of the last
// radix-16 pass are formed: X[u] = sum_m buf[g(u) + m] w16^(m (u / 256)) with
// g(u) = (u % 16) * 256 + ((u / 16) % 16) * 16 (that pass has no twiddles),
// 16 lanes per channel summed by shuffles.
constexpr int kBandThreads = 256;
__host__ __device__ inline size_t stage_band_smem() {
  return sizeof(float2) * ((size_t)padded_len(4096) + 1024 + 16);
}

__device__ __forceinline__ void band_outputs(const float2* buf, const float2* w16, int u0, int nu, bool mirror, int s,
                                             int O, float2* __restrict__ ob, int tid) {
  constexpr int P = 4096;
  const int l16 = tid & 15, grp = tid >> 4;  // 16 groups of 16 lanes
  const int nu16 = (nu + 15) & ~15;
  for (int i = grp; i < nu16; i += kBandThreads / 16) {
    const int ub = u0 + min(i, nu - 1);
    const int u = mirror ? P - 1 - ub : ub;
    const int g = (u & 15) * 256 + ((u >> 4) & 15) * 16;
    float2 p = cmul(buf[pidx(g) + l16], w16[(l16 * (u >> 8)) & 15]);
#pragma unroll
    for (int off = 8; off >= 1; off >>= 1) {
      p.x += __shfl_xor_sync(0xffffffffu, p.x, off);
      p.y += __shfl_xor_sync(0xffffffffu, p.y, off);
    }
    if (l16 == 0 && i < nu) ob[(int64_t)i * O + s] = mirror ? cconj(p) : p;
  }
}

__global__ void __launch_bounds__(kBandThreads, 3)
    pfb_stage_band_kernel(const float* __restrict__ W, int O, int64_t nb, const float2* __restrict__ twL,
                          const float2* __restrict__ tws, int u0, int u1, float2* __restrict__ out) {
  constexpr int P = 4096, PER = P / kBandThreads;
  extern __shared__ float2 sm2[];
  float2* buf = sm2;
  float2* vtw = buf + padded_len(P);  // hi[512], lo[512]: exp(-2 pi i e / L)
  float2* w16 = vtw + 1024;           // exp(-2 pi i m / 16)
  const int GW = O < 8 ? O : 8, NG = O / GW;
  const int c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const int in = blockIdx.z;
  const int L = P * O;
  const int tid = threadIdx.x;
  const int nhi = (L + 511) / 512;
  for (int i = tid; i < nhi; i += kBandThreads) vtw[i] = __ldg(&twL[(int64_t)i * 512]);
  for (int i = tid; i < 512; i += kBandThreads) vtw[512 + i] = i < L ? __ldg(&twL[i]) : make_float2(1.f, 0.f);
  if (tid < 16) w16[tid] = __ldg(&twL[(int64_t)tid * (L / 16)]);
  // W_c of sample phase n at src + n * GW
  const int g = (2 * c) / GW, e = (2 * c) % GW;
  const float* src = W + ((((int64_t)in * nb + b) * NG + g) * P) * GW + e;
  const int nu = u1 - u0;
  float2* ob = out + ((int64_t)in * nb + b) * ((int64_t)nu * O);
  __syncthreads();
  const int ntr = (c == 0) ? 2 : 1;
  for (int h = 0; h < ntr; h++) {
    const int s = (c == 0) ? (h ? O / 2 : 0) : c;
#pragma unroll 4
    for (int q = 0; q < PER; q++) {
      const int n = tid + q * kBandThreads;
      const float2 wq = __ldg(reinterpret_cast<const float2*>(src + (size_t)n * GW));
      float2 x = (c == 0) ? make_float2(h ? wq.y : wq.x, 0.f) : wq;
      if (s) {
        const int ex = s * n;
        x = cmul(x, cmul(vtw[ex >> 9], vtw[512 + (ex & 511)]));
      }
      buf[pidx(n)] = x;
    }
    __syncthreads();
    spass<16, 256, 4096, kBandThreads, false>(buf, tws + Plan4096::tw_off(0), tid);
    __syncthreads();
    spass<16, 16, 4096, kBandThreads, false>(buf, tws + Plan4096::tw_off(1), tid);
    __syncthreads();
    band_outputs(buf, w16, u0, nu, false, s, O, ob, tid);
    if (c != 0) band_outputs(buf, w16, u0, nu, true, O - c, O, ob, tid);
    __syncthreads();
  }
}

// The same stage with two slots per CTA (O >= 4): slots 2j and 2j+1 fill the
// two 16-byte halves of W's 32-byte (n, group) records, so a CTA reads whole
// halves and each sector passes L1 twice instead of four times (once per
// slot CTA).  Their transforms run side by side in two buffers; the pair
// holding slot 0 takes W_{O/2}'s transform in a second round.  The twiddle
// w_L^(s n) comes from three 64-entry tables (e = s n mod L < 2^18 split in
// 6-bit digits), so two buffers still leave room for three CTAs per SM.
__host__ __device__ inline size_t stage_band2_smem() {
  return sizeof(float2) * (2 * (size_t)padded_len(4096) + 3 * 64 + 16 + 32);
}

__device__ __forceinline__ float2 tw3(const float2* t, int e) {  // exp(-2 pi i e / L), e < 2^18
  return cmul(t[e >> 12], cmul(t[64 + ((e >> 6) & 63)], t[128 + (e & 63)]));
}

__global__ void __launch_bounds__(kBandThreads, 3)
    pfb_stage_band2_kernel(const float* __restrict__ W, int O, int64_t nb, const float2* __restrict__ twL,
                           const float2* __restrict__ tws, int u0, int u1, float2* __restrict__ out) {
  constexpr int P = 4096, PER = P / kBandThreads;
  extern __shared__ float2 sm2[];
  float2* bufA = sm2;
  float2* bufB = bufA + padded_len(P);
  float2* t3 = bufB + padded_len(P);  // [64] w^(4096 i), [64] w^(64 i), [64] w^i
  float2* w16 = t3 + 192;             // exp(-2 pi i m / 16)
  float2* qtw = w16 + 16;             // [2][16] w_L^(256 s q) for the two slots
  const int GW = O < 8 ? O : 8, NG = O / GW;
  const int j = blockIdx.x;  // slots 2j, 2j + 1
  const int64_t b = blockIdx.y;
  const int in = blockIdx.z;
  const int L = P * O;
  const int tid = threadIdx.x;
  if (tid < 192) {
    const int d = tid >> 6, i = tid & 63;
    const int64_t e = d == 0 ? (int64_t)i * 4096 : d == 1 ? (int64_t)i * 64 : i;
    t3[tid] = e < L ? __ldg(&twL[e]) : make_float2(1.f, 0.f);
  }
  if (tid < 16) w16[tid] = __ldg(&twL[(int64_t)tid * (L / 16)]);
  const int c0 = 2 * j;
  const int sA = c0, sB = c0 + 1;
  // w_L^(s n) for n = tid + 256 q is w_L^(s tid) w_L^(256 s q): one factor per
  // thread, one per q (exact table entries, so two roundings as tw3)
  if (tid < 32) {
    const int s = tid < 16 ? sA : sB, q = tid & 15;
    qtw[tid] = __ldg(&twL[((int64_t)s * kBandThreads * q) % L]);
  }
  const int g = (2 * c0) / GW, e0 = (2 * c0) % GW;  // slot c0 at float e0 of group g (0 or 4)
  const float* src = W + ((((int64_t)in * nb + b) * NG + g) * P) * GW + e0;
  const int nu = u1 - u0;
  float2* ob = out + ((int64_t)in * nb + b) * ((int64_t)nu * O);
  __syncthreads();
  const float2 bA = tw3(t3, (int)(((int64_t)sA * tid) % L)), bB = tw3(t3, (int)(((int64_t)sB * tid) % L));
#pragma unroll 16
  for (int q = 0; q < PER; q++) {
    const int n = tid + q * kBandThreads;
    const float4 v = __ldg(reinterpret_cast<const float4*>(src + (size_t)n * GW));
    float2 xa = j == 0 ? make_float2(v.x, 0.f) : make_float2(v.x, v.y);  // slot 0: the real W_0
    if (sA) xa = cmul(cmul(xa, bA), qtw[q]);
    bufA[pidx(n)] = xa;
    bufB[pidx(n)] = cmul(cmul(make_float2(v.z, v.w), bB), qtw[16 + q]);
  }
  __syncthreads();
  spass<16, 256, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(0), tid);
  spass<16, 256, 4096, kBandThreads, false>(bufB, tws + Plan4096::tw_off(0), tid);
  __syncthreads();
  spass<16, 16, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(1), tid);
  spass<16, 16, 4096, kBandThreads, false>(bufB, tws + Plan4096::tw_off(1), tid);
  __syncthreads();
  band_outputs(bufA, w16, u0, nu, false, sA, O, ob, tid);
  if (sA != 0) band_outputs(bufA, w16, u0, nu, true, O - sA, O, ob, tid);
  band_outputs(bufB, w16, u0, nu, false, sB, O, ob, tid);
  band_outputs(bufB, w16, u0, nu, true, O - sB, O, ob, tid);
  if (j == 0) {  // W_{O/2}, the second real value of slot 0
    const int sH = O / 2;
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < PER; q++) {
      const int n = tid + q * kBandThreads;
      const float wv = __ldg(src + (size_t)n * GW + 1);
      bufA[pidx(n)] = cmul(make_float2(wv, 0.f), tw3(t3, (int)(((int64_t)sH * n) % L)));
    }
    __syncthreads();
    spass<16, 256, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(0), tid);
    __syncthreads();
    spass<16, 16, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(1), tid);
    __syncthreads();
    band_outputs(bufA, w16, u0, nu, false, sH, O, ob, tid);
  }
}


// Persistent TMA form of the two-slot band DFT.  One CTA of kBtThreads per SM
// walks the (slot pair, block, input) tiles.  A tile's W records (4096 sample
// phases x the 16 bytes its two slots share) arrive as 16 TMA boxes (4 floats
// x 256 phases each) in a 64 KB landing tile and complete on one mbarrier;
// once they are twiddled into the two FFT buffers the landing tile is free,
// and the next tile's boxes are issued into it at once, so they arrive while
// this tile's radix-16 passes and band outputs run.  The two slots' passes run
// side by side, one per half of the CTA.  The arithmetic is that of
// pfb_stage_band2_kernel.  A wait that runs out (about 2 s) sets *fault and
// stops the CTA; the fine correlator then writes NaN into the visibilities.
constexpr int kBtThreads = 512;

__host__ __device__ inline size_t stage_band_tma_smem() {
  return 1024 + (size_t)4096 * 16 + sizeof(float2) * (2 * (size_t)padded_len(4096) + 3 * 64 + 16 + 32) + 64;
}

__global__ void __launch_bounds__(kBtThreads, 1)
    pfb_stage_band_tma_kernel(const __grid_constant__ CUtensorMap wmap, int O, int64_t nb, int ninputs,
                              const float2* __restrict__ twL, const float2* __restrict__ tws, int u0, int u1,
                              float2* __restrict__ out, int* __restrict__ fault) {
  constexpr int P = 4096;
  extern __shared__ uint8_t smb[];
  const uint32_t raw_s = smem_u32(smb);
  const uint32_t pad = (1024u - (raw_s & 1023u)) & 1023u;
  float4* stage = reinterpret_cast<float4*>(smb + pad);  // [4096]: the pair's 4 floats of W per sample phase
  const uint32_t stage_s = raw_s + pad;
  float2* bufA = reinterpret_cast<float2*>(smb + pad + 4096 * 16);
  float2* bufB = bufA + padded_len(P);
  float2* t3 = bufB + padded_len(P);  // [64] w^(4096 i), [64] w^(64 i), [64] w^i
  float2* w16 = t3 + 192;
  float2* qtw = w16 + 16;             // [2][16] w_L^(256 s q) for the tile's two slots
  uint64_t* barp = reinterpret_cast<uint64_t*>(qtw + 32);
  int* abort_flag = reinterpret_cast<int*>(barp + 1);
  const uint32_t bar = smem_u32(barp);
  const int GW = O < 8 ? O : 8, NG = O / GW, NJ = O / 4;
  const int L = P * O;
  const int tid = threadIdx.x, half = tid >> 8, ht = tid & 255;
  const int64_t ntile = (int64_t)NJ * nb * ninputs;
  const int nu = u1 - u0;
  if (tid < 192) {
    const int d = tid >> 6, i = tid & 63;
    const int64_t e = d == 0 ? (int64_t)i * 4096 : d == 1 ? (int64_t)i * 64 : i;
    t3[tid] = e < L ? __ldg(&twL[e]) : make_float2(1.f, 0.f);
  }
  if (tid < 16) w16[tid] = __ldg(&twL[(int64_t)tid * (L / 16)]);
  if (tid == 0) {
    *abort_flag = 0;
    mbar_init(bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  // the 16 boxes of tile t: x = the pair's first float in its 8-float group,
  // y = the W row (((in nb + b) NG + g) P + n) of sample phase n = 256 r
  auto issue = [&](int64_t t) {
    const int j = (int)(t % NJ);
    const int64_t rest = t / NJ, b = rest % nb, in = rest / nb;
    const int g = (4 * j) / GW, e0 = (4 * j) % GW;
    const int64_t row0 = ((in * nb + b) * NG + g) * P;
    fence_proxy_async();
    mbar_arrive_expect_tx(bar, 4096 * 16);
#pragma unroll 1
    for (int r = 0; r < 16; r++) tma_load_2d(stage_s + r * 256 * 16, &wmap, e0, (int)(row0 + 256 * r), bar);
  };
  if (tid == 0 && blockIdx.x < ntile) issue(blockIdx.x);
  uint32_t phase = 0;
  for (int64_t t = blockIdx.x; t < ntile; t += gridDim.x, phase ^= 1) {
    const int j = (int)(t % NJ);
    const int64_t rest = t / NJ, b = rest % nb, in = rest / nb;
    const int sA = 2 * j, sB = 2 * j + 1;
    if (tid < 32) {
      const int s = tid < 16 ? sA : sB, q = tid & 15;
      qtw[tid] = __ldg(&twL[((int64_t)s * 256 * q) % L]);
    }
    if (tid == 0 && !mbar_wait(bar, phase)) {
      atomicExch(fault, 1);
      *abort_flag = 1;
    }
    __syncthreads();
    if (*abort_flag) break;
    float2* ob = out + ((int64_t)in * nb + b) * ((int64_t)nu * O);
    // twiddle both slots into their buffers: phases n = ht + 256 q, q in this half's 8
    const float2 bA = tw3(t3, (int)(((int64_t)sA * ht) % L)), bB = tw3(t3, (int)(((int64_t)sB * ht) % L));
    float wv[8];  // slot O/2 (the second real value of slot 0's record) when j == 0
#pragma unroll
    for (int qq = 0; qq < 8; qq++) {
      const int q = 8 * half + qq, n = ht + 256 * q;
      const float4 v = stage[n];
      float2 xa = j == 0 ? make_float2(v.x, 0.f) : make_float2(v.x, v.y);  // slot 0: the real W_0
      if (sA) xa = cmul(cmul(xa, bA), qtw[q]);
      bufA[pidx(n)] = xa;
      bufB[pidx(n)] = cmul(cmul(make_float2(v.z, v.w), bB), qtw[16 + q]);
      wv[qq] = v.y;
    }
    // the next tile's boxes are written by the asynchronous proxy: every
    // thread orders its generic reads of the landing tile before them
    fence_proxy_async();
    __syncthreads();  // the landing tile is consumed: fetch the next tile into it
    if (tid == 0 && t + gridDim.x < ntile) issue(t + gridDim.x);
    float2* buf = half ? bufB : bufA;
    spass<16, 256, 4096, 256, false>(buf, tws + Plan4096::tw_off(0), ht);
    __syncthreads();
    spass<16, 16, 4096, 256, false>(buf, tws + Plan4096::tw_off(1), ht);
    __syncthreads();
    if (half == 0) {
      band_outputs(bufA, w16, u0, nu, false, sA, O, ob, ht);
      if (sA != 0) band_outputs(bufA, w16, u0, nu, true, O - sA, O, ob, ht);
    } else {
      band_outputs(bufB, w16, u0, nu, false, sB, O, ob, ht);
      band_outputs(bufB, w16, u0, nu, true, O - sB, O, ob, ht);
    }
    if (j == 0) {  // W_{O/2}: the pair holding slot 0 takes a third transform
      const int sH = O / 2;
      __syncthreads();
#pragma unroll
      for (int qq = 0; qq < 8; qq++) {
        const int n = ht + 256 * (8 * half + qq);
        bufA[pidx(n)] = cmul(make_float2(wv[qq], 0.f), tw3(t3, (int)(((int64_t)sH * n) % L)));
      }
      __syncthreads();
      if (half == 0) spass<16, 256, 4096, 256, false>(bufA, tws + Plan4096::tw_off(0), ht);
      __syncthreads();
      if (half == 0) spass<16, 16, 4096, 256, false>(bufA, tws + Plan4096::tw_off(1), ht);
      __syncthreads();
      if (half == 0) band_outputs(bufA, w16, u0, nu, false, sH, O, ob, ht);
    }
    __syncthreads();  // buffers and slot twiddles are rewritten by the next tile
  }
}


// TMA form with three CTAs per SM: one CTA per tile as pfb_stage_band2_kernel,
// whose 16 TMA boxes land in the space of its two FFT buffers (64 KB of the
// 69.6 KB); each thread reads its 16 records from there into registers, and
// after a barrier writes the twiddled values over them.  The other two CTAs
// of the SM transform while a CTA's boxes are in flight.  A wait that runs
// out (about 2 s) sets *fault; the CTA then writes nothing.
__host__ __device__ inline size_t stage_band2_tma_smem() { return 1024 + stage_band2_smem() + 16; }

__global__ void __launch_bounds__(kBandThreads, 3)
    pfb_stage_band2_tma_kernel(const __grid_constant__ CUtensorMap wmap, const float* __restrict__ W, int O,
                               int64_t nb, const float2* __restrict__ twL, const float2* __restrict__ tws, int u0,
                               int u1, float2* __restrict__ out, int* __restrict__ fault) {
  constexpr int P = 4096, PER = P / kBandThreads;
  extern __shared__ uint8_t smb2[];
  const uint32_t raw_s = smem_u32(smb2);
  const uint32_t pad = (1024u - (raw_s & 1023u)) & 1023u;
  float2* bufA = reinterpret_cast<float2*>(smb2 + pad);
  float2* bufB = bufA + padded_len(P);
  const float4* stage = reinterpret_cast<const float4*>(bufA);  // landing tile, [4096] float4 over bufA/bufB
  const uint32_t stage_s = raw_s + pad;
  float2* t3 = bufB + padded_len(P);
  float2* w16 = t3 + 192;
  float2* qtw = w16 + 16;
  uint64_t* barp = reinterpret_cast<uint64_t*>(qtw + 32);
  int* ok_flag = reinterpret_cast<int*>(barp + 1);
  const uint32_t bar = smem_u32(barp);
  const int GW = O < 8 ? O : 8, NG = O / GW;
  const int j = blockIdx.x;
  const int64_t b = blockIdx.y;
  const int in = blockIdx.z;
  const int L = P * O;
  const int tid = threadIdx.x;
  const int c0 = 2 * j;
  const int sA = c0, sB = c0 + 1;
  const int g = (2 * c0) / GW, e0 = (2 * c0) % GW;
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init_fence();
    mbar_arrive_expect_tx(bar, 4096 * 16);
    const int64_t row0 = (((int64_t)in * nb + b) * NG + g) * P;
#pragma unroll 1
    for (int r = 0; r < 16; r++) tma_load_2d(stage_s + r * 256 * 16, &wmap, e0, (int)(row0 + 256 * r), bar);
  }
  if (tid < 192) {
    const int d = tid >> 6, i = tid & 63;
    const int64_t e = d == 0 ? (int64_t)i * 4096 : d == 1 ? (int64_t)i * 64 : i;
    t3[tid] = e < L ? __ldg(&twL[e]) : make_float2(1.f, 0.f);
  }
  if (tid < 16) w16[tid] = __ldg(&twL[(int64_t)tid * (L / 16)]);
  if (tid < 32) {
    const int s = tid < 16 ? sA : sB, q = tid & 15;
    qtw[tid] = __ldg(&twL[((int64_t)s * kBandThreads * q) % L]);
  }
  const int nu = u1 - u0;
  float2* ob = out + ((int64_t)in * nb + b) * ((int64_t)nu * O);
  if (tid == 0) {
    const bool ok = mbar_wait(bar, 0);
    if (!ok) atomicExch(fault, 1);
    *ok_flag = ok;
  }
  __syncthreads();
  if (!*ok_flag) return;
  float4 v[PER];
#pragma unroll
  for (int q = 0; q < PER; q++) v[q] = stage[tid + q * kBandThreads];
  __syncthreads();  // the landing tile is read: the buffers are written over it
  const float2 bA = tw3(t3, (int)(((int64_t)sA * tid) % L)), bB = tw3(t3, (int)(((int64_t)sB * tid) % L));
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int n = tid + q * kBandThreads;
    float2 xa = j == 0 ? make_float2(v[q].x, 0.f) : make_float2(v[q].x, v[q].y);
    if (sA) xa = cmul(cmul(xa, bA), qtw[q]);
    bufA[pidx(n)] = xa;
    bufB[pidx(n)] = cmul(cmul(make_float2(v[q].z, v[q].w), bB), qtw[16 + q]);
  }
  __syncthreads();
  spass<16, 256, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(0), tid);
  spass<16, 256, 4096, kBandThreads, false>(bufB, tws + Plan4096::tw_off(0), tid);
  __syncthreads();
  spass<16, 16, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(1), tid);
  spass<16, 16, 4096, kBandThreads, false>(bufB, tws + Plan4096::tw_off(1), tid);
  __syncthreads();
  band_outputs(bufA, w16, u0, nu, false, sA, O, ob, tid);
  if (sA != 0) band_outputs(bufA, w16, u0, nu, true, O - sA, O, ob, tid);
  band_outputs(bufB, w16, u0, nu, false, sB, O, ob, tid);
  band_outputs(bufB, w16, u0, nu, true, O - sB, O, ob, tid);
  if (j == 0) {  // W_{O/2}, the second real value of slot 0
    const int sH = O / 2;
    __syncthreads();
    const float* src = W + ((((int64_t)in * nb + b) * NG + g) * P) * GW + e0;  // slot 0's record (re-read)
#pragma unroll 4
    for (int q = 0; q < PER; q++) {
      const int n = tid + q * kBandThreads;
      const float wv = __ldg(src + (size_t)n * GW + 1);
      bufA[pidx(n)] = cmul(make_float2(wv, 0.f), tw3(t3, (int)(((int64_t)sH * n) % L)));
    }
    __syncthreads();
    spass<16, 256, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(0), tid);
    __syncthreads();
    spass<16, 16, 4096, kBandThreads, false>(bufA, tws + Plan4096::tw_off(1), tid);
    __syncthreads();
    band_outputs(bufA, w16, u0, nu, false, sH, O, ob, tid);
  }
}

int launch_pfb_stage_a(const TsSrc& src, int ninputs, int P, int O, int ntap, int64_t row0, int64_t nb,
                       const float* win, float* W, const float2* tw64, cudaStream_t s) {
  AB_CHECK_ARG(P % kFoldCols == 0, "pfb: lblock/osamp %d must be a multiple of %d", P, kFoldCols);
  AB_CHECK_ARG(ntap >= 1 && ntap <= 16, "pfb: ntap %d out of range", ntap);
  if (nb <= 0) return AB_OK;
  size_t smem = stage_a_smem(O, ntap);
  AB_CHECK_ARG(smem <= 220 * 1024, "pfb: tile of %zu bytes too large (osamp %d, ntap %d)", smem, O, ntap);
  // float4 tile loads need 16-byte aligned column rows
  const int vec4 = !src.natural && src.ld % 4 == 0 && src.off % 4 == 0 && src.prev_off % 4 == 0 &&
                   row0 % 4 == 0 && ((kFoldBlocks + ntap - 1) * O) % 4 == 0 && ((uintptr_t)src.cur & 15) == 0 &&
                   ((uintptr_t)src.prev & 15) == 0;
  dim3 grid((unsigned)((nb + kFoldBlocks - 1) / kFoldBlocks), (unsigned)(P / kFoldCols), (unsigned)ninputs);
  dim3 block(kFoldCols * kFoldBlocks);
#define AB_STAGE_A(OO)                                                                                        \
  case OO:                                                                                                   \
    AB_CUDA(cudaFuncSetAttribute(pfb_stage_a_kernel<OO>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024)); \
    pfb_stage_a_kernel<OO><<<grid, block, smem, s>>>(src, P, ntap, row0, nb, win, W, tw64, vec4);             \
    break;
  switch (O) {
    AB_STAGE_A(1)
    AB_STAGE_A(2)
    AB_STAGE_A(4)
    AB_STAGE_A(8)
    AB_STAGE_A(16)
    AB_STAGE_A(32)
    AB_STAGE_A(64)
    default:
      set_error("pfb: osamp %d not supported (1..64, power of two)", O);
      return AB_ERR_UNSUPPORTED;
  }
#undef AB_STAGE_A
  AB_LAUNCH_CHECK();
  return AB_OK;
}

int launch_pfb_stage_b(ab_ctx* ctx, const float* W, int ninputs, int P, int O, int64_t nb, const FftPlan& planP,
                       const float2* twL, int u0, int u1, float2* out, cudaStream_t s, int* fault) {
  if (nb <= 0) return AB_OK;
  const int GW = O < 8 ? O : 8;
  size_t smem = sizeof(float) * (size_t)P * GW + sizeof(float2) * ((size_t)padded_len(P) + smem_tw_len(P * O));
  AB_CHECK_ARG(smem <= 220 * 1024, "pfb: stage B needs %zu bytes of shared memory", smem);
  dim3 grid((unsigned)nb, (unsigned)(O / GW), (unsigned)ninputs);
  const int64_t wrows = (int64_t)ninputs * nb * (O / GW) * P;
  if (fault && ctx->pfb_tma && P == Plan4096::N && O >= 4 && O <= 64 && u1 >= 0 && ((uintptr_t)W & 15) == 0 &&
      wrows < (1ll << 31) && nb <= 65535 && stage_band_tma_smem() <= ctx->smem_optin) {
    // W as a 2-D tensor: rows of GW floats (32 or 16 bytes), boxes of 4 floats x 256 rows
    CUtensorMap map;
    const uint64_t dims[2] = {(uint64_t)GW, (uint64_t)wrows}, strides[1] = {(uint64_t)GW * sizeof(float)};
    const uint32_t box[2] = {4, 256};
    AB_TRY(encode_tmap(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, W, dims, strides, box));
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    if (ctx->pfb_tma == 2) {
      const size_t sm = stage_band_tma_smem();
      AB_CUDA(cudaFuncSetAttribute(pfb_stage_band_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      const int64_t ntile = (int64_t)(O / 4) * nb * ninputs;
      const unsigned g = (unsigned)std::min<int64_t>(ntile, std::max(ctx->num_sms, 1));
      pfb_stage_band_tma_kernel<<<g, kBtThreads, sm, s>>>(map, O, nb, ninputs, twL, tws, u0, u1, out, fault);
    } else {
      const size_t sm = stage_band2_tma_smem();
      AB_CUDA(cudaFuncSetAttribute(pfb_stage_band2_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      dim3 g2((unsigned)(O / 4), (unsigned)nb, (unsigned)ninputs);
      pfb_stage_band2_tma_kernel<<<g2, kBandThreads, sm, s>>>(map, W, O, nb, twL, tws, u0, u1, out, fault);
    }
  } else if (P == Plan4096::N && O >= 4 && O <= 64 && nb <= 65535 && u1 >= 0 && ((uintptr_t)W & 15) == 0) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    size_t sm = stage_band2_smem();
    AB_CUDA(cudaFuncSetAttribute(pfb_stage_band2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dim3 g2((unsigned)(O / 4), (unsigned)nb, (unsigned)ninputs);
    pfb_stage_band2_kernel<<<g2, kBandThreads, sm, s>>>(W, O, nb, twL, tws, u0, u1, out);
  } else if (P == Plan4096::N && O >= 2 && nb <= 65535 && u1 >= 0) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    size_t sm = stage_band_smem();
    AB_CUDA(cudaFuncSetAttribute(pfb_stage_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dim3 g2((unsigned)(O / 2), (unsigned)nb, (unsigned)ninputs);
    pfb_stage_band_kernel<<<g2, kBandThreads, sm, s>>>(W, O, nb, twL, tws, u0, u1, out);
  } else if (P == Plan4096::N && O >= 2 && nb <= 65535) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    size_t sm = stage_bslot_smem();
    AB_CUDA(cudaFuncSetAttribute(pfb_stage_bslot_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dim3 g2((unsigned)(O / 2), (unsigned)nb, (unsigned)ninputs);
    pfb_stage_bslot_kernel<<<g2, kBSThreads, sm, s>>>(W, O, nb, twL, tws, u0, u1, out);
  } else if (P == Plan4096::N && O >= 8) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    size_t sm2 = stage_b2_smem();
    AB_CUDA(cudaFuncSetAttribute(pfb_stage_b4096_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
    pfb_stage_b4096_kernel<<<grid, kB2Threads, sm2, s>>>(W, O, nb, twL, tws, u0, u1, out);
  } else if (P == Plan4096::N) {
    const float2* tws;
    AB_TRY(get_twiddle_stream(ctx, P, {16, 16, 16}, &tws));
    AB_CUDA(cudaFuncSetAttribute(pfb_stage_b_kernel<Plan4096>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    pfb_stage_b_kernel<Plan4096><<<grid, kStageBThreads, smem, s>>>(W, P, O, nb, planP, twL, tws, u0, u1, out);
  } else {
    AB_CUDA(cudaFuncSetAttribute(pfb_stage_b_kernel<NoPlanB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    pfb_stage_b_kernel<NoPlanB><<<grid, kStageBThreads, smem, s>>>(W, P, O, nb, planP, twL, nullptr, u0, u1, out);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

// split lblock into P (<= 4096) and O = lblock / P
static bool split_lblock(int64_t L, int* P, int* O) {
  if (L < 64 || (L & (L - 1))) return false;
  *P = (int)(L < 4096 ? L : 4096);
  *O = (int)(L / *P);
  return *O <= 64;
}

static int pfb_common(ab_ctx* ctx, const float* ts, int64_t nsamp, const float* win, int64_t nchan, int64_t ntap,
                      int64_t q0, int64_t q1, bool band, float* out, void* stream) {
  const char* name = band ? "ab_pfb_band" : "ab_pfb";
  AB_CHECK_ARG(ctx && ts && win && out, "%s: NULL pointer", name);
  AB_CHECK_ARG(nchan >= 2 && ntap >= 1, "%s: bad nchan/ntap", name);
  const int64_t L = 2 * (nchan - 1);
  int P, O;
  if (!split_lblock(L, &P, &O)) {
    set_error("%s: lblock %lld must be a power of two in [64, 262144]", name, (long long)L);
    return AB_ERR_UNSUPPORTED;
  }
  int64_t nblock = nsamp / L - (ntap - 1);
  AB_CHECK_ARG(nblock >= 0, "%s: timestream shorter than ntap blocks", name);
  if (nblock == 0) return AB_OK;
  int u0 = -1, u1 = -1;
  if (band) {
    AB_CHECK_ARG(q0 % O == 0 && q1 % O == 0 && q0 >= 0 && q1 > q0 && q1 <= (int64_t)P * O / 2 + 1,
                 "ab_pfb_band: band [%lld, %lld) must be multiples of osamp %d inside the spectrum", (long long)q0,
                 (long long)q1, O);
    u0 = (int)(q0 / O);
    u1 = (int)(q1 / O);
    AB_CHECK_ARG(u1 <= P / 2 || (u1 == P / 2 + 1 && O == 1), "ab_pfb_band: band beyond Nyquist");
  }
  FftPlan planP;
  if (!ctx_plan(ctx, P, &planP)) return AB_ERR_UNSUPPORTED;
  const float2* twL;
  AB_TRY(get_twiddles(ctx, L, &twL));
  void* Wv = nullptr;
  AB_TRY(get_scratch(ctx, kScratchPfbW, sizeof(float) * (size_t)(nblock * L), &Wv));
  TsSrc src{ts, nullptr, 0, 0, 0, nsamp / P, 1};
  cudaStream_t s = as_stream(stream);
  AB_TRY(launch_pfb_stage_a(src, 1, P, O, (int)ntap, 0, nblock, win, (float*)Wv, ctx->tw64, s));
  AB_TRY(launch_pfb_stage_b(ctx, (const float*)Wv, 1, P, O, nblock, planP, twL, u0, u1, (float2*)out, s, nullptr));
  return AB_OK;
}

}  // namespace ab

using namespace ab;

extern "C" int ab_pfb(ab_ctx* ctx, const float* timestream, int64_t nsamp, const float* win, int64_t nchan,
                      int64_t ntap, float* out, void* stream) {
  return pfb_common(ctx, timestream, nsamp, win, nchan, ntap, 0, 0, false, out, stream);
}

extern "C" int ab_pfb_band(ab_ctx* ctx, const float* timestream, int64_t nsamp, const float* win, int64_t nchan,
                           int64_t ntap, int64_t q0, int64_t q1, float* out, void* stream) {
  return pfb_common(ctx, timestream, nsamp, win, nchan, ntap, q0, q1, true, out, stream);
}
