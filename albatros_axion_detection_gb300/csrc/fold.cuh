// fold.cuh -- fused PFB fold + osamp-point real DFT (stage A of the forward
// PFB) over one sample phase's IPFB output held in shared memory; shared by
// the FFT-based and the FIR-based time stages of the streaming chain.
#pragma once
#include "fft.cuh"
#include "ipfb.cuh"

namespace ab {

// Warp-level PFB fold + osamp-point real DFT over the IPFB output of one
// sample phase n held in shared memory.  Timestream row rr of the chunk is
// float (fa.cut + rr) of `buf` in the pidx-padded float2 layout (row pair
// (2s, 2s+1) in slot pidx(s)); rows >= fa.acclen read as zero; rows < 0 come
// from `stail` (the previous chunk's last 4*O rows) unless TAILBUF, in which
// case they are in `buf` as well.  Blocks b in [b0, b1) start at row
// fa.row0 + b*O.  A group of G = O/2 lanes owns one block: lane m folds
// rows 2m, 2m+1 (z_m = y[2m] + i y[2m+1]) with the ntap window taps, the group
// takes a G-point complex DFT by shuffles (decimation in frequency, output in
// bit-reversed lane order) and untangles the real-input spectrum W_k,
// k = 0..O/2, written to W[in][b][g][n][GW] (the stage-A layout).
template <int G, int NTAP, bool TAILBUF>
__device__ __forceinline__ void fold_blocks(const float2* buf, const float* stail, const FoldArgs& fa, int P, int n,
                                            int in, const float2* __restrict__ tw64, int b0, int b1) {
  constexpr int O = 2 * G;
  constexpr int LOG = G == 1 ? 0 : G == 2 ? 1 : G == 4 ? 2 : G == 8 ? 3 : G == 16 ? 4 : 5;
  constexpr int GW = O < 8 ? O : 8;
  constexpr int BPW = 32 / G;  // blocks per warp
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int m = lane % G, grp = lane / G;
  // window taps of rows 2m, 2m+1 for this sample phase
  float w0[NTAP], w1[NTAP];
#pragma unroll
  for (int i = 0; i < NTAP; i++) {
    w0[i] = __ldg(&fa.win[(int64_t)(i * O + 2 * m) * P + n]);
    w1[i] = __ldg(&fa.win[(int64_t)(i * O + 2 * m + 1) * P + n]);
  }
  // per-stage DIF twiddles exp(-2 pi i (m mod h) / (2h)) and lane roles
  float2 stw[LOG > 0 ? LOG : 1];
  bool upper[LOG > 0 ? LOG : 1];
#pragma unroll
  for (int st = 0; st < LOG; st++) {
    const int h = G >> (st + 1);
    stw[st] = tw64[(m % h) * (32 / h)];
    upper[st] = (m & h) != 0;
  }
  // bit-reversed frequency held by this lane after the DFT, and its partner
  int k = 0, src_lane = 0;
#pragma unroll
  for (int bit = 0; bit < LOG; bit++) k |= ((m >> bit) & 1) << (LOG - 1 - bit);
  const int kc = (G - k) % G;
#pragma unroll
  for (int bit = 0; bit < LOG; bit++) src_lane |= ((kc >> bit) & 1) << (LOG - 1 - bit);
  src_lane += grp * G;
  const float2 wk = tw64[(k * (64 / O)) & 63];  // exp(-2 pi i k / O)
  const bool kzero = (k == 0);
  const int pk = 2 * k;                       // packed float position ((W_0, W_{O/2}) for k = 0)
  // W[in][b][g][n][GW] with g = pk / GW, e = pk % GW
  float* const wbase = fa.W + (int64_t)in * fa.nb * ((int64_t)O * P) + ((int64_t)(pk / GW) * P + n) * GW + (pk % GW);
  const int64_t bstride = (int64_t)O * P;
  const int row0 = (int)fa.row0, cut = fa.cut, acclen = fa.acclen;
  const int nbw = (b1 - b0 + BPW - 1) / BPW;
  const float* fbuf = reinterpret_cast<const float*>(buf);
  // rows of a block start at an even IPFB row when cut + row0 is even: then
  // each lane's pair (2m, 2m+1) is one float2 slot of the column buffer
  const bool even = ((cut + row0) & 1) == 0;
  for (int wb = warp; wb < nbw; wb += nwarps) {
    const int b = b0 + wb * BPW + grp;
    const bool valid = b < b1;
    const int rfirst = row0 + b * O;
    float2 z = make_float2(0.f, 0.f);
    if (valid) {
      if (even && (TAILBUF || rfirst >= 0) && rfirst + NTAP * O <= acclen) {
        const int s0 = ((cut + rfirst) >> 1) + m;  // slot of rows (2m, 2m+1)
        const int ps0 = pidx(s0);
#pragma unroll
        for (int i = 0; i < NTAP; i++) {
          const float2 v = buf[(G % 16 == 0) ? ps0 + i * (G + G / 16) : pidx(s0 + i * G)];
          z.x = fmaf(v.x, w0[i], z.x);
          z.y = fmaf(v.y, w1[i], z.y);
        }
      } else {
        auto get = [&](int rr) -> float {
          if (!TAILBUF && rr < 0) return stail[rr + 4 * O];
          if (rr >= acclen) return 0.f;
          const int t = cut + rr;
          return fbuf[2 * pidx(t >> 1) + (t & 1)];
        };
        const int rb = rfirst + 2 * m;
#pragma unroll
        for (int i = 0; i < NTAP; i++) {
          z.x = fmaf(get(rb + i * O), w0[i], z.x);
          z.y = fmaf(get(rb + i * O + 1), w1[i], z.y);
        }
      }
    }
    // G-point DIF across the group (branch-free)
#pragma unroll
    for (int st = 0; st < LOG; st++) {
      const int h = G >> (st + 1);
      float2 v;
      v.x = __shfl_xor_sync(0xffffffffu, z.x, h);
      v.y = __shfl_xor_sync(0xffffffffu, z.y, h);
      const float2 lo = cadd(z, v), hi = cmul(csub(v, z), stw[st]);
      z = upper[st] ? hi : lo;
    }
    // untangle: W_k = (Z_k + conj Z_{G-k})/2 + w^k (Z_k - conj Z_{G-k})/(2i)
    float2 zc;
    zc.x = __shfl_sync(0xffffffffu, z.x, src_lane);
    zc.y = __shfl_sync(0xffffffffu, z.y, src_lane);
    const float2 c = cconj(zc);
    const float2 E = cscale(cadd(z, c), 0.5f);
    const float2 D = csub(z, c);  // 2 i O_k
    const float2 Od = make_float2(0.5f * D.y, -0.5f * D.x);
    float2 outv = cadd(E, cmul(wk, Od));
    if (kzero) outv = make_float2(z.x + z.y, z.x - z.y);  // (W_0, W_{O/2})
    if (valid) *reinterpret_cast<float2*>(wbase + (int64_t)b * bstride) = outv;
  }
}

}  // namespace ab
