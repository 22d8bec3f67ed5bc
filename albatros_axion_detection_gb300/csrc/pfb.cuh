// pfb.cuh -- internal launch interfaces of the forward-PFB stages.
//
// For lblock L = P * O (P = 4096 coarse samples, O = osamp), a PFB block of
// tap-folded samples y[k], k = n + P t' (n < P, t' < O), has the spectrum
//   Y[O u + s] = sum_n exp(-2 pi i u n / P) exp(-2 pi i s n / L)
//                     sum_t' y[n + P t'] exp(-2 pi i s t' / O)
// Stage A folds the ntap taps and takes the O-point real DFT over t' for
// every sample phase n (W_s[n], s <= O/2); stage B twiddles and takes the
// P-point DFT over n for each fine offset s.  Output bin q = O u + s, i.e.
// u is the coarse channel and s the fine offset inside it.
#pragma once
#include "common.cuh"

namespace ab {

// Where stage A reads timestream row r (a row = P consecutive samples) of
// sample phase n for input `in`:
//   natural layout: cur[r * P + n] (single input, row-major);
//   column layout : cur[(in*P + n)*ld + off + r] for r >= 0, and
//                   prev[(in*P + n)*ld + prev_off + r] for r < 0.
// Rows >= nrows_valid read as zero.
struct TsSrc {
  const float* cur;
  const float* prev;
  int64_t ld;
  int64_t off;
  int64_t prev_off;
  int64_t nrows_valid;
  int natural;
};

// W layout: W[in][b][g][n][GW], GW = min(O, 8) floats per group,
// NG = O / GW groups: packed (W_0, W_{O/2}, Re W_1, Im W_1, ...).
int launch_pfb_stage_a(const TsSrc& src, int ninputs, int P, int O, int ntap, int64_t row0, int64_t nb,
                       const float* win, float* W, const float2* tw64, cudaStream_t s);

// Stage B.  band: u in [u0, u1), out[(in*nb + b)*(u1-u0)*O + (u-u0)*O + s];
// full (u1 < 0): out[(in*nb + b)*(L/2+1) + q] for q <= L/2.
// fault: a device word set when an asynchronous copy of the TMA form does not
// arrive in time (the TMA form runs only when fault is given).
int launch_pfb_stage_b(ab_ctx* ctx, const float* W, int ninputs, int P, int O, int64_t nb, const FftPlan& planP,
                       const float2* twL, int u0, int u1, float2* out, cudaStream_t s, int* fault = nullptr);

}  // namespace ab
