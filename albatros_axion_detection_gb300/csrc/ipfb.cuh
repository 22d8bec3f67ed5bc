// ipfb.cuh -- internal launch interfaces of the IPFB stages shared by the
// one-shot ab_ipfb() entry point and the streaming chain.
#pragma once
#include "common.cuh"

namespace ab {

// Sample-phase-major ("[n][t]") intermediate: element (t, n) of an input's
// (nslice, P) timestream lives at buf[(input * P + n) * ld + t].  This is the
// memory layout of the reference's returned IPFB view (res.T of a C-ordered
// (P, nslice) array), and makes the time-axis transform of one sample phase a
// contiguous column.

// Stage 1 source: 4-bit packets of nant antennas, both pols per antenna.
struct Packed4Src {
  const uint8_t* raw;        // antenna a at raw + a * ant_stride
  int64_t ant_stride;        // bytes
  int64_t row_bytes;         // 2 * nchan_raw (4-bit) or nchan_raw / 2 (1-bit)
  const int32_t* spec_map;   // optional: raw row of global spectrum g (or <0)
  int64_t map_stride;        // per-antenna stride of spec_map
  int64_t g0;                // global spectrum of local row 0 (may be negative)
  const int32_t* chan_cols;  // device (nsel): raw column per selected channel
  const int32_t* chan_abs;   // device (nsel): absolute bin 0..P/2
  int nsel;
  int bits;                  // 4: one byte per channel per pol; 1: sign bits,
                             // byte j = channels 2j, 2j+1 (r0 i0 r1 i1 each, MSB first)
};

// Row stage for packed 4-bit input: local rows t in [0, nrows) of every
// antenna; output input m = 2a+p into out (ld = column stride).
int launch_row_stage_packed4(ab_ctx* ctx, const Packed4Src& src, int nant, int nrows, int P, const FftPlan& plan,
                             const float2* twP, float* out, int64_t ld, cudaStream_t s);

// Row stage on the tensor cores (row_tc.cu): 4-bit packets, 1 <= nsel <= 64,
// P a multiple of 256, ld % 8 == 0 and a 32-byte aligned out.  The basis of
// the channel set (absolute bins kabs) comes from get_row_tc_basis (cached in
// the context; kb = K-blocks of 64 fp16).  *fault is set when a bounded wait
// runs out.
int get_row_tc_basis(ab_ctx* ctx, int P, const std::vector<int32_t>& kabs, const uint16_t** out, int* kb);
int launch_row_stage_tc(ab_ctx* ctx, const Packed4Src& src, int nant, int nrows, int P, const uint16_t* basis, int kb,
                        float* out, int64_t ld, int* fault, cudaStream_t s);

// Row stage for dense c64 rows (nslice, P/2+1): out (P, ld) for one input.
int launch_row_stage_c64(ab_ctx* ctx, const float2* dat, int64_t nslice, int P, const FftPlan& plan,
                         const float2* twP, float* out, int64_t ld, cudaStream_t s);

// Time stage, in place on ninputs columns sets of (P, ld) floats with
// nslice = N valid rows.  Filter either from a c64 table (P, N/2+1) or, when
// table == nullptr, evaluated on the fly from the window taps wtaps
// (ntap, P) float32 and thresh.
int launch_time_stage(ab_ctx* ctx, float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM,
                      const float2* twN, const float2* table, const float* wtaps, int ntap, float thresh,
                      cudaStream_t s);

// Fused PFB fold epilogue of the time stage (streaming chain).  After the
// inverse transform the CTA holds this chunk's IPFB output of one sample
// phase n; timestream row r of the chunk is IPFB row cut + r (r in
// [0, acclen)), rows r < 0 come from `state` (the previous chunk's last
// 4*osamp rows of the same column, zero before the first chunk) and rows
// >= acclen read as zero.  For blocks b in [0, nb) starting at row
// row0 + b*osamp the kernel folds ntap taps with the fine window and takes the
// osamp-point real DFT over the block's rows, writing W in the layout of
// launch_pfb_stage_a; then it stores this chunk's last 4*osamp rows to state.
struct FoldArgs {
  int O;               // osamp (4..64, power of two)
  int ntap;
  int cut;
  int acclen;
  int64_t row0;        // local row of block 0 (may be negative)
  int64_t nb;          // blocks to produce
  const float* win;    // fine window (ntap * P * O)
  float* W;            // stage-A output
  float* state;        // (ninputs, P, 4*O) tail rows, read then rewritten
};

// Time stage with the fused fold epilogue (the column is not written back).
int launch_time_fold(ab_ctx* ctx, float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM,
                     const float2* twN, const float* wtaps, int ntap, float thresh, const FoldArgs& fa,
                     const float2* tw64, cudaStream_t s);

// FIR form of the time stage (fir.cu).  Taps h_n[j], |j| <= J, of the
// reference's Wiener filter at nslice bins, FP64-derived, (P, 2J+1) float;
// J = 0 when no supported J keeps the dropped tail below 1e-7 (then the FFT
// time stage must run).  Cached in ctx per (P, nslice, ntap, thresh).
int get_fir_taps(ab_ctx* ctx, int P, int N, int ntap, float thresh, int* J, const float** taps);

// IIR form (fir.cu): per-column (g w0..g w3, a1..a3, 0, then 1/A's impulse
// response at the row tiles' state-advance lags), (P, 24) float, and the
// state-carry length IW (40 or 80; 0 when the factorisation fails or needs
// longer).  Cached in ctx per (P, ntap, thresh); ntap must be 4.
int get_iir_coeffs(ab_ctx* ctx, int P, int ntap, float thresh, int* IW, const float** coef);

struct FirArgs {
  const float* data;      // [n][t] window columns, column stride ld
  int64_t ld;
  int P, ninputs, nslice, cut, acclen;
  const float* taps;      // FIR taps (P, 2J+1) or IIR coefficients (P, 24)
  int J;                  // FIR: 32 or 64 (ignored when iir_w > 0)
  int row_tile;           // rows-per-thread class: 16 or 32
  const float* state_in;  // previous chunk's last 4*O rows (ninputs, P, 4*O)
  float* state_out;       // this chunk's last 4*O rows (the other buffer)
  const float2* tw64;
  int num_sms;            // persistent grid: CTAs per SM x num_sms
  int iir_w;              // > 0: IIR form, states carried over iir_w rows
};
// Per-device constants of the FIR time stage (call once per device).
int fir_init_device();
// Time stage by FIR over the kept rows, fused with the PFB fold (fa: O, ntap
// = 4, row0, nb, win, W; fa.cut/acclen/state unused).
int launch_fir_fold(const FirArgs& a, const FoldArgs& fa, cudaStream_t s);

// sinc-Hamming window of ntap*lblock samples in double (pfb_utils.py:4-7)
void sinc_hamming_host(int ntap, int64_t lblock, std::vector<double>& w);

}  // namespace ab
