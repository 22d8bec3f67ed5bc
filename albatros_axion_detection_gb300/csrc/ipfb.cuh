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
  int64_t row_bytes;         // 2 * nchan_raw
  const int32_t* spec_map;   // optional: raw row of global spectrum g (or <0)
  int64_t map_stride;        // per-antenna stride of spec_map
  int64_t g0;                // global spectrum of local row 0 (may be negative)
  const int32_t* chan_cols;  // device (nsel): raw column per selected channel
  const int32_t* chan_abs;   // device (nsel): absolute bin 0..P/2
  int nsel;
};

// Row stage for packed 4-bit input: local rows t in [0, nrows) of every
// antenna; output input m = 2a+p into out (ld = column stride).
int launch_row_stage_packed4(const Packed4Src& src, int nant, int nrows, int P, const FftPlan& plan,
                             const float2* twP, float* out, int64_t ld, cudaStream_t s);

// Row stage for dense c64 rows (nslice, P/2+1): out (P, ld) for one input.
int launch_row_stage_c64(const float2* dat, int64_t nslice, int P, const FftPlan& plan, const float2* twP,
                         float* out, int64_t ld, cudaStream_t s);

// Time stage, in place on ninputs columns sets of (P, ld) floats with
// nslice = N valid rows.  Filter either from a c64 table (P, N/2+1) or, when
// table == nullptr, evaluated on the fly from the window taps wtaps
// (ntap, P) float32 and thresh.
int launch_time_stage(float* buf, int64_t ld, int ninputs, int P, int N, const FftPlan& planM,
                      const float2* twN, const float2* table, const float* wtaps, int ntap, float thresh,
                      size_t smem_optin, cudaStream_t s);

// sinc-Hamming window of ntap*lblock samples in double (pfb_utils.py:4-7)
void sinc_hamming_host(int ntap, int64_t lblock, std::vector<double>& w);

}  // namespace ab
