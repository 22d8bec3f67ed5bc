// common.cuh -- status codes, error capture, the library context (twiddle
// tables, FFT plans, grow-only scratch) shared by all translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/albatros_gb300.h"
#include "fft.cuh"

namespace ab {

// thread-local detail message for the last failing call
void set_error(const char* fmt, ...);

#define AB_CHECK_ARG(cond, ...)        \
  do {                                 \
    if (!(cond)) {                     \
      ::ab::set_error(__VA_ARGS__);    \
      return AB_ERR_ARG;               \
    }                                  \
  } while (0)

#define AB_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      ::ab::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                      __LINE__);                                                       \
      return AB_ERR_CUDA;                                                              \
    }                                                                                  \
  } while (0)

#define AB_LAUNCH_CHECK()                                                                 \
  do {                                                                                    \
    cudaError_t e_ = cudaGetLastError();                                                  \
    if (e_ != cudaSuccess) {                                                              \
      ::ab::set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, \
                      __LINE__);                                                          \
      return AB_ERR_CUDA;                                                                 \
    }                                                                                     \
  } while (0)

#define AB_TRY(expr)          \
  do {                        \
    int rc_ = (expr);         \
    if (rc_ != AB_OK) return rc_; \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Factorise n into supported radices (8, 4, 2, 7, 5, 3). Returns false if n
// has another prime factor.
bool make_plan(int n, FftPlan* p);
// Any length: the factors 2, 3, 4, 5, 7, 8 as register passes, every other
// prime factor as a direct DFT pass (needs FftPlan::gscratch at launch).
bool make_plan_any(int n, FftPlan* p);
// The Bluestein pass of prime radix R (cached per context): convolution
// length L (the smallest 7-smooth length >= 2R - 1), L's plan, the chirp,
// the filter spectrum (FP64 on the host, rounded once) and L's twiddles.
int get_bluestein(ab_ctx* ctx, int R, BluesteinPass* out);
// Storage position of frequency f after the forward passes of plan p.
int plan_pos(const FftPlan& p, int f);
// True when the plan has a direct DFT pass.
inline bool plan_has_generic(const FftPlan& p) {
  for (int q = 0; q < p.npass; q++) {
    const int r = p.radix[q];
    if (r != 2 && r != 3 && r != 4 && r != 5 && r != 7 && r != 8) return true;
  }
  return false;
}

}  // namespace ab

// The opaque context of the C-ABI.
struct ab_ctx {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  std::mutex mu;
  // twiddle tables exp(-2 pi i e / T), e in [0, T), keyed by T
  std::map<int64_t, float2*> twiddles;
  std::map<std::vector<int>, float2*> streams;
  std::map<std::vector<int>, int2*> pair_tables;
  std::map<int, ab::BluesteinPass> bluestein;  // keyed by the prime radix
  std::map<std::vector<int>, uint16_t*> row_bases;  // tensor-core row stage: basis image per (P, channel bins)
  // FFT plans chosen by the autotuner: length -> radix order (forces the
  // runtime-plan kernels for that length)
  std::map<int, std::vector<int>> plan_override;
  // FIR taps of the time stage keyed by (P, nslice, ntap, thresh bits):
  // (J, device (P, 2J+1) floats or null when J = 0)
  std::map<std::vector<int64_t>, std::pair<int, const float*>> fir_taps;
  // 0: IIR, else FIR, else FFT, the first that is accurate (default);
  // 1: always FFT; 2: FFT where it runs, else IIR/FIR; 3: FIR, else FFT
  int time_filter_mode = 0;
  int fir_row_tile = 16;     // rows-per-thread class of the IIR / FIR time stage (16: 21 / 17 rows)
  int row_prefetch = 2;      // time-paired row stage: persistent + prefetch (1), + shared twiddles (2), one CTA per tile (0)
  bool coarse_f16 = true;    // coarse correlator on fp16 (exact) instead of int8 tensor-core MMA
  int coarse_engine = 0;     // fp16 coarse correlator: 0 = tcgen05 from 9 antennas up, 1 = warp-level mma.sync, 2 = tcgen05
  int coarse_tc_slice = 0;   // samples per CTA of the tcgen05 form (0: chosen per call)
  int coarse_tc_tma = 1;     // tcgen05 form: packet bytes staged by TMA (1) or loaded into registers (0)
  int row_tc = 1;            // streaming row stage on the tensor cores where it applies (1) or the FFT (0)
  int test_withhold_stage = 0;  // failure-path test: 1 the next tcgen05 correlator call, 2 the next tensor-core
                                // row-stage launch, withholds its first stage
  int pfb_tma = 0;           // streaming PFB band DFT: plain loads (0), TMA into the FFT buffers (1), persistent TMA (2)
  int row_ffts_per_cta = 8;  // row stage: 8 = time-paired spectra of one input per CTA;
                             // 4 or 2 = pol-paired spectra of one antenna per CTA
  // grow-only scratch buffers keyed by slot
  std::map<int, std::pair<void*, size_t>> scratch;
  float2* tw64 = nullptr;  // exp(-2 pi i e / 64)
};

namespace ab {
// Device twiddle table of length T (cached in ctx; uploaded synchronously on
// first use, so call outside stream capture).
int get_twiddles(ab_ctx* ctx, int64_t T, const float2** out);
// Device twiddle stream of a plan (radices applied in order), cached in ctx:
// stream_q[(k-1) S_q + j] = exp(-2 pi i j k / (R_q S_q)), q = 0..npass-1.
int get_twiddle_stream(ab_ctx* ctx, int n, const std::vector<int>& radices, const float2** out);
// Plan of length n for this context: the tuned override if one is set,
// else the default factorisation.  *overridden tells whether it was tuned.
bool ctx_plan(ab_ctx* ctx, int n, FftPlan* p, bool* overridden = nullptr);
// Factorise n with the given radix order (for plans whose order matters).
bool make_plan_from(int n, const std::vector<int>& radices, FftPlan* p);
// Device table of the real-FFT untangle pairs of a plan of M points: for
// k in [0, M/2], (pidx(pos(k)), pidx(pos(M-k))) where pos is the storage
// position after the forward DIF and pidx the padded shared-memory index.
int get_pair_table(ab_ctx* ctx, const FftPlan& p, const int2** out);
// Grow-only device scratch; the pointer stays valid until a larger request
// for the same slot.
int get_scratch(ab_ctx* ctx, int slot, size_t bytes, void** out);
// Per-device constant tables of the FIR time stage (fir.cu).
int fir_init_device();
enum ScratchSlot { kScratchPfbW = 1, kScratchXcorrG = 2, kScratchChain = 3, kScratchYband = 4, kScratchFault = 5,
                  kScratchDftPass = 6 };
}  // namespace ab
