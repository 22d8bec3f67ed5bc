// chain.cu -- streaming unpack -> IPFB -> PFB(osamp) -> fine xcorr, the
// GB300 form of repfb_xcorr_avg
// (albatros_analysis/scripts/xcorr/helper_gpu_stream_clean.py:295-456).
//
// Per pushed chunk of acclen new spectra (all M = 2*nant inputs at once):
//   1. row stage   : decode the 4-bit (or 1-bit) packets of local rows
//                    [0, nslice) (global spectra chunk*acclen - 2cut ...)
//                    through the spectrum map, place the selected channels,
//                    P-point inverse FFT, write the [n][t] intermediate;
//   2. time stage  : per column, the Wiener deconvolution along time, in one
//                    of three forms (fir.cu, ipfb.cu): the IIR factorisation
//                    (default), a (2J+1)-tap FIR, or rfft -> filter -> irfft;
//   3. PFB stage A : tap fold + osamp-point DFT for every fine block whose
//                    ntap*osamp rows are now available;
//   4. PFB stage B : osamp fine offsets x P-point DFT, keeping only the
//                    fine band [q0, q1);
//   5. correlate   : accumulate Y_i conj(Y_j) / nblock into each block's job.
// With osamp >= 4 and ntap = 4 ("fused"), step 3 runs inside the IIR / FIR
// time stage, and the last 4*osamp timestream rows of every column are kept
// in `state` for the blocks that straddle the next chunk; otherwise the
// intermediate is a ping-pong pair (buffer chunk % 2) and step 3 reads the
// previous chunk's rows from the other buffer.
//
// The reference's overlap state (the 2*cut coarse rows carried between IPFB
// chunks and the ntap-1 fine blocks carried between PFB jobs) is realised by
// re-decoding the previous 2*cut packets in step 1 and by the carried rows
// of step 3; no packets are copied between chunks.
#include <algorithm>

#include "ipfb.cuh"
#include "pfb.cuh"

namespace ab {
int launch_xcorr_accum(const float2* Y, int M, int64_t nb, int64_t F, int64_t b_lo, int64_t b_hi, float2* vis,
                       float scale, cudaStream_t s, const int* fault);
}

using namespace ab;

struct ab_stream {
  ab_ctx* ctx = nullptr;
  int nant = 0, M = 0, P = 4096, O = 1, ntap = 4;
  int64_t nchan_raw = 0, nsel = 0, acclen = 0, cut = 0, nslice = 0;
  int64_t ld = 0;  // column stride of the [n][t] intermediate: nslice rounded up to 32 floats (128 B)
  int bits = 4;
  int64_t nblock = 0, njobs = 0, q0 = 0, q1 = 0, nq = 0;
  float thresh = 0.f;
  FftPlan planP{}, planM{};
  const float2 *twP = nullptr, *twN = nullptr, *twL = nullptr;
  int32_t *d_cols = nullptr, *d_abs = nullptr;
  float* d_wtaps = nullptr;  // IPFB filter window taps (ntap, P)
  float* d_win = nullptr;    // PFB window (ntap * L)
  float* interm[2] = {nullptr, nullptr};
  bool fused = false;        // PFB fold fused into the time stage (osamp >= 4)
  float* state = nullptr;    // fused: last 4*osamp timestream rows per column (x2 for the FIR path)
  int fir_J = 0;             // > 0: time stage as a (2J+1)-tap FIR (fir.cu)
  int iir_W = 0;             // > 0: time stage as the IIR factorisation, states carried over iir_W rows (fir.cu)
  int fir_row_tile = 16;     // rows-per-thread class of the IIR / FIR stage
  const float* fir_taps = nullptr;
  float* W = nullptr;
  float2* Y = nullptr;
  float2* vis = nullptr;
  int* d_fault = nullptr;    // set by a stage whose asynchronous copies did not arrive; vis is then NaN
  const uint16_t* row_basis = nullptr;  // tensor-core row stage: basis image of the channel set (context cache)
  int row_kb = 0;                       // its K-blocks (64 fp16 each)
  bool owns_scratch = true;  // interm[0], W, Y allocated here (not a shared workspace)
  int64_t nb_max = 0;
  int64_t chunks_done = 0;  // next chunk expected
  int64_t blocks_done = 0;  // fine blocks already correlated
  int64_t launches = 0;
  // optional per-stage timing (row, time, PFB A, PFB B, xcorr)
  bool profile = false;
  double stage_ms[5] = {0, 0, 0, 0, 0};
  int64_t stage_launches[5] = {0, 0, 0, 0, 0};
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

static void stream_free(ab_stream* st) {
  for (auto& e : st->ev)
    if (e) cudaEventDestroy(e);
  cudaFree(st->d_cols);
  cudaFree(st->d_abs);
  cudaFree(st->d_wtaps);
  cudaFree(st->d_win);
  if (st->owns_scratch) {
    cudaFree(st->interm[0]);
    cudaFree(st->W);
    cudaFree(st->Y);
  }
  cudaFree(st->interm[1]);
  cudaFree(st->state);
  cudaFree(st->vis);
  cudaFree(st->d_fault);
}

// Per-push scratch of a fused stream, as carved from one workspace: the IPFB
// intermediate, the folded fine blocks W and the band spectra Y (each region
// 256-byte aligned).  Nothing in it outlives a push.
static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
static void workspace_parts(const ab_stream* st, size_t part[3]) {
  const int64_t L = (int64_t)st->P * st->O;
  part[0] = align256(sizeof(float) * (size_t)st->M * st->P * st->ld);
  part[1] = align256(sizeof(float) * (size_t)st->M * st->nb_max * L);
  part[2] = align256(sizeof(float2) * (size_t)st->M * st->nb_max * st->nq);
}

#define AB_ALLOC(ptr, bytes)                                              \
  do {                                                                    \
    if (cudaMalloc((void**)&(ptr), (bytes)) != cudaSuccess) {             \
      set_error("ab_stream_create: cudaMalloc of %zu bytes failed", (size_t)(bytes)); \
      stream_free(st);                                                    \
      delete st;                                                          \
      return AB_ERR_NOMEM;                                                \
    }                                                                     \
  } while (0)

extern "C" int ab_stream_create(ab_ctx* ctx, int64_t nant, int64_t nchan_raw, int64_t bits, const int64_t* chan_cols,
                                const int64_t* chan_abs, int64_t nsel, int64_t acclen, int64_t cut, int64_t osamp,
                                int64_t ntap, double thresh, int64_t nblock, int64_t njobs, int64_t q0, int64_t q1,
                                ab_stream** out) {
  AB_CHECK_ARG(ctx && chan_cols && chan_abs && out, "ab_stream_create: NULL pointer");
  AB_CHECK_ARG(bits == 4 || bits == 1, "ab_stream_create: bits must be 4 or 1");
  AB_CHECK_ARG(bits == 4 || nchan_raw % 2 == 0, "ab_stream_create: 1-bit data needs an even channel count");
  AB_CHECK_ARG(nant >= 1 && nchan_raw >= 1 && nsel >= 1 && acclen >= 1 && cut >= 1 && ntap >= 1 && ntap <= 8,
               "ab_stream_create: bad sizes (cut >= 1, 1 <= ntap <= 8)");
  AB_CHECK_ARG(acclen >= 2 * cut, "ab_stream_create: acclen must be >= 2*cut");
  AB_CHECK_ARG(acclen >= ntap * osamp, "ab_stream_create: acclen must be >= ntap*osamp");
  AB_CHECK_ARG(osamp >= 1 && osamp <= 64 && (osamp & (osamp - 1)) == 0, "ab_stream_create: osamp must be 1..64, power of two");
  AB_CHECK_ARG(nblock >= 1 && njobs >= 0, "ab_stream_create: bad nblock/njobs");
  const int P = 4096;
  AB_CHECK_ARG(q0 % osamp == 0 && q1 % osamp == 0 && q0 >= 0 && q1 > q0 && q1 / osamp <= P / 2,
               "ab_stream_create: band [%lld, %lld) must be multiples of osamp inside [0, 2048*osamp]", (long long)q0,
               (long long)q1);
  for (int64_t k = 0; k < nsel; k++) {
    AB_CHECK_ARG(chan_cols[k] >= 0 && chan_cols[k] < nchan_raw, "ab_stream_create: channel column out of range");
    AB_CHECK_ARG(chan_abs[k] >= 0 && chan_abs[k] <= P / 2, "ab_stream_create: absolute channel out of range");
  }
  ab_stream* st = new ab_stream();
  st->ctx = ctx;
  st->nant = (int)nant;
  st->M = (int)(2 * nant);
  st->P = P;
  st->O = (int)osamp;
  st->ntap = (int)ntap;
  st->nchan_raw = nchan_raw;
  st->bits = (int)bits;
  st->nsel = nsel;
  st->acclen = acclen;
  st->cut = cut;
  st->nslice = acclen + 2 * cut;
  // every column starts on a 128-byte boundary whatever nslice is (the
  // reference's default cut = 10 gives nslice = acclen + 20), so the row
  // stage's 32-byte column stores and the time stage's 16-byte staging copies
  // stay aligned; rows [nslice, ld) are never written or read
  st->ld = (st->nslice + 31) / 32 * 32;
  st->nblock = nblock;
  st->njobs = njobs;
  st->q0 = q0;
  st->q1 = q1;
  st->nq = q1 - q0;
  st->thresh = (float)thresh;
  st->fused = osamp >= 4 && ntap == 4;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    st->fir_row_tile = ctx->fir_row_tile;
  }
  int mode;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    mode = ctx->time_filter_mode;
  }
  // can the FFT time stage run this nslice?
  FftPlan pm{};
  const bool fft_ok = st->nslice % 2 == 0 && ctx_plan(ctx, (int)(st->nslice / 2), &pm) &&
                      (size_t)(st->nslice / 2) * sizeof(float2) <= ctx->smem_optin;
  if (st->fused && (mode == 0 || mode == 3 || (mode == 2 && !fft_ok)) && st->nslice <= (int64_t)1 << 30) {
    int rc = AB_OK;
    if (mode != 3) rc = get_iir_coeffs(ctx, P, (int)ntap, (float)thresh, &st->iir_W, &st->fir_taps);
    if (rc == AB_OK && st->iir_W == 0)
      rc = get_fir_taps(ctx, P, (int)st->nslice, (int)ntap, (float)thresh, &st->fir_J, &st->fir_taps);
    if (rc != AB_OK) {
      delete st;
      return rc;
    }
  }
  const bool fir_path = st->fir_J > 0 || st->iir_W > 0;
  if (!ctx_plan(ctx, P, &st->planP)) {
    set_error("ab_stream_create: no FFT plan for lblock %d", P);
    delete st;
    return AB_ERR_UNSUPPORTED;
  }
  if (!fir_path && (st->nslice % 2 || !ctx_plan(ctx, (int)(st->nslice / 2), &st->planM))) {
    set_error("ab_stream_create: nslice = acclen + 2*cut = %lld must be even with nslice/2 factoring into 2,3,5,7",
              (long long)st->nslice);
    delete st;
    return AB_ERR_UNSUPPORTED;
  }
  if (!fir_path && (size_t)(st->nslice / 2) * sizeof(float2) > ctx->smem_optin) {
    set_error("ab_stream_create: nslice %lld exceeds the shared-memory column limit", (long long)st->nslice);
    delete st;
    return AB_ERR_UNSUPPORTED;
  }
  int rc;
  if ((rc = get_twiddles(ctx, P, &st->twP)) != AB_OK ||
      (!fir_path && (rc = get_twiddles(ctx, st->nslice, &st->twN)) != AB_OK) ||
      (rc = get_twiddles(ctx, (int64_t)P * osamp, &st->twL)) != AB_OK) {
    delete st;
    return rc;
  }
  const int64_t L = (int64_t)P * osamp;
  const int M = st->M;
  // largest number of fine blocks one push produces (the last push also
  // produces the zero-padded tail of the planned jobs)
  {
    int64_t done = 0, mx = 0, total = njobs * nblock;
    for (int64_t c = 0; done < total; c++) {
      int64_t be = ((c + 1) * acclen) / osamp - ntap + 1;
      if (be > total) be = total;
      if (be < done) be = done;
      mx = std::max(mx, be - done);
      done = be;
      if (c > total + 2) break;
    }
    st->nb_max = std::max<int64_t>(mx, acclen / osamp + 1);
    // the final push also completes the blocks that straddle the end of the
    // data (their taps read zeros past it); blocks that start past the end
    // are all zeros and are not produced (they add nothing to the jobs)
    st->nb_max = std::max<int64_t>(st->nb_max, acclen / osamp + ntap + 1);
  }
  AB_ALLOC(st->d_cols, sizeof(int32_t) * nsel);
  AB_ALLOC(st->d_abs, sizeof(int32_t) * nsel);
  AB_ALLOC(st->d_wtaps, sizeof(float) * ntap * P);
  AB_ALLOC(st->d_win, sizeof(float) * ntap * L);
  for (int i = 0; i < (st->fused ? 1 : 2); i++) AB_ALLOC(st->interm[i], sizeof(float) * (size_t)M * P * st->ld);
  if (st->fused) AB_ALLOC(st->state, sizeof(float) * (size_t)2 * M * P * 4 * osamp);
  AB_ALLOC(st->W, sizeof(float) * (size_t)M * st->nb_max * L);
  AB_ALLOC(st->Y, sizeof(float2) * (size_t)M * st->nb_max * st->nq);
  AB_ALLOC(st->vis, sizeof(float2) * (size_t)std::max<int64_t>(njobs, 1) * M * M * st->nq);
  AB_ALLOC(st->d_fault, sizeof(int));
  std::vector<int32_t> hc(nsel), ha(nsel);
  for (int64_t k = 0; k < nsel; k++) {
    hc[k] = (int32_t)chan_cols[k];
    ha[k] = (int32_t)chan_abs[k];
  }
  std::vector<double> w;
  sinc_hamming_host((int)ntap, P, w);  // IPFB: window of the coarse PFB (lblock 4096)
  std::vector<float> wf(w.begin(), w.end());
  sinc_hamming_host((int)ntap, L, w);  // PFB: window of the fine PFB
  std::vector<float> wl(w.begin(), w.end());
  bool ok = cudaMemcpy(st->d_cols, hc.data(), sizeof(int32_t) * nsel, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(st->d_abs, ha.data(), sizeof(int32_t) * nsel, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(st->d_wtaps, wf.data(), sizeof(float) * wf.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(st->d_win, wl.data(), sizeof(float) * wl.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemset(st->vis, 0, sizeof(float2) * (size_t)std::max<int64_t>(njobs, 1) * M * M * st->nq) == cudaSuccess &&
            cudaMemset(st->d_fault, 0, sizeof(int)) == cudaSuccess &&
            (!st->fused || cudaMemset(st->state, 0, sizeof(float) * (size_t)2 * M * P * 4 * osamp) == cudaSuccess);
  if (!ok) {
    set_error("ab_stream_create: upload failed");
    stream_free(st);
    delete st;
    return AB_ERR_CUDA;
  }
  // the row stage as a tensor-core matrix product where it applies (else the FFT)
  if (ctx->row_tc && nsel <= 64 && P % 256 == 0 &&
      get_row_tc_basis(ctx, P, ha, &st->row_basis, &st->row_kb) != AB_OK) {
    st->row_basis = nullptr;
    set_error("");
  }
  *out = st;
  return AB_OK;
}

extern "C" int ab_stream_destroy(ab_stream* st) {
  if (!st) return AB_OK;
  stream_free(st);
  delete st;
  return AB_OK;
}

extern "C" int ab_stream_reset(ab_stream* st, void* stream) {
  AB_CHECK_ARG(st, "ab_stream_reset: NULL stream object");
  st->chunks_done = 0;
  st->blocks_done = 0;
  st->launches = 0;
  AB_CUDA(cudaMemsetAsync(st->vis, 0, sizeof(float2) * (size_t)std::max<int64_t>(st->njobs, 1) * st->M * st->M * st->nq,
                          as_stream(stream)));
  if (st->fused)
    AB_CUDA(cudaMemsetAsync(st->state, 0, sizeof(float) * (size_t)2 * st->M * st->P * 4 * st->O, as_stream(stream)));
  AB_CUDA(cudaMemsetAsync(st->d_fault, 0, sizeof(int), as_stream(stream)));
  return AB_OK;
}

extern "C" int ab_stream_profile(ab_stream* st, int enable) {
  AB_CHECK_ARG(st, "ab_stream_profile: NULL stream object");
  if (enable && !st->ev[0]) {
    AB_CUDA(cudaEventCreate(&st->ev[0]));
    AB_CUDA(cudaEventCreate(&st->ev[1]));
  }
  st->profile = enable != 0;
  for (int i = 0; i < 5; i++) {
    st->stage_ms[i] = 0;
    st->stage_launches[i] = 0;
  }
  return AB_OK;
}

extern "C" int ab_stream_stage_times(const ab_stream* st, double* ms, int64_t* launches) {
  AB_CHECK_ARG(st && ms && launches, "ab_stream_stage_times: NULL pointer");
  for (int i = 0; i < 5; i++) {
    ms[i] = st->stage_ms[i];
    launches[i] = st->stage_launches[i];
  }
  return AB_OK;
}

extern "C" int64_t ab_stream_workspace_bytes(const ab_stream* st) {
  if (!st || !st->fused) return -1;
  size_t part[3];
  workspace_parts(st, part);
  return (int64_t)(part[0] + part[1] + part[2]);
}

extern "C" int ab_stream_set_workspace(ab_stream* st, void* ws, int64_t bytes) {
  AB_CHECK_ARG(st, "ab_stream_set_workspace: NULL stream object");
  if (!st->fused) {
    set_error("ab_stream_set_workspace: only streams with the fused PFB fold (osamp >= 4, ntap = 4) keep no "
              "state in their scratch");
    return AB_ERR_UNSUPPORTED;
  }
  AB_CHECK_ARG(ws && ((uintptr_t)ws & 255) == 0, "ab_stream_set_workspace: workspace must be 256-byte aligned");
  size_t part[3];
  workspace_parts(st, part);
  AB_CHECK_ARG(bytes >= (int64_t)(part[0] + part[1] + part[2]),
               "ab_stream_set_workspace: %lld bytes given, %lld needed", (long long)bytes,
               (long long)(part[0] + part[1] + part[2]));
  if (st->owns_scratch) {
    AB_CUDA(cudaDeviceSynchronize());  // no push of this stream may still use the old buffers
    cudaFree(st->interm[0]);
    cudaFree(st->W);
    cudaFree(st->Y);
  }
  char* p = (char*)ws;
  st->interm[0] = (float*)p;
  st->W = (float*)(p + part[0]);
  st->Y = (float2*)(p + part[0] + part[1]);
  st->owns_scratch = false;
  return AB_OK;
}

extern "C" const float* ab_stream_vis(const ab_stream* st) { return st ? (const float*)st->vis : nullptr; }
extern "C" int64_t ab_stream_kernel_launches(const ab_stream* st) { return st ? st->launches : -1; }
extern "C" int64_t ab_stream_fir_taps(const ab_stream* st) { return st ? st->fir_J : -1; }
extern "C" int ab_stream_time_filter(const ab_stream* st, int32_t* kind, int32_t* param) {
  AB_CHECK_ARG(st && kind && param, "ab_stream_time_filter: NULL pointer");
  *kind = st->iir_W > 0 ? 2 : st->fir_J > 0 ? 1 : 0;
  *param = st->iir_W > 0 ? st->iir_W : st->fir_J;
  return AB_OK;
}

// Stage timing (profiling mode only): events around one stage, synchronised
// immediately, so this mode serialises the host with the device.
struct StageTimer {
  ab_stream* st;
  cudaStream_t s;
  int stage;
  StageTimer(ab_stream* st_, cudaStream_t s_, int stage_) : st(st_), s(s_), stage(stage_) {
    if (st->profile) cudaEventRecord(st->ev[0], s);
  }
  void done(int nlaunch) {
    st->launches += nlaunch;
    if (!st->profile) return;
    cudaEventRecord(st->ev[1], s);
    cudaEventSynchronize(st->ev[1]);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, st->ev[0], st->ev[1]);
    st->stage_ms[stage] += ms;
    st->stage_launches[stage] += nlaunch;
  }
};

// Push chunk `chunk`.  final != 0 marks the last chunk of the stream: the
// remaining blocks of the planned jobs that hold data are then produced with
// zeros past the end (the reference's zero-padded last job,
// helper_gpu_stream_clean.py:163-167); the all-zero blocks after them add
// nothing to the visibilities and are not computed.
static int stream_push(ab_stream* st, const uint8_t* raw, int64_t ant_stride, const int32_t* spec_map,
                       int64_t map_stride, int64_t chunk, bool final, cudaStream_t s) {
  AB_CHECK_ARG(raw, "ab_stream_push: NULL raw pointer");
  AB_CHECK_ARG(chunk == st->chunks_done, "ab_stream_push: expected chunk %lld, got %lld", (long long)st->chunks_done,
               (long long)chunk);
  const int P = st->P, O = st->O, M = st->M;
  const int64_t acclen = st->acclen, cut = st->cut, nslice = st->nslice, ld = st->ld;
  // the row stage reads spectra up to (chunk+1)*acclen - 1: through the map,
  // or as raw rows when there is none
  const int64_t need = (chunk + 1) * acclen, row_bytes = st->bits == 4 ? 2 * st->nchan_raw : st->nchan_raw / 2;
  if (spec_map)
    AB_CHECK_ARG(map_stride >= need, "ab_stream_push: spectrum map of %lld entries, chunk %lld needs %lld",
                 (long long)map_stride, (long long)chunk, (long long)need);
  else
    AB_CHECK_ARG(ant_stride >= need * row_bytes, "ab_stream_push: %lld bytes per antenna, chunk %lld needs %lld",
                 (long long)ant_stride, (long long)chunk, (long long)(need * row_bytes));
  float* cur = st->fused ? st->interm[0] : st->interm[chunk & 1];
  float* prev = (!st->fused && chunk > 0) ? st->interm[(chunk - 1) & 1] : nullptr;
  // fine blocks completed by this chunk: block B needs timestream rows
  // [B*O, (B+ntap)*O); rows [0, (chunk+1)*acclen) exist after this chunk.
  const int64_t total_blocks = st->njobs * st->nblock;
  const int64_t rows_avail = (chunk + 1) * acclen;
  int64_t b_end = rows_avail / O - st->ntap + 1;  // exclusive
  // the final push completes every planned block that holds data: the
  // reference zero-pads the last job (helper_gpu_stream_clean.py:163-167);
  // blocks starting at or past the end of the data are zeros throughout, so
  // they contribute nothing to their job's visibilities and are skipped
  if (final) b_end = std::min<int64_t>(total_blocks, (rows_avail + O - 1) / O);
  if (b_end > total_blocks) b_end = total_blocks;
  if (b_end < st->blocks_done) b_end = st->blocks_done;
  const int64_t nb_all = b_end - st->blocks_done;
  const int64_t row0_all = st->blocks_done * O - chunk * acclen;  // local row of the first block
  AB_CHECK_ARG(!st->fused || nb_all <= st->nb_max, "ab_stream_push: %lld blocks exceed the buffer", (long long)nb_all);
  AB_CHECK_ARG(row0_all >= -4 * (int64_t)O || chunk == 0 || !st->fused, "ab_stream_push: block bookkeeping error");
  // 1. row stage
  Packed4Src src{raw,       ant_stride, st->bits == 4 ? 2 * st->nchan_raw : st->nchan_raw / 2,
                 spec_map,  map_stride, chunk * acclen - 2 * cut,
                 st->d_cols, st->d_abs, (int)st->nsel, st->bits};
  {
    StageTimer t(st, s, 0);
    if (st->row_basis && ld % 8 == 0 && ((uintptr_t)cur & 31) == 0)
      AB_TRY(launch_row_stage_tc(st->ctx, src, st->nant, (int)nslice, P, st->row_basis, st->row_kb, cur, ld,
                                 st->d_fault, s));
    else
      AB_TRY(launch_row_stage_packed4(st->ctx, src, st->nant, (int)nslice, P, st->planP, st->twP, cur, ld, s));
    t.done(1);
  }
  // 2. time stage (with the PFB fold fused in when osamp >= 4)
  if (st->fir_J > 0 || st->iir_W > 0) {
    StageTimer t(st, s, 1);
    const size_t half = (size_t)M * P * 4 * O;
    FirArgs fa_fir{cur, ld, P, M, (int)nslice, (int)cut, (int)acclen, st->fir_taps, st->fir_J,
                   st->fir_row_tile, st->state + (chunk & 1) * half, st->state + ((chunk + 1) & 1) * half,
                   st->ctx->tw64, st->ctx->num_sms, st->iir_W};
    FoldArgs fa{O, st->ntap, (int)cut, (int)acclen, row0_all, nb_all, st->d_win, st->W, nullptr};
    AB_TRY(launch_fir_fold(fa_fir, fa, s));
    t.done(1);
  } else if (st->fused) {
    StageTimer t(st, s, 1);
    FoldArgs fa{O, st->ntap, (int)cut, (int)acclen, row0_all, nb_all, st->d_win, st->W, st->state};
    AB_TRY(launch_time_fold(st->ctx, cur, ld, M, P, (int)nslice, st->planM, st->twN, st->d_wtaps, st->ntap,
                            st->thresh, fa, st->ctx->tw64, s));
    t.done(1);
  } else {
    StageTimer t(st, s, 1);
    AB_TRY(launch_time_stage(st->ctx, cur, ld, M, P, (int)nslice, st->planM, st->twN, nullptr, st->d_wtaps,
                             st->ntap, st->thresh, s));
    t.done(1);
  }
  st->chunks_done++;
  int64_t done = 0;
  while (done < nb_all) {
    const int64_t nb = st->fused ? nb_all : std::min(nb_all - done, st->nb_max);
    if (!st->fused) {
      const int64_t row0 = row0_all + done * O;
      TsSrc ts{cur, prev, ld, cut, cut + acclen, acclen, 0};
      StageTimer t(st, s, 2);
      AB_TRY(launch_pfb_stage_a(ts, M, P, O, st->ntap, row0, nb, st->d_win, st->W, st->ctx->tw64, s));
      t.done(1);
    }
    {
      StageTimer t(st, s, 3);
      AB_TRY(launch_pfb_stage_b(st->ctx, st->W, M, P, O, nb, st->planP, st->twL, (int)(st->q0 / O), (int)(st->q1 / O),
                                st->Y, s, st->d_fault));
      t.done(1);
    }
    // correlate, split at job boundaries
    const int64_t bfirst = st->blocks_done + done;
    int64_t b = bfirst, bend = bfirst + nb;
    StageTimer tx(st, s, 4);
    int nx = 0;
    while (b < bend) {
      int64_t job = b / st->nblock;
      int64_t jend = std::min(bend, (job + 1) * st->nblock);
      AB_TRY(launch_xcorr_accum(st->Y, M, nb, st->nq, b - bfirst, jend - bfirst,
                                st->vis + job * (int64_t)M * M * st->nq, 1.0f / (float)st->nblock, s, st->d_fault));
      nx++;
      b = jend;
    }
    tx.done(nx);
    done += nb;
  }
  st->blocks_done = b_end;
  return AB_OK;
}

extern "C" int ab_stream_push(ab_stream* st, const uint8_t* raw, int64_t ant_stride, const int32_t* spec_map,
                              int64_t map_stride, int64_t chunk, void* stream) {
  AB_CHECK_ARG(st, "ab_stream_push: NULL stream object");
  return stream_push(st, raw, ant_stride, spec_map, map_stride, chunk, false, as_stream(stream));
}

// Last chunk of a stream: also produces the zero-padded tail blocks.
extern "C" int ab_stream_push_final(ab_stream* st, const uint8_t* raw, int64_t ant_stride, const int32_t* spec_map,
                                    int64_t map_stride, int64_t chunk, void* stream) {
  AB_CHECK_ARG(st, "ab_stream_push_final: NULL stream object");
  return stream_push(st, raw, ant_stride, spec_map, map_stride, chunk, true, as_stream(stream));
}
