// api.cu -- context, status strings, twiddle tables, FFT plans, scratch.
#include <math.h>
#include <stdarg.h>
#include <string.h>

#include <cudaTypedefs.h>

#include "async.cuh"
#include "common.cuh"

namespace ab {

// The driver's tensor-map encoder, looked up once through the runtime.
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

int encode_tmap(CUtensorMap* map, CUtensorMapDataType dtype, int rank, const void* base, const uint64_t* dims,
                const uint64_t* strides, const uint32_t* box, CUtensorMapSwizzle swizzle) {
  auto fn = tmap_encoder();
  if (!fn) {
    set_error("tensor map: the driver's cuTensorMapEncodeTiled is not available");
    return AB_ERR_UNSUPPORTED;
  }
  cuuint64_t gd[3], gs[2];
  cuuint32_t bx[3], es[3] = {1, 1, 1};
  for (int i = 0; i < rank; i++) {
    gd[i] = dims[i];
    bx[i] = box[i];
  }
  for (int i = 0; i + 1 < rank; i++) gs[i] = strides[i];
  CUresult r = fn(map, dtype, (cuuint32_t)rank, const_cast<void*>(base), gd, gs, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("tensor map: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return AB_ERR_ARG;
  }
  return AB_OK;
}

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

bool make_plan(int n, FftPlan* p) {
  if (n < 1) return false;
  p->n = n;
  p->npass = 0;
  p->gscratch = nullptr;
  p->bs = BluesteinPass{};
  int m = n;
  const int order[] = {8, 4, 2, 7, 5, 3};
  // Prefer radix 8; a single leftover factor 2 or 4 is taken as radix 2/4.
  for (int r : order) {
    while (m % r == 0) {
      if (p->npass >= kMaxPasses) return false;
      p->radix[p->npass++] = r;
      m /= r;
    }
  }
  if (m != 1) return false;
  int prod = 1;
  for (int q = 0; q < p->npass; q++) {
    prod *= p->radix[q];
    p->span[q] = n / prod;
  }
  return true;
}

bool make_plan_any(int n, FftPlan* p) {
  if (make_plan(n, p)) return true;
  if (n < 1) return false;
  p->npass = 0;
  p->gscratch = nullptr;
  int m = n;
  const int order[] = {8, 4, 2, 7, 5, 3};
  for (int r : order)
    while (m % r == 0) {
      if (p->npass >= kMaxPasses) return false;
      p->radix[p->npass++] = r;
      m /= r;
    }
  for (int f = 11; (int64_t)f * f <= m; f += 2)  // the remaining prime factors, direct DFT passes
    while (m % f == 0) {
      if (p->npass >= kMaxPasses) return false;
      p->radix[p->npass++] = f;
      m /= f;
    }
  if (m > 1) {
    if (p->npass >= kMaxPasses) return false;
    p->radix[p->npass++] = m;
  }
  int prod = 1;
  for (int q = 0; q < p->npass; q++) {
    prod *= p->radix[q];
    p->span[q] = n / prod;
  }
  return true;
}

bool make_plan_from(int n, const std::vector<int>& radices, FftPlan* p) {
  if ((int)radices.size() > kMaxPasses) return false;
  p->gscratch = nullptr;
  p->bs = BluesteinPass{};
  p->n = n;
  p->npass = (int)radices.size();
  int prod = 1;
  for (int q = 0; q < p->npass; q++) {
    p->radix[q] = radices[q];
    prod *= radices[q];
    p->span[q] = n / prod;
  }
  return prod == n;
}

bool ctx_plan(ab_ctx* ctx, int n, FftPlan* p, bool* overridden) {
  if (overridden) *overridden = false;
  if (ctx) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->plan_override.find(n);
    if (it != ctx->plan_override.end()) {
      if (overridden) *overridden = true;
      return make_plan_from(n, it->second, p);
    }
  }
  return make_plan(n, p);
}

static int host_pos(const FftPlan& p, int f) {
  int pos = 0;
  for (int q = 0; q < p.npass; q++) {
    pos += (f % p.radix[q]) * p.span[q];
    f /= p.radix[q];
  }
  return pos;
}
static int host_pidx(int i) { return i + (i >> 4); }

int get_pair_table(ab_ctx* ctx, const FftPlan& p, const int2** out) {
  std::vector<int> key(p.radix, p.radix + p.npass);
  key.insert(key.begin(), p.n);
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->pair_tables.find(key);
  if (it != ctx->pair_tables.end()) {
    *out = it->second;
    return AB_OK;
  }
  const int M = p.n;
  std::vector<int2> h((size_t)M / 2 + 1);
  for (int k = 0; k <= M / 2; k++) {
    int c = (M - k) % M;
    h[(size_t)k] = make_int2(host_pidx(host_pos(p, k)), host_pidx(host_pos(p, c)));
  }
  int2* d = nullptr;
  if (cudaMalloc(&d, sizeof(int2) * h.size()) != cudaSuccess) {
    set_error("cudaMalloc of a pair table failed");
    return AB_ERR_NOMEM;
  }
  AB_CUDA(cudaMemcpy(d, h.data(), sizeof(int2) * h.size(), cudaMemcpyHostToDevice));
  ctx->pair_tables[key] = d;
  *out = d;
  return AB_OK;
}

int plan_pos(const FftPlan& p, int f) { return host_pos(p, f); }

int get_bluestein(ab_ctx* ctx, int R, BluesteinPass* out) {
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->bluestein.find(R);
    if (it != ctx->bluestein.end()) {
      *out = it->second;
      return AB_OK;
    }
  }
  BluesteinPass bs{};
  bs.R = R;
  FftPlan lp;
  int L = 2 * R - 1;
  while (!make_plan(L, &lp)) L++;  // the smallest 7-smooth length >= 2R - 1
  bs.L = L;
  bs.npass = lp.npass;
  for (int q = 0; q < kMaxPasses; q++) {
    bs.radix[q] = q < lp.npass ? lp.radix[q] : 0;
    bs.span[q] = q < lp.npass ? lp.span[q] : 0;
  }
  const double pi = 3.14159265358979323846;
  // chirp c_e = exp(-i pi e / R), e < 2R
  std::vector<float2> ch((size_t)2 * R);
  for (int e = 0; e < 2 * R; e++) ch[e] = make_float2((float)cos(pi * e / R), (float)-sin(pi * e / R));
  // b[m] = conj(c_(m^2 mod 2R)) for |m| < R, wrapped to length L; its DFT / L
  std::vector<double> br((size_t)L, 0.0), bi((size_t)L, 0.0);
  for (int m = 0; m < R; m++) {
    const int64_t e = ((int64_t)m * m) % (2 * R);
    const double c = cos(pi * (double)e / R), sn = sin(pi * (double)e / R);
    br[m] = c;
    bi[m] = sn;
    if (m > 0) {
      br[L - m] = c;
      bi[L - m] = sn;
    }
  }
  std::vector<double> cl((size_t)L), sl((size_t)L);
  for (int e = 0; e < L; e++) {
    cl[e] = cos(2.0 * pi * e / L);
    sl[e] = sin(2.0 * pi * e / L);
  }
  std::vector<float2> filt((size_t)L);
  for (int f = 0; f < L; f++) {
    double xr = 0.0, xi = 0.0;
    int64_t e = 0;
    for (int m = 0; m < L; m++) {  // sum_m b[m] exp(-2 pi i f m / L)
      xr += br[m] * cl[e] + bi[m] * sl[e];
      xi += bi[m] * cl[e] - br[m] * sl[e];
      e += f;
      if (e >= L) e -= L;
    }
    filt[(size_t)host_pos(lp, f)] = make_float2((float)(xr / L), (float)(xi / L));
  }
  const float2* twL = nullptr;
  AB_TRY(get_twiddles(ctx, L, &twL));
  float2 *dch = nullptr, *dfl = nullptr;
  if (cudaMalloc(&dch, sizeof(float2) * ch.size()) != cudaSuccess ||
      cudaMalloc(&dfl, sizeof(float2) * filt.size()) != cudaSuccess) {
    cudaFree(dch);
    set_error("Bluestein tables: device allocation failed");
    return AB_ERR_NOMEM;
  }
  AB_CUDA(cudaMemcpy(dch, ch.data(), sizeof(float2) * ch.size(), cudaMemcpyHostToDevice));
  AB_CUDA(cudaMemcpy(dfl, filt.data(), sizeof(float2) * filt.size(), cudaMemcpyHostToDevice));
  bs.chirp = dch;
  bs.filt = dfl;
  bs.twL = twL;
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->bluestein.find(R);
  if (it != ctx->bluestein.end()) {  // another thread built it meanwhile
    cudaFree(dch);
    cudaFree(dfl);
    *out = it->second;
    return AB_OK;
  }
  ctx->bluestein[R] = bs;
  *out = bs;
  return AB_OK;
}

int get_twiddles(ab_ctx* ctx, int64_t T, const float2** out) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->twiddles.find(T);
  if (it != ctx->twiddles.end()) {
    *out = it->second;
    return AB_OK;
  }
  std::vector<float2> h((size_t)T);
  // exp(-2 pi i e / T) evaluated in double precision and rounded once to
  // float; the exponent is first folded into [0, T/8] by the symmetries of
  // sin/cos so the double argument stays small.
  const double twopi = 6.283185307179586476925286766559;
  for (int64_t e = 0; e < T; e++) {
    // reduce e/T to an angle in [0, pi/4] and rebuild (c, s) by symmetry
    int64_t e8 = e * 8;  // octant = floor(8 e / T)
    int oct = (int)(e8 / T);
    int64_t rem = e8 - (int64_t)oct * T;  // in [0, T)
    double c, s;
    if (oct % 2 == 0) {
      double a = twopi * (double)rem / (8.0 * (double)T);
      c = cos(a); s = sin(a);
    } else {
      double a = twopi * (double)(T - rem) / (8.0 * (double)T);
      c = sin(a); s = cos(a);  // angle = (oct+1)*pi/4 - a
    }
    // (c, s) is (cos, sin) of the angle within the octant pair; rotate by
    // the octant's multiple of pi/2
    double cc, ss;
    switch (oct / 2) {
      case 0: cc = c; ss = s; break;
      case 1: cc = -s; ss = c; break;
      case 2: cc = -c; ss = -s; break;
      default: cc = s; ss = -c; break;
    }
    h[(size_t)e] = make_float2((float)cc, (float)(-ss));
  }
  float2* d = nullptr;
  if (cudaMalloc(&d, sizeof(float2) * (size_t)T) != cudaSuccess) {
    set_error("cudaMalloc of %lld twiddles failed", (long long)T);
    return AB_ERR_NOMEM;
  }
  AB_CUDA(cudaMemcpy(d, h.data(), sizeof(float2) * (size_t)T, cudaMemcpyHostToDevice));
  ctx->twiddles[T] = d;
  *out = d;
  return AB_OK;
}

int get_twiddle_stream(ab_ctx* ctx, int n, const std::vector<int>& radices, const float2** out) {
  std::vector<int> key = radices;
  key.insert(key.begin(), n);
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->streams.find(key);
  if (it != ctx->streams.end()) {
    *out = it->second;
    return AB_OK;
  }
  std::vector<float2> h;
  int prod = 1;
  const double twopi = 6.283185307179586476925286766559;
  for (int R : radices) {
    prod *= R;
    int S = n / prod;
    int B = R * S;
    for (int k = 1; k < R; k++)
      for (int j = 0; j < S; j++) {
        long long e = ((long long)j * k) % B;
        double a = twopi * (double)e / (double)B;
        h.push_back(make_float2((float)cos(a), (float)(-sin(a))));
      }
  }
  if (prod != n) {
    set_error("twiddle stream: radices do not multiply to %d", n);
    return AB_ERR_ARG;
  }
  float2* d = nullptr;
  size_t bytes = sizeof(float2) * (h.empty() ? 1 : h.size());
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    set_error("cudaMalloc of a twiddle stream failed");
    return AB_ERR_NOMEM;
  }
  if (!h.empty()) AB_CUDA(cudaMemcpy(d, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice));
  ctx->streams[key] = d;
  *out = d;
  return AB_OK;
}

int get_scratch(ab_ctx* ctx, int slot, size_t bytes, void** out) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto& e = ctx->scratch[slot];
  if (e.second < bytes) {
    if (e.first) cudaFree(e.first);
    e.first = nullptr;
    e.second = 0;
    if (cudaMalloc(&e.first, bytes) != cudaSuccess) {
      set_error("cudaMalloc of %zu scratch bytes failed", bytes);
      return AB_ERR_NOMEM;
    }
    e.second = bytes;
  }
  *out = e.first;
  return AB_OK;
}

}  // namespace ab

extern "C" {

int ab_version(void) { return 10000; }

const char* ab_strerror(int code) {
  switch (code) {
    case AB_OK: return "ok";
    case AB_ERR_ARG: return "invalid argument";
    case AB_ERR_CUDA: return "CUDA error";
    case AB_ERR_UNSUPPORTED: return "unsupported size";
    case AB_ERR_NOMEM: return "device allocation failed";
    case AB_ERR_STATE: return "invalid state";
    default: return "unknown status";
  }
}

const char* ab_last_error(void) { return ab::g_err; }

int ab_ctx_destroy(ab_ctx* ctx);

int ab_ctx_create(int device, ab_ctx** out) {
  AB_CHECK_ARG(out != nullptr, "ab_ctx_create: out is NULL");
  AB_CUDA(cudaSetDevice(device));
  ab_ctx* c = new ab_ctx();
  c->device = device;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete c;
    ab::set_error("cudaGetDeviceProperties: %s", cudaGetErrorString(e));
    return AB_ERR_CUDA;
  }
  c->num_sms = prop.multiProcessorCount;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  const float2* t64 = nullptr;
  int rc = ab::get_twiddles(c, 64, &t64);
  if (rc != AB_OK) {
    delete c;
    return rc;
  }
  c->tw64 = const_cast<float2*>(t64);
  rc = ab::fir_init_device();
  if (rc != AB_OK) {
    ab_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return AB_OK;
}

int ab_ctx_set_fft_plan(ab_ctx* ctx, int64_t n, const int32_t* radices, int64_t npass) {
  AB_CHECK_ARG(ctx, "ab_ctx_set_fft_plan: NULL context");
  AB_CHECK_ARG(n >= 1 && npass >= 0 && npass <= ab::kMaxPasses, "ab_ctx_set_fft_plan: bad sizes");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (npass == 0) {  // clear
    ctx->plan_override.erase((int)n);
    return AB_OK;
  }
  AB_CHECK_ARG(radices, "ab_ctx_set_fft_plan: NULL radices");
  std::vector<int> r;
  long long prod = 1;
  for (int64_t q = 0; q < npass; q++) {
    int R = radices[q];
    AB_CHECK_ARG(R == 2 || R == 3 || R == 4 || R == 5 || R == 7 || R == 8,
                 "ab_ctx_set_fft_plan: radix %d not supported (2, 3, 4, 5, 7, 8)", R);
    r.push_back(R);
    prod *= R;
  }
  AB_CHECK_ARG(prod == n, "ab_ctx_set_fft_plan: radices multiply to %lld, not %lld", prod, (long long)n);
  ctx->plan_override[(int)n] = r;
  return AB_OK;
}

int ab_ctx_set_time_filter(ab_ctx* ctx, int32_t mode, int32_t row_tile) {
  AB_CHECK_ARG(ctx, "ab_ctx_set_time_filter: NULL context");
  AB_CHECK_ARG(mode >= 0 && mode <= 3,
               "ab_ctx_set_time_filter: mode must be 0 (IIR/FIR first), 1 (FFT only), 2 (FFT first) or 3 (FIR)");
  AB_CHECK_ARG(row_tile == 0 || row_tile == 16 || row_tile == 32 || row_tile == 64,
               "ab_ctx_set_time_filter: row_tile must be 0, 16, 32 or 64");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->time_filter_mode = mode;
  if (row_tile) ctx->fir_row_tile = row_tile;
  return AB_OK;
}

int ab_ctx_set_option(ab_ctx* ctx, int32_t option, int32_t value) {
  AB_CHECK_ARG(ctx, "ab_ctx_set_option: NULL context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  switch (option) {
    case AB_OPT_ROW_FFTS_PER_CTA:
      AB_CHECK_ARG(value == 2 || value == 4 || value == 8,
                   "ab_ctx_set_option: row stage spectra per CTA must be 8 (time-paired), 4 or 2 (pol-paired)");
      ctx->row_ffts_per_cta = value;
      return AB_OK;
    case AB_OPT_ROW_PREFETCH:
      AB_CHECK_ARG(value >= 0 && value <= 2, "ab_ctx_set_option: row prefetch must be 0, 1 or 2");
      ctx->row_prefetch = value;
      return AB_OK;
    case AB_OPT_COARSE_MMA_BITS:
      AB_CHECK_ARG(value == 8 || value == 16, "ab_ctx_set_option: coarse MMA input bits must be 8 or 16");
      ctx->coarse_f16 = value == 16;
      return AB_OK;
    case AB_OPT_COARSE_ENGINE:
      AB_CHECK_ARG(value >= 0 && value <= 2,
                   "ab_ctx_set_option: coarse engine must be 0 (auto), 1 (warp-level MMA) or 2 (tcgen05)");
      ctx->coarse_engine = value;
      return AB_OK;
    case AB_OPT_PFB_TMA:
      AB_CHECK_ARG(value >= 0 && value <= 2, "ab_ctx_set_option: PFB TMA staging must be 0, 1 or 2");
      ctx->pfb_tma = value;
      return AB_OK;
    case AB_OPT_FAULT_TEST:
      AB_CHECK_ARG(value >= 0 && value <= 2, "ab_ctx_set_option: fault test must be 0, 1 or 2");
      ctx->test_withhold_stage = value;
      return AB_OK;
    case AB_OPT_COARSE_TC_TMA:
      AB_CHECK_ARG(value == 0 || value == 1, "ab_ctx_set_option: coarse TMA staging must be 0 or 1");
      ctx->coarse_tc_tma = value;
      return AB_OK;
    case AB_OPT_ROW_TC:
      AB_CHECK_ARG(value == 0 || value == 1, "ab_ctx_set_option: tensor-core row stage must be 0 or 1");
      ctx->row_tc = value;
      return AB_OK;
    case AB_OPT_COARSE_TC_SLICE:
      AB_CHECK_ARG(value >= 0 && value % 64 == 0 && value <= (1 << 17),
                   "ab_ctx_set_option: tensor-core slice must be 0 (auto) or a multiple of 64 up to 131072");
      ctx->coarse_tc_slice = value;
      return AB_OK;
    default:
      ab::set_error("ab_ctx_set_option: unknown option %d", option);
      return AB_ERR_ARG;
  }
}

int ab_ctx_destroy(ab_ctx* ctx) {
  if (!ctx) return AB_OK;
  cudaSetDevice(ctx->device);
  for (auto& kv : ctx->twiddles) cudaFree(kv.second);
  for (auto& kv : ctx->streams) cudaFree(kv.second);
  for (auto& kv : ctx->pair_tables) cudaFree(kv.second);
  for (auto& kv : ctx->bluestein) {
    cudaFree(const_cast<float2*>(kv.second.chirp));
    cudaFree(const_cast<float2*>(kv.second.filt));
  }
  for (auto& kv : ctx->fir_taps) cudaFree((void*)kv.second.second);
  for (auto& kv : ctx->row_bases) cudaFree(kv.second);
  for (auto& kv : ctx->scratch)
    if (kv.second.first) cudaFree(kv.second.first);
  delete ctx;
  return AB_OK;
}

}  // extern "C"
