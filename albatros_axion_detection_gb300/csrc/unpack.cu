// unpack.cu -- packed-baseband decode kernels: 4-bit and 1-bit unpack to c64
// or int8 complex, device sortpols, make_continuous placement, and the
// quantisation histograms.
//
// 4-bit rule (albatros_analysis/src/correlations/unpacking.c:187-202): a
// nibble v maps to v-16 when v > 8, else v, so 0x8 decodes to +8.  In integer
// form that is ((v + 7) & 15) - 7, which the kernels use.
#include <algorithm>

#include "common.cuh"

namespace ab {

__device__ __forceinline__ float dec4(unsigned v) { return (float)((int)((v + 7u) & 15u) - 7); }

// One thread per (row, selected column). Output pairs are written as float4
// (pol0 and pol1 are separate arrays, each thread stores one float2 in each).
__global__ void unpack4_kernel(const uint8_t* __restrict__ data, float2* __restrict__ pol0,
                               float2* __restrict__ pol1, int64_t rowstart, int64_t nrows,
                               const int64_t* __restrict__ channels, int64_t ncols, int64_t rowbytes) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = nrows * ncols;
  if (idx >= total) return;
  int64_t r = idx / ncols, k = idx - r * ncols;
  int64_t c = __ldg(&channels[k]);
  const uint8_t* p = data + (rowstart + r) * rowbytes + 2 * c;
  uchar2 b = *reinterpret_cast<const uchar2*>(p);
  pol0[idx] = make_float2(dec4(b.x >> 4), dec4(b.x & 15u));
  pol1[idx] = make_float2(dec4(b.y >> 4), dec4(b.y & 15u));
}

// Fast path for contiguous channels [c0, c0+ncols): each thread decodes 8
// bytes (4 channels x 2 pols) from one aligned 64-bit load.
__global__ void unpack4_contig_kernel(const uint8_t* __restrict__ data, float4* __restrict__ pol0,
                                      float4* __restrict__ pol1, int64_t rowstart, int64_t nrows, int64_t c0,
                                      int64_t ncols, int64_t rowbytes) {
  int64_t q = ncols / 4;  // quads per row
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows * q) return;
  int64_t r = idx / q, j = idx - r * q;
  const uint8_t* p = data + (rowstart + r) * rowbytes + 2 * (c0 + 4 * j);
  uint2 w = *reinterpret_cast<const uint2*>(p);
  // bytes: ch0p0 ch0p1 ch1p0 ch1p1 | ch2p0 ch2p1 ch3p0 ch3p1
  unsigned b[8] = {w.x & 255u, (w.x >> 8) & 255u, (w.x >> 16) & 255u, w.x >> 24,
                   w.y & 255u, (w.y >> 8) & 255u, (w.y >> 16) & 255u, w.y >> 24};
  float4* o0 = pol0 + (r * ncols + 4 * j) / 2;
  float4* o1 = pol1 + (r * ncols + 4 * j) / 2;
  o0[0] = make_float4(dec4(b[0] >> 4), dec4(b[0] & 15u), dec4(b[2] >> 4), dec4(b[2] & 15u));
  o0[1] = make_float4(dec4(b[4] >> 4), dec4(b[4] & 15u), dec4(b[6] >> 4), dec4(b[6] & 15u));
  o1[0] = make_float4(dec4(b[1] >> 4), dec4(b[1] & 15u), dec4(b[3] >> 4), dec4(b[3] & 15u));
  o1[1] = make_float4(dec4(b[5] >> 4), dec4(b[5] & 15u), dec4(b[7] >> 4), dec4(b[7] & 15u));
}

// 1-bit: byte column col holds channels 2j, 2j+1; bits MSB first
// r0c0 i0c0 r1c0 i1c0 r0c1 i0c1 r1c1 i1c1 (unpacking.py:177-189).
__global__ void unpack1_kernel(const uint8_t* __restrict__ data, float4* __restrict__ pol0,
                               float4* __restrict__ pol1, int64_t rowstart, int64_t nrows,
                               const int64_t* __restrict__ cols, int64_t nbytes_sel, int64_t rowbytes) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows * nbytes_sel) return;
  int64_t r = idx / nbytes_sel, j = idx - r * nbytes_sel;
  unsigned b = data[(rowstart + r) * rowbytes + __ldg(&cols[j])];
#define PM1(s) ((float)((int)(((b) >> (s)) & 1u) * 2 - 1))
  pol0[idx] = make_float4(PM1(7), PM1(6), PM1(3), PM1(2));
  pol1[idx] = make_float4(PM1(5), PM1(4), PM1(1), PM1(0));
#undef PM1
}

// Int8-complex outputs (re, im as a char2 per value; the 4-bit levels -7..8
// and the 1-bit +-1 fit exactly), for consumers that keep small integers.
__device__ __forceinline__ signed char dec4i(unsigned v) { return (signed char)((int)((v + 7u) & 15u) - 7); }

__global__ void unpack4_i8_kernel(const uint8_t* __restrict__ data, char2* __restrict__ pol0, char2* __restrict__ pol1,
                                  int64_t rowstart, int64_t nrows, const int64_t* __restrict__ channels, int64_t ncols,
                                  int64_t rowbytes) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows * ncols) return;
  const int64_t r = idx / ncols, k = idx - r * ncols;
  const uchar2 b = *reinterpret_cast<const uchar2*>(data + (rowstart + r) * rowbytes + 2 * __ldg(&channels[k]));
  pol0[idx] = make_char2(dec4i(b.x >> 4), dec4i(b.x & 15u));
  pol1[idx] = make_char2(dec4i(b.y >> 4), dec4i(b.y & 15u));
}

__global__ void unpack1_i8_kernel(const uint8_t* __restrict__ data, char4* __restrict__ pol0, char4* __restrict__ pol1,
                                  int64_t rowstart, int64_t nrows, const int64_t* __restrict__ cols, int64_t nbytes_sel,
                                  int64_t rowbytes) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows * nbytes_sel) return;
  const int64_t r = idx / nbytes_sel, j = idx - r * nbytes_sel;
  const unsigned b = data[(rowstart + r) * rowbytes + __ldg(&cols[j])];
#define PM1I(s) ((signed char)((int)(((b) >> (s)) & 1u) * 2 - 1))
  pol0[idx] = make_char4(PM1I(7), PM1I(6), PM1I(3), PM1I(2));  // channels 2j, 2j+1 of pol0
  pol1[idx] = make_char4(PM1I(5), PM1I(4), PM1I(1), PM1I(0));
#undef PM1I
}

// Device sortpols (unpacking.c:248-368). One thread per output byte.
__global__ void sortpols_kernel(const uint8_t* __restrict__ data, uint8_t* __restrict__ pol0,
                                uint8_t* __restrict__ pol1, int64_t rowstart, int64_t nrows, int64_t ncols,
                                int64_t nchan, int bits, int64_t chanstart, int64_t chanend) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows * ncols) return;
  int64_t i = idx / ncols, j = idx - i * ncols;
  if (bits == 4) {
    int64_t k = chanstart + j;
    uint8_t a = 0, b = 0;
    if (k < chanend) {
      const uint8_t* p = data + (i + rowstart) * 2 * nchan + 2 * k;
      a = p[0];
      b = p[1];
    }
    pol0[idx] = a;
    pol1[idx] = b;
    return;
  }
  const uint8_t* row = data + (i + rowstart) * (nchan / 2) + chanstart / 2;
  int64_t left = (chanend - chanstart) - 4 * j;
  int nch = left >= 4 ? 4 : (int)left;
  unsigned p0 = 0, p1 = 0;
  for (int c = 0; c < nch; c++) {
    unsigned byte = row[2 * j + c / 2];
    unsigned v = (byte >> ((c & 1) ? 0 : 4)) & 15u;
    p0 |= ((v >> 2) & 3u) << (6 - 2 * c);
    p1 |= (v & 3u) << (6 - 2 * c);
  }
  pol0[idx] = (uint8_t)p0;
  pol1[idx] = (uint8_t)p1;
}

__global__ void fill_zero_kernel(float4* __restrict__ out, int64_t n4) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n4; i += stride) out[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void place_kernel(const float2* __restrict__ spec, int64_t nrows, int64_t ncols,
                             const int64_t* __restrict__ specnum, int64_t start, const int64_t* __restrict__ channels,
                             int64_t nspec, int64_t nchans, float2* __restrict__ out) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrows * ncols) return;
  int64_t r = idx / ncols, k = idx - r * ncols;
  int64_t row = (specnum[r] - start) % nspec;
  if (row < 0) row += nspec;
  out[row * nchans + channels[k]] = spec[idx];
}


// ---------------------------------------------------------------------------
// Quantisation histograms (hist_4bit / hist_1bit,
// albatros_analysis/src/correlations/unpacking.c:7-153): hist[bin][c] counts
// the real and imaginary levels of channel c (pol0, pol1 or both), a 4-bit
// level at its raw nibble (bins 0..15), a 1-bit level at its bit (bins 0, 1).
// One thread per (channel or byte column, row phase); CTAs cover a slab of
// rows, so the reads of a warp are a contiguous piece of each row.
constexpr int kHistTC = 128, kHistRY = 2;

// 4-bit: per-CTA 32-bit counters in shared memory, [bin][column in tile]
// (lanes on consecutive columns never share a bank), added into the 64-bit
// global histogram once per CTA.
__global__ void __launch_bounds__(kHistTC* kHistRY)
    hist4_kernel(const uint8_t* __restrict__ data, int64_t row_bytes, int64_t rowstart, int64_t nrows, int nchan,
                 int mode, int64_t rows_per_cta, unsigned long long* __restrict__ hist) {
  __shared__ unsigned sh[16 * kHistTC];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kHistTC + tx;
  for (int i = tid; i < 16 * kHistTC; i += kHistTC * kHistRY) sh[i] = 0u;
  __syncthreads();
  const int c = blockIdx.x * kHistTC + tx;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per_cta;
  const int64_t r1 = min(nrows, r0 + rows_per_cta);
  if (c < nchan) {
    const uint8_t* p = data + (rowstart + r0 + ty) * row_bytes + 2 * c;
#pragma unroll 4
    for (int64_t r = r0 + ty; r < r1; r += kHistRY, p += kHistRY * row_bytes) {
      const uchar2 b = *reinterpret_cast<const uchar2*>(p);  // pol0 byte, pol1 byte
      if (mode != 1) {
        atomicAdd(&sh[(b.x >> 4) * kHistTC + tx], 1u);
        atomicAdd(&sh[(b.x & 15) * kHistTC + tx], 1u);
      }
      if (mode != 0) {
        atomicAdd(&sh[(b.y >> 4) * kHistTC + tx], 1u);
        atomicAdd(&sh[(b.y & 15) * kHistTC + tx], 1u);
      }
    }
  }
  __syncthreads();
  if (c < nchan)
    for (int bin = ty; bin < 16; bin += kHistRY) {
      const unsigned v = sh[bin * kHistTC + tx];
      if (v) atomicAdd(&hist[(int64_t)bin * nchan + c], (unsigned long long)v);
    }
}

// 1-bit: byte j of a row holds channels 2j (bits 7..4: r pol0, i pol0,
// r pol1, i pol1) and 2j+1 (bits 3..0, same order); each thread counts the
// set bits of its column's two channels in registers.
__global__ void __launch_bounds__(kHistTC* kHistRY)
    hist1_kernel(const uint8_t* __restrict__ data, int64_t row_bytes, int64_t rowstart, int64_t nrows, int ncols,
                 int mode, int64_t rows_per_cta, unsigned long long* __restrict__ hist) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int j = blockIdx.x * kHistTC + tx;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per_cta;
  const int64_t r1 = min(nrows, r0 + rows_per_cta);
  if (j >= ncols || r0 + ty >= r1) return;
  const unsigned m0 = mode == 0 ? 0xC0u : mode == 1 ? 0x30u : 0xF0u;  // channel 2j's bits
  const unsigned m1 = m0 >> 4;                                        // channel 2j+1's bits
  unsigned ones0 = 0, ones1 = 0;
  const uint8_t* p = data + (rowstart + r0 + ty) * row_bytes + j;
  int64_t rows = 0;
#pragma unroll 4
  for (int64_t r = r0 + ty; r < r1; r += kHistRY, p += kHistRY * row_bytes) {
    const unsigned b = *p;
    ones0 += __popc(b & m0);
    ones1 += __popc(b & m1);
    rows++;
  }
  const unsigned long long levels = (unsigned long long)rows * (mode == -1 ? 4u : 2u);
  const int nchan = 2 * ncols;
  atomicAdd(&hist[nchan + 2 * j], (unsigned long long)ones0);
  atomicAdd(&hist[nchan + 2 * j + 1], (unsigned long long)ones1);
  atomicAdd(&hist[2 * j], levels - ones0);
  atomicAdd(&hist[2 * j + 1], levels - ones1);
}

static int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n <= 0)
      n = 1;
  }
  return n;
}
}  // namespace ab

using namespace ab;

extern "C" int ab_unpack_4bit(const uint8_t* data, float* pol0, float* pol1, int64_t rowstart, int64_t rowend,
                              const int64_t* channels, int64_t ncols, int64_t nchan, void* stream) {
  AB_CHECK_ARG(data && pol0 && pol1 && channels, "ab_unpack_4bit: NULL pointer");
  AB_CHECK_ARG(rowstart >= 0 && rowend >= rowstart && ncols >= 0 && nchan > 0, "ab_unpack_4bit: bad sizes");
  int64_t nrows = rowend - rowstart;
  int64_t total = nrows * ncols;
  if (total == 0) return AB_OK;
  int64_t blocks = (total + 255) / 256;
  unpack4_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(data, (float2*)pol0, (float2*)pol1, rowstart,
                                                                   nrows, channels, ncols, 2 * nchan);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

// Contiguous-channel variant used by the Python layer when channels form a
// range starting at a multiple of 4 and every row is 8-byte aligned.
extern "C" int ab_unpack_4bit_range(const uint8_t* data, float* pol0, float* pol1, int64_t rowstart,
                                    int64_t rowend, int64_t c0, int64_t ncols, int64_t nchan, void* stream) {
  AB_CHECK_ARG(data && pol0 && pol1, "ab_unpack_4bit_range: NULL pointer");
  AB_CHECK_ARG(ncols % 4 == 0 && c0 % 4 == 0 && nchan % 4 == 0 && ((uintptr_t)data & 7) == 0,
               "ab_unpack_4bit_range: needs 4-aligned channel range and 8-byte aligned rows");
  AB_CHECK_ARG(((uintptr_t)pol0 & 15) == 0 && ((uintptr_t)pol1 & 15) == 0, "ab_unpack_4bit_range: outputs must be 16-byte aligned");
  int64_t nrows = rowend - rowstart;
  int64_t total = nrows * (ncols / 4);
  if (total <= 0) return AB_OK;
  unpack4_contig_kernel<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
      data, (float4*)pol0, (float4*)pol1, rowstart, nrows, c0, ncols, 2 * nchan);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_unpack_4bit_i8(const uint8_t* data, int8_t* pol0, int8_t* pol1, int64_t rowstart, int64_t rowend,
                                 const int64_t* channels, int64_t ncols, int64_t nchan, void* stream) {
  AB_CHECK_ARG(data && pol0 && pol1 && channels, "ab_unpack_4bit_i8: NULL pointer");
  AB_CHECK_ARG(rowstart >= 0 && rowend >= rowstart && ncols >= 0 && nchan > 0, "ab_unpack_4bit_i8: bad sizes");
  AB_CHECK_ARG(((uintptr_t)data & 1) == 0 && ((uintptr_t)pol0 & 1) == 0 && ((uintptr_t)pol1 & 1) == 0,
               "ab_unpack_4bit_i8: buffers must be 2-byte aligned");
  const int64_t total = (rowend - rowstart) * ncols;
  if (total == 0) return AB_OK;
  unpack4_i8_kernel<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
      data, (char2*)pol0, (char2*)pol1, rowstart, rowend - rowstart, channels, ncols, 2 * nchan);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_unpack_1bit_i8(const uint8_t* data, int8_t* pol0, int8_t* pol1, int64_t rowstart, int64_t rowend,
                                 const int64_t* cols, int64_t ncols_bytes, int64_t nchan, void* stream) {
  AB_CHECK_ARG(data && pol0 && pol1 && cols, "ab_unpack_1bit_i8: NULL pointer");
  AB_CHECK_ARG(rowstart >= 0 && rowend >= rowstart && ncols_bytes >= 0 && nchan > 1 && nchan % 2 == 0,
               "ab_unpack_1bit_i8: bad sizes (1-bit rows hold an even channel count)");
  AB_CHECK_ARG(((uintptr_t)pol0 & 3) == 0 && ((uintptr_t)pol1 & 3) == 0, "ab_unpack_1bit_i8: outputs must be 4-byte aligned");
  const int64_t total = (rowend - rowstart) * ncols_bytes;
  if (total == 0) return AB_OK;
  unpack1_i8_kernel<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
      data, (char4*)pol0, (char4*)pol1, rowstart, rowend - rowstart, cols, ncols_bytes, nchan / 2);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_unpack_1bit(const uint8_t* data, float* pol0, float* pol1, int64_t rowstart, int64_t rowend,
                              const int64_t* cols, int64_t ncols_bytes, int64_t nchan, void* stream) {
  AB_CHECK_ARG(data && pol0 && pol1 && cols, "ab_unpack_1bit: NULL pointer");
  AB_CHECK_ARG(rowstart >= 0 && rowend >= rowstart && ncols_bytes >= 0 && nchan > 1 && nchan % 2 == 0,
               "ab_unpack_1bit: bad sizes (1-bit rows hold an even channel count)");
  AB_CHECK_ARG(((uintptr_t)pol0 & 15) == 0 && ((uintptr_t)pol1 & 15) == 0, "ab_unpack_1bit: outputs must be 16-byte aligned");
  int64_t nrows = rowend - rowstart;
  int64_t total = nrows * ncols_bytes;
  if (total == 0) return AB_OK;
  unpack1_kernel<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
      data, (float4*)pol0, (float4*)pol1, rowstart, nrows, cols, ncols_bytes, nchan / 2);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_sortpols(const uint8_t* data, uint8_t* pol0, uint8_t* pol1, int64_t rowstart, int64_t rowend,
                           int64_t ncols, int64_t nchan, int bit_depth, int64_t chanstart, int64_t chanend,
                           void* stream) {
  AB_CHECK_ARG(data && pol0 && pol1, "ab_sortpols: NULL pointer");
  AB_CHECK_ARG(bit_depth == 1 || bit_depth == 4, "ab_sortpols: bit_depth must be 1 or 4");
  AB_CHECK_ARG(chanstart >= 0 && chanend <= nchan && chanend > chanstart, "ab_sortpols: bad channel range");
  AB_CHECK_ARG(bit_depth == 4 || chanstart % 2 == 0, "ab_sortpols: 1-bit start channel must be even");
  int64_t nrows = rowend - rowstart;
  int64_t total = nrows * ncols;
  if (total <= 0) return AB_OK;
  sortpols_kernel<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
      data, pol0, pol1, rowstart, nrows, ncols, nchan, bit_depth, chanstart, chanend);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_make_continuous(const float* spec, int64_t nrows, int64_t ncols, const int64_t* specnum,
                                  int64_t start_specnum, const int64_t* channels, int64_t nspec, int64_t nchans,
                                  float* out, void* stream) {
  AB_CHECK_ARG(spec && specnum && channels && out, "ab_make_continuous: NULL pointer");
  AB_CHECK_ARG(nspec > 0 && nchans > 0 && nrows >= 0 && ncols >= 0, "ab_make_continuous: bad sizes");
  AB_CHECK_ARG(((uintptr_t)out & 15) == 0, "ab_make_continuous: out must be 16-byte aligned");
  cudaStream_t s = as_stream(stream);
  int64_t n = nspec * nchans * 2;  // floats
  if (n % 4 == 0) {
    fill_zero_kernel<<<1184, 256, 0, s>>>((float4*)out, n / 4);
  } else {
    AB_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * (size_t)n, s));
  }
  AB_LAUNCH_CHECK();
  int64_t total = nrows * ncols;
  if (total > 0) {
    place_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>((const float2*)spec, nrows, ncols, specnum,
                                                                  start_specnum, channels, nspec, nchans,
                                                                  (float2*)out);
    AB_LAUNCH_CHECK();
  }
  return AB_OK;
}

extern "C" int ab_hist(const uint8_t* data, uint64_t* hist, int64_t rowstart, int64_t rowend, int64_t nchan,
                       int bit_depth, int mode, void* stream) {
  AB_CHECK_ARG(data && hist, "ab_hist: NULL pointer");
  AB_CHECK_ARG(bit_depth == 1 || bit_depth == 4, "ab_hist: bit_depth must be 1 or 4");
  AB_CHECK_ARG(mode == 0 || mode == 1 || mode == -1, "ab_hist: mode must be 0, 1 or -1");
  AB_CHECK_ARG(nchan > 0 && nchan <= (1 << 30) && rowstart >= 0 && rowend >= rowstart, "ab_hist: bad sizes");
  AB_CHECK_ARG(bit_depth == 4 || nchan % 2 == 0, "ab_hist: 1-bit data needs an even channel count");
  AB_CHECK_ARG(bit_depth == 1 || ((uintptr_t)data & 1) == 0, "ab_hist: 4-bit data must be 2-byte aligned");
  cudaStream_t s = as_stream(stream);
  const int64_t nbins = bit_depth == 4 ? 15 : 1;
  AB_CUDA(cudaMemsetAsync(hist, 0, sizeof(uint64_t) * (size_t)((nbins + 1) * nchan), s));
  const int64_t nrows = rowend - rowstart;
  if (nrows == 0) return AB_OK;
  const int64_t cols = bit_depth == 4 ? nchan : nchan / 2;  // thread columns
  const int64_t gx = (cols + kHistTC - 1) / kHistTC;
  AB_CHECK_ARG(gx <= 65535, "ab_hist: too many channels");
  // about 8 CTAs per SM, each at least 256 rows
  const int64_t want = std::max<int64_t>(1, (8 * (int64_t)sm_count() + gx - 1) / gx);
  const int64_t gy = std::min<int64_t>(std::min<int64_t>(want, (nrows + 255) / 256), 65535);
  const int64_t rows_per = (nrows + gy - 1) / gy;
  AB_CHECK_ARG(rows_per < (1LL << 29), "ab_hist: too many rows per CTA");
  const dim3 grid((unsigned)gx, (unsigned)((nrows + rows_per - 1) / rows_per)), block(kHistTC, kHistRY);
  if (bit_depth == 4)
    hist4_kernel<<<grid, block, 0, s>>>(data, 2 * nchan, rowstart, nrows, (int)nchan, mode, rows_per,
                                        reinterpret_cast<unsigned long long*>(hist));
  else
    hist1_kernel<<<grid, block, 0, s>>>(data, nchan / 2, rowstart, nrows, (int)(nchan / 2), mode, rows_per,
                                        reinterpret_cast<unsigned long long*>(hist));
  AB_LAUNCH_CHECK();
  return AB_OK;
}
