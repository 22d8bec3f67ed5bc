// unpack.cu -- packed-baseband decode kernels: 4-bit and 1-bit unpack to c64,
// device sortpols, and make_continuous placement.
//
// 4-bit rule (albatros_analysis/src/correlations/unpacking.c:187-202): a
// nibble v maps to v-16 when v > 8, else v, so 0x8 decodes to +8.  In integer
// form that is ((v + 7) & 15) - 7, which the kernels use.
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

extern "C" int ab_unpack_1bit(const uint8_t* data, float* pol0, float* pol1, int64_t rowstart, int64_t rowend,
                              const int64_t* cols, int64_t ncols_bytes, int64_t nchan, void* stream) {
  AB_CHECK_ARG(data && pol0 && pol1 && cols, "ab_unpack_1bit: NULL pointer");
  AB_CHECK_ARG(rowstart >= 0 && rowend >= rowstart && ncols_bytes >= 0 && nchan > 1, "ab_unpack_1bit: bad sizes");
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
