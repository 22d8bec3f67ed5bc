// ingest.cu -- baseband file body -> spectrum rows and the spectrum map the
// streaming chain reads.
//
// File layout (albatros_analysis/src/correlations/baseband_data_classes.py:
// 156-216): after the header, packets of bytes_per_packet bytes, each a
// big-endian uint32 spectrum number followed by spectra_per_packet spectra of
// row_bytes bytes.  The reference copies the whole spectra block to the GPU
// and keeps the spectrum numbers on the host, expanding them per spectrum
// (fill_arr :16-45) and locating each chunk's rows with searchsorted
// (get_rows_from_specnum :493-519) inside BasebandFileIterator.__next__
// (:614-715), chunk by chunk in Python.  Here one kernel splits the file
// body into dense rows on the device and a second writes, for every spectrum
// number of the run, the row that holds it (or -1), so the chain's row stage
// gathers gaps as zeros without a host loop.
#include <algorithm>

#include "common.cuh"

namespace ab {

// rows[p*spp + j][:] = body[p][4 + j*row_bytes : 4 + (j+1)*row_bytes], as
// 32-bit words when the packet size and the body are 4-byte aligned.
__global__ void packets_to_rows_w4(const uint32_t* __restrict__ body, int64_t npkt, int64_t words_per_packet,
                                   uint32_t* __restrict__ rows) {
  const int64_t pw = words_per_packet - 1;  // payload words
  const int64_t n = npkt * pw;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / pw, w = i - p * pw;
    rows[i] = __ldg(&body[p * words_per_packet + 1 + w]);
  }
}

__global__ void packets_to_rows_b(const uint8_t* __restrict__ body, int64_t npkt, int64_t bytes_per_packet,
                                  uint8_t* __restrict__ rows) {
  const int64_t pb = bytes_per_packet - 4;
  const int64_t n = npkt * pb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / pb, b = i - p * pb;
    rows[i] = body[p * bytes_per_packet + 4 + b];
  }
}

// spec_map[g] = min over rows r holding spectrum start + g of r (row0 + p*spp + j
// for packet p's spectrum specnum[p] + j); atomicMin keeps the earliest row
// when a spectrum number repeats, as the reference's in-order reading does.
__global__ void spec_map_scatter(const int64_t* __restrict__ specnum, int64_t npkt, int spp, int64_t row0,
                                 int64_t start, int64_t nmap, int32_t* __restrict__ spec_map) {
  const int64_t n = npkt * spp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / spp, j = i - p * spp;
    const int64_t g = specnum[p] + j - start;
    if (g >= 0 && g < nmap) atomicMin(&spec_map[g], (int32_t)(row0 + i));
  }
}

__global__ void fill_i32(int32_t* __restrict__ a, int64_t n, int32_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}

__global__ void unset_to_missing(int32_t* __restrict__ a, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (a[i] == INT32_MAX) a[i] = -1;
}

static unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 8 * 152); }

}  // namespace ab

using namespace ab;

extern "C" int ab_packets_to_rows(const uint8_t* body, int64_t npkt, int64_t bytes_per_packet, uint8_t* rows,
                                  void* stream) {
  AB_CHECK_ARG(body && rows, "ab_packets_to_rows: NULL pointer");
  AB_CHECK_ARG(npkt >= 0 && bytes_per_packet > 4, "ab_packets_to_rows: bad sizes");
  if (npkt == 0) return AB_OK;
  cudaStream_t s = as_stream(stream);
  const bool w4 = bytes_per_packet % 4 == 0 && ((uintptr_t)body & 3) == 0 && ((uintptr_t)rows & 3) == 0;
  if (w4) {
    const int64_t n = npkt * (bytes_per_packet / 4 - 1);
    packets_to_rows_w4<<<grid_for(n), 256, 0, s>>>((const uint32_t*)body, npkt, bytes_per_packet / 4,
                                                   (uint32_t*)rows);
  } else {
    const int64_t n = npkt * (bytes_per_packet - 4);
    packets_to_rows_b<<<grid_for(n), 256, 0, s>>>(body, npkt, bytes_per_packet, rows);
  }
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_spec_map_init(int32_t* spec_map, int64_t nmap, void* stream) {
  AB_CHECK_ARG(spec_map && nmap >= 0, "ab_spec_map_init: bad arguments");
  if (nmap == 0) return AB_OK;
  fill_i32<<<grid_for(nmap), 256, 0, as_stream(stream)>>>(spec_map, nmap, INT32_MAX);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_spec_map_add(const int64_t* specnum, int64_t npkt, int32_t spp, int64_t row0, int64_t start,
                               int32_t* spec_map, int64_t nmap, void* stream) {
  AB_CHECK_ARG(specnum && spec_map, "ab_spec_map_add: NULL pointer");
  AB_CHECK_ARG(npkt >= 0 && spp > 0 && row0 >= 0 && nmap >= 0, "ab_spec_map_add: bad sizes");
  AB_CHECK_ARG(row0 + npkt * (int64_t)spp <= INT32_MAX, "ab_spec_map_add: row index beyond int32");
  if (npkt == 0 || nmap == 0) return AB_OK;
  spec_map_scatter<<<grid_for(npkt * spp), 256, 0, as_stream(stream)>>>(specnum, npkt, spp, row0, start, nmap,
                                                                        spec_map);
  AB_LAUNCH_CHECK();
  return AB_OK;
}

extern "C" int ab_spec_map_finish(int32_t* spec_map, int64_t nmap, void* stream) {
  AB_CHECK_ARG(spec_map && nmap >= 0, "ab_spec_map_finish: bad arguments");
  if (nmap == 0) return AB_OK;
  unset_to_missing<<<grid_for(nmap), 256, 0, as_stream(stream)>>>(spec_map, nmap);
  AB_LAUNCH_CHECK();
  return AB_OK;
}
