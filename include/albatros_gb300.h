/*
 * albatros_gb300.h -- C-ABI of the GB300 (sm_103a) ALBATROS baseband library.
 *
 * Every compute entry point takes DEVICE pointers (plain pointers and sizes,
 * no framework types), a CUDA stream passed as `void*` (NULL = legacy default
 * stream), launches asynchronously, and returns an int status: AB_OK (0) or a
 * negative AB_ERR_* code.  Nothing ever calls exit() or prints.
 * ab_last_error() gives a human-readable detail for the calling thread.
 *
 * Complex arrays are interleaved float32 (re, im) pairs ("c64").
 *
 * Each declaration names the reference interface it replaces, as
 * path:line inside the PhilJ0ly/albatros_axion_detection project
 * (albatros_analysis/...).
 */
#ifndef ALBATROS_GB300_H
#define ALBATROS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AB_OK 0
#define AB_ERR_ARG (-1)         /* invalid argument (shape, size, alignment) */
#define AB_ERR_CUDA (-2)        /* a CUDA runtime call or launch failed */
#define AB_ERR_UNSUPPORTED (-3) /* valid but unsupported size (e.g. FFT length) */
#define AB_ERR_NOMEM (-4)       /* device allocation failed */
#define AB_ERR_STATE (-5)       /* object used in the wrong state */

typedef struct ab_ctx ab_ctx;       /* per-device tables, plans and scratch */
typedef struct ab_stream ab_stream; /* streaming unpack->IPFB->PFB->xcorr state */

/* ---- library / context ------------------------------------------------ */
int ab_version(void);
const char *ab_strerror(int code);
const char *ab_last_error(void);
/* Create a context on `device` (makes it current for the calling thread).
   Replaces the reference's per-call cuBLAS handle and cuFFT plan cache
   (albatros_analysis/src/correlations/cgemm_batch.cu:26-31,
    albatros_analysis/src/utils/pycufft.py:27-90). */
int ab_ctx_create(int device, ab_ctx **out);
int ab_ctx_destroy(ab_ctx *ctx);
/* Set (npass > 0) or clear (npass = 0) the FFT radix order used for
 * transforms of length n in this context (radices from {2,3,4,5,7,8}, applied
 * in order, product n).  Used by the autotuner (albatros_axion_detection_gb300/
 * autotune.py); a set plan replaces the built-in compile-time plan of that
 * length.  No reference counterpart: the reference delegates FFT planning to
 * cuFFT (albatros_analysis/src/utils/pycufft.cu:201-303). */
int ab_ctx_set_fft_plan(ab_ctx *ctx, int64_t n, const int32_t *radices, int64_t npass);
/* Time-axis deconvolution of streams created after this call.  Three forms
 * compute the reference's circular Wiener deconvolution:
 *  - IIR: the filter W(z)(1+t^2)/D(z) factored (FP64, Wilson's spectral
 *    factorisation) into a 4-tap FIR and causal + anti-causal 3-pole
 *    recursions, whose states are carried over 40 or 80 rows; usable when the
 *    factorisation converges and the poles decay fast enough;
 *  - FIR: a (2J+1)-tap FIR (J = 32 or 64, taps of the FP64 filter at the same
 *    nslice bins), usable when the dropped tail is below 1e-7 of the norm;
 *  - FFT: nslice-point transforms (nslice/2 must factor into 2,3,5,7).
 * IIR and FIR need the fused PFB fold (osamp >= 4, ntap = 4) and run any
 * nslice.  mode 0 (default): IIR, else FIR, else FFT; mode 1: FFT only;
 * mode 2: FFT where it runs, else IIR/FIR; mode 3: FIR, else FFT.
 * row_tile: rows-per-thread class of the IIR / FIR stages (16, the default:
 * 21 / 17 rows a thread; 32: 41 / 33; 64: 67 rows a thread for the IIR form,
 * one CTA per SM, 33 for the FIR form; 0 keeps the current value), taken by
 * streams created after the call.  No reference counterpart: the reference
 * always filters with cuFFT (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91). */
int ab_ctx_set_time_filter(ab_ctx *ctx, int32_t mode, int32_t row_tile);
/* Launch-shape options of this context (no reference counterpart; set by the
 * autotuner, albatros_axion_detection_gb300/autotune.py).
 * AB_OPT_ROW_FFTS_PER_CTA: spectra per CTA of the streaming row stage, read
 * at each push: 8 (default; 8 consecutive spectra of one input, transformed
 * in time pairs, 32-byte column stores), or 4 / 2 (both pols of 4 / 2
 * spectra, 16 / 8-byte column stores). */
#define AB_OPT_ROW_FFTS_PER_CTA 1
/* AB_OPT_COARSE_MMA_BITS: input type of the coarse correlator's tensor-core
 * MMA, 16 (default: fp16 operands, fp32 partial sums, exact) or 8 (int8
 * operands, int32 partial sums). */
#define AB_OPT_COARSE_MMA_BITS 3
/* AB_OPT_ROW_PREFETCH: 1 runs the time-paired row stage as persistent CTAs
 * that prefetch the next tile's spectrum-map rows and packet words with
 * cp.async (when at most 256 channels are selected and packet rows are
 * 4-byte multiples); 2 (default) does the same with the FFT twiddles copied
 * into shared memory once per CTA; 0 launches one CTA per tile. */
#define AB_OPT_ROW_PREFETCH 5
/* AB_OPT_COARSE_ENGINE: tensor-core path of the fp16 coarse correlator.
 * 0 (default): fifth-generation tensor cores (tcgen05.mma, accumulators in
 * tensor memory) for 9 to 32 antennas, warp-level mma.sync below; 1: always
 * warp-level mma.sync; 2: tcgen05 for any count up to 32.  Both are exact. */
#define AB_OPT_COARSE_ENGINE 6
/* AB_OPT_COARSE_TC_SLICE: time samples one CTA of the tcgen05 form sums
 * before adding into the int64 totals: 0 (default) chooses per call (about
 * four CTAs per SM), else a multiple of 64 up to 131072 (the largest for
 * which every fp32 partial sum stays an exact integer). */
#define AB_OPT_COARSE_TC_SLICE 7
/* AB_OPT_PFB_TMA: how the streaming chain's PFB band DFT fetches a tile's W
 * records: 0 (default) plain 16-byte loads into registers, one CTA per tile,
 * three per SM; 1 TMA tensor copies (cp.async.bulk.tensor) landing in the
 * CTA's FFT buffers, three CTAs per SM; 2 persistent CTAs (one per SM) that
 * fetch the next tile with TMA while transforming the current one.  The
 * arithmetic is the same (bitwise the same output).  Read at each push. */
#define AB_OPT_PFB_TMA 9
/* AB_OPT_FAULT_TEST: 1 makes the next call of the tcgen05 coarse correlator
 * test its failure path without any fault: its producers withhold their
 * first stage, so the MMA thread's bounded wait (about 2 s) runs out, the
 * call's outputs are all INT64_MIN, and the tensor memory is freed.  2 does
 * the same for the next launch of the streaming chain's tensor-core row
 * stage: its workers withhold their first item's decoded tiles, every role's
 * bounded wait runs out, the stream's fault word is set (its visibilities
 * are NaN until ab_stream_reset), and the tensor memory is freed.  The
 * setting applies to one call or launch. */
#define AB_OPT_FAULT_TEST 10
/* AB_OPT_COARSE_TC_TMA: how the tcgen05 coarse correlator (up to 16
 * antennas, contiguous 16-byte-aligned channel groups, no row lists) fetches
 * its packet bytes: 1 (default) TMA tensor copies (cp.async.bulk.tensor, a
 * box of 16 bytes x 64 samples x 16 antennas per stage) into a 4-slot ring
 * in shared memory; 0 plain 16-byte loads into registers.  Both are exact. */
#define AB_OPT_COARSE_TC_TMA 11
/* AB_OPT_ROW_TC: the streaming chain's IPFB row stage (inverse real FFT of
 * every spectrum) for 4-bit or 1-bit packets with at most 64 selected channels:
 * 1 (default) as a matrix product on the tcgen05 tensor cores (the decoded
 * levels, exact in fp16, times an FP64-built cos/sin basis split into two
 * fp16 parts, fp32 accumulation); 0 the FFT.  Taken by streams created after
 * the call. */
#define AB_OPT_ROW_TC 12
int ab_ctx_set_option(ab_ctx *ctx, int32_t option, int32_t value);

/* ---- unpacking ----------------------------------------------------------
 * ab_unpack_4bit: replaces unpack_4bit / _unpack_4bit_float_gpu
 * (albatros_analysis/src/correlations/unpacking.py:140-155,193-245; CPU
 * albatros_analysis/src/correlations/unpacking.c:155-205).
 * data: (nspec, 2*nchan) bytes; rows [rowstart,rowend); channels: device
 * int64 column indices (ncols); pol0/pol1: c64 (rowend-rowstart, ncols).
 * Nibble decode v>8 -> v-16 (0x8 -> +8). */
int ab_unpack_4bit(const uint8_t *data, float *pol0, float *pol1, int64_t rowstart, int64_t rowend,
                   const int64_t *channels, int64_t ncols, int64_t nchan, void *stream);
/* Same as ab_unpack_4bit for the contiguous channels [c0, c0+ncols) with
 * c0, ncols, nchan multiples of 4 (one 8-byte load per 4 channels). */
int ab_unpack_4bit_range(const uint8_t *data, float *pol0, float *pol1, int64_t rowstart, int64_t rowend,
                         int64_t c0, int64_t ncols, int64_t nchan, void *stream);

/* ab_unpack_1bit: replaces unpack_1bit / _unpack_1bit_float_gpu
 * (albatros_analysis/src/correlations/unpacking.py:165-191,248-302; CPU
 * albatros_analysis/src/correlations/unpacking.c:207-246).
 * data: (nspec, nchan/2) bytes; cols: device int64 byte columns (the
 * reference's channels[::2]//2), ncols_bytes of them; pol0/pol1: c64
 * (rows, 2*ncols_bytes) with even output channels from the high half-byte. */
int ab_unpack_1bit(const uint8_t *data, float *pol0, float *pol1, int64_t rowstart, int64_t rowend,
                   const int64_t *cols, int64_t ncols_bytes, int64_t nchan, void *stream);

/* ab_unpack_4bit_i8 / ab_unpack_1bit_i8: the same decodes (arguments as
 * ab_unpack_4bit / ab_unpack_1bit) into int8 complex, (re, im) byte pairs:
 * pol0/pol1 (rows, ncols, 2) int8.  The levels (-7..8 for 4-bit, +-1 for
 * 1-bit) are exact in int8; for consumers that keep small integers. */
int ab_unpack_4bit_i8(const uint8_t *data, int8_t *pol0, int8_t *pol1, int64_t rowstart, int64_t rowend,
                      const int64_t *channels, int64_t ncols, int64_t nchan, void *stream);
int ab_unpack_1bit_i8(const uint8_t *data, int8_t *pol0, int8_t *pol1, int64_t rowstart, int64_t rowend,
                      const int64_t *cols, int64_t ncols_bytes, int64_t nchan, void *stream);

/* ab_sortpols: replaces sortpols (albatros_analysis/src/correlations/unpacking.c:248-368,
 * albatros_analysis/src/correlations/unpacking.py:305-377), on the device.
 * pol0/pol1: (rowend-rowstart, ncols) bytes. bit_depth 4 or 1. */
int ab_sortpols(const uint8_t *data, uint8_t *pol0, uint8_t *pol1, int64_t rowstart, int64_t rowend,
                int64_t ncols, int64_t nchan, int bit_depth, int64_t chanstart, int64_t chanend,
                void *stream);

/* ab_hist: replaces hist_4bit / hist_1bit
 * (albatros_analysis/src/correlations/unpacking.c:7-153) behind hist
 * (albatros_analysis/src/correlations/unpacking.py:82-138), on the device.
 * data: (nspec, 2*nchan) bytes (bit_depth 4) or (nspec, nchan/2) (bit_depth
 * 1, nchan even); hist: device uint64 (2^bit_depth, nchan), overwritten:
 * hist[v][c] = number of real and imaginary levels of channel c in rows
 * [rowstart, rowend) equal to v (the raw nibble for 4-bit, the bit for
 * 1-bit), over pol0 (mode 0), pol1 (mode 1) or both (mode -1). */
int ab_hist(const uint8_t *data, uint64_t *hist, int64_t rowstart, int64_t rowend, int64_t nchan,
            int bit_depth, int mode, void *stream);

/* Baseband file ingest on the device (replaces the per-chunk host loop of
 * BasebandFileIterator.__next__, albatros_analysis/src/correlations/
 * baseband_data_classes.py:614-715, with fill_arr :16-45 and
 * get_rows_from_specnum :493-519).
 * ab_packets_to_rows: body = npkt packets of bytes_per_packet bytes (a
 *   big-endian uint32 spectrum number, then the spectra); rows = the
 *   npkt*(bytes_per_packet-4) spectra bytes, packet after packet.
 * ab_spec_map_init / _add / _finish: build spec_map (nmap int32) with
 *   spec_map[g] = the lowest row holding spectrum number start + g, or -1;
 *   _add is called once per file with its wrap-corrected per-packet
 *   spectrum numbers (device int64, npkt) and the file's first row row0. */
int ab_packets_to_rows(const uint8_t *body, int64_t npkt, int64_t bytes_per_packet, uint8_t *rows, void *stream);
int ab_spec_map_init(int32_t *spec_map, int64_t nmap, void *stream);
int ab_spec_map_add(const int64_t *specnum, int64_t npkt, int32_t spp, int64_t row0, int64_t start,
                    int32_t *spec_map, int64_t nmap, void *stream);
int ab_spec_map_finish(int32_t *spec_map, int64_t nmap, void *stream);

/* ab_make_continuous: replaces make_continuous_gpu
 * (albatros_analysis/src/correlations/baseband_data_classes.py:48-73).
 * spec: c64 (nrows, ncols); specnum: device int64 (nrows); channels: device
 * int64 absolute channel numbers (ncols); out: c64 (nspec, nchans), fully
 * written (zeros where nothing is placed). Rows go to (specnum-start) mod nspec. */
int ab_make_continuous(const float *spec, int64_t nrows, int64_t ncols, const int64_t *specnum,
                       int64_t start_specnum, const int64_t *channels, int64_t nspec, int64_t nchans,
                       float *out, void *stream);

/* ---- IPFB / PFB ---------------------------------------------------------
 * ab_get_matft: replaces get_matft (albatros_analysis/src/utils/pfb_gpu_utils.py:123-137),
 * computed directly in FP64 as a 4-term DFT per (k, f) and rounded to c64.
 * matft: c64 (lblock, nslice/2+1), lblock = 2*(nchan-1). */
int ab_get_matft(ab_ctx *ctx, float *matft, int64_t nslice, int64_t nchan, int64_t ntap, void *stream);

/* ab_calculate_filter: replaces calculate_filter
 * (albatros_analysis/src/utils/pfb_gpu_utils.py:29-36), evaluated in FP64. */
int ab_calculate_filter(const float *matft, float *filt, int64_t n, double thresh, void *stream);

/* ab_build_filter: calculate_filter(get_matft(nslice, nchan, ntap), thresh)
 * (albatros_analysis/scripts/xcorr/helper_gpu_stream_clean.py:281-292) in one
 * FP64 pass, rounded to c64 (lblock, nslice/2+1). */
int ab_build_filter(ab_ctx *ctx, float *filt, int64_t nslice, int64_t nchan, int64_t ntap, double thresh,
                    void *stream);

/* ab_ipfb: replaces cupy_ipfb(dat, filt) (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91).
 * dat: c64 (nslice, nchan); filt: c64 (lblock, nslice/2+1);
 * out: float32 (lblock, nslice) row-major, i.e. the reference's returned
 * F-ordered (nslice, lblock) transposed view.  nslice must be even, nslice/2
 * and lblock must factor into 2, 3, 5, 7. */
int ab_ipfb(ab_ctx *ctx, const float *dat, const float *filt, float *out, int64_t nslice, int64_t nchan,
            void *stream);

/* ab_pfb: replaces cupy_pfb(timestream, win, out=None, nchan, ntap)
 * (albatros_analysis/src/utils/pfb_gpu_utils.py:105-121).
 * timestream: float32, nsamp samples; win: float32 (ntap*lblock);
 * out: c64 (nblock, nchan) with nblock = nsamp/lblock - (ntap-1),
 * lblock = 2*(nchan-1) a power of two >= 64. */
int ab_pfb(ab_ctx *ctx, const float *timestream, int64_t nsamp, const float *win, int64_t nchan,
           int64_t ntap, float *out, void *stream);

/* ab_pfb_band: cupy_pfb followed by the fine-band slice [q0, q1) of
 * scripts/xcorr/helper_gpu_stream_clean.py:375-380, without forming the
 * other bins. q0, q1 multiples of osamp = lblock/4096 (lblock >= 4096).
 * out: c64 (nblock, q1-q0). */
int ab_pfb_band(ab_ctx *ctx, const float *timestream, int64_t nsamp, const float *win, int64_t nchan,
                int64_t ntap, int64_t q0, int64_t q1, float *out, void *stream);

/* ---- correlators --------------------------------------------------------
 * ab_avg_xcorr_all_ant: replaces avg_xcorr_all_ant_gpu
 * (albatros_analysis/src/correlations/correlations_gpu.py:95-121) and its
 * cublasCgemmStridedBatched call (albatros_analysis/src/correlations/cgemm_batch.cu:8-53).
 * x: c64 F-ordered (M, ntime, nfreq), M = nant*npol; out: c64 F-ordered
 * (M, M, nfreq) = sum_t x_i conj(x_j) / ntime. */
int ab_avg_xcorr_all_ant(const float *x, int64_t nant, int64_t npol, int64_t ntime, int64_t nfreq,
                         float *out, void *stream);

/* ab_xcorr_coarse_4bit: exact all-baseline coarse correlator on raw 4-bit
 * packets; the integer form of avg_xcorr_all_ant_gpu for unpacked 4-bit data
 * (albatros_analysis/src/correlations/correlations_gpu.py:95-121) and of the
 * CPU avg_xcorr_4bit family (albatros_analysis/src/correlations/correlations_cpu.c:128-271).
 * raw: nant arrays of (nspec, 2*nchan) bytes, antenna a at raw + a*ant_stride;
 * rows: optional device int32 (nant, nrows) row indices per antenna (NULL =
 * rows rowstart..rowstart+nrows-1 for every antenna); channels: device int64
 * (ncols).  Rows are split into chunks of chunk_rows (0 = one chunk).
 * out_re/out_im: int64 (nchunks, M, M, ncols), M = 2*nant, unnormalised sums
 * of Re/Im x_i conj(x_j).  Tensor cores (mma.sync s8, int32 partials flushed
 * into int64): bit-exact. */
int ab_xcorr_coarse_4bit(ab_ctx *ctx, const uint8_t *raw, int64_t ant_stride, int64_t nant, int64_t nspec,
                         int64_t nchan, int64_t rowstart, int64_t nrows, const int32_t *rows,
                         const int64_t *channels, int64_t ncols, int64_t chunk_rows, int64_t *out_re,
                         int64_t *out_im, void *stream);

/* ab_xcorr_coarse_4bit_noalloc: no counterpart in the reference.  Same
 * arguments and results as ab_xcorr_coarse_4bit without the context, for
 * callers that must not allocate device memory while they run (a service
 * that fixes its memory budget at start-up, a host whose own allocator owns
 * the device, a loop where an allocation could stall or fail).  Its partial
 * sums live in a 16 MiB buffer built into the library (held on every device
 * that loads it until exit); calls needing more scratch than that, i.e.
 * nchunks * ncols * (16*ceil(nant/4))^2 * 8 bytes, return AB_ERR_ARG.  Each
 * call made outside stream capture looks up the buffer's device address; a
 * call made during a capture reuses the last address found on that device, so
 * the first call on a device must come before any stream capture.  All calls
 * share the buffer (cleared at the start of each call), so calls that overlap
 * on the GPU race. */
int ab_xcorr_coarse_4bit_noalloc(const uint8_t *raw, int64_t ant_stride, int64_t nant, int64_t nspec, int64_t nchan,
                                 int64_t rowstart, int64_t nrows, const int32_t *rows, const int64_t *channels,
                                 int64_t ncols, int64_t chunk_rows, int64_t *out_re, int64_t *out_im, void *stream);

/* ab_avg_xcorr_4bit_pairs: device form of avg_xcorr_4bit / avg_xcorr_4bit_2ant
 * (albatros_analysis/src/correlations/correlations_cpu.c:128-271) on sortpols'd
 * 4-bit data (rows, ncol). rows0/rows1: device int32 matched row indices
 * (nmatch) or NULL for rows 0..nmatch-1. Exact int64 sums re/im (ncol). */
int ab_avg_xcorr_4bit_pairs(const uint8_t *data0, const uint8_t *data1, const int32_t *rows0,
                            const int32_t *rows1, int64_t nmatch, int64_t ncol, int64_t *re, int64_t *im,
                            void *stream);

/* ab_avg_xcorr_1bit_pairs: device form of avg_xcorr_1bit
 * (albatros_analysis/src/correlations/correlations_cpu.c:273-433) and of the
 * Van Vleck partial sums (albatros_analysis/src/correlations/correlations_cpu.c:435-638).
 * data: (rows, ncol) sortpols'd 1-bit bytes; nchan channels.
 * sums: int64 (6, nchan) = Re, Im, R0, R1, IM0, IM1 (unnormalised). */
int ab_avg_xcorr_1bit_pairs(const uint8_t *data0, const uint8_t *data1, const int32_t *rows0,
                            const int32_t *rows1, int64_t nmatch, int64_t ncol, int64_t nchan, int64_t *sums,
                            void *stream);

/* ---- streaming chain ----------------------------------------------------
 * The streaming unpack -> IPFB -> PFB(osamp) -> fine xcorr of
 * repfb_xcorr_avg (albatros_analysis/scripts/xcorr/helper_gpu_stream_clean.py:295-456),
 * with the IPFB overlap rows and the ntap-1 PFB overlap blocks kept on the
 * device between chunks.  Inputs are 4-bit or 1-bit packets of nant
 * antennas, 2 pols each (M = 2*nant inputs).
 *
 * ab_stream_create: acclen new spectra per chunk, nslice = acclen + 2*cut;
 * bits: 4 (rows of 2*nchan_raw bytes) or 1 (rows of nchan_raw/2 bytes, the
 * sign-bit format of albatros_analysis/src/correlations/unpacking.c:207-246);
 * chan_cols / chan_abs: HOST int64 arrays (nsel) of raw column index and
 * absolute channel number (0..2048) of the selected coarse channels;
 * fine band [q0, q1) (multiples of osamp); nblock fine rows per job, njobs
 * jobs (from the reference's job planner). Allocates all device state. */
int ab_stream_create(ab_ctx *ctx, int64_t nant, int64_t nchan_raw, int64_t bits, const int64_t *chan_cols,
                     const int64_t *chan_abs, int64_t nsel, int64_t acclen, int64_t cut, int64_t osamp,
                     int64_t ntap, double thresh, int64_t nblock, int64_t njobs, int64_t q0, int64_t q1,
                     ab_stream **out);
int ab_stream_destroy(ab_stream *st);
/* Reset to the state before the first chunk (zero overlap, zero vis). */
int ab_stream_reset(ab_stream *st, void *stream);
/* Push chunk `chunk` (0,1,2,... in order): raw is the device base of packets
 * (nant arrays of ant_stride bytes, rows of 2*nchan_raw bytes); spectrum
 * g (global, 0-based) of antenna a is row spec_map[a*map_stride + g] when
 * spec_map != NULL (negative = missing, zero-filled), else row g. Rows for
 * g in [chunk*acclen - 2*cut, (chunk+1)*acclen) are read.  Rows are
 * 2*nchan_raw bytes (4-bit) or nchan_raw/2 bytes (1-bit).  AB_ERR_ARG when
 * map_stride (with a map) or ant_stride / row bytes (without) is below
 * (chunk+1)*acclen; map entries must name rows inside the antenna's array. */
int ab_stream_push(ab_stream *st, const uint8_t *raw, int64_t ant_stride, const int32_t *spec_map,
                   int64_t map_stride, int64_t chunk, void *stream);
/* The last chunk: as ab_stream_push, then every remaining fine block of the
 * njobs planned jobs is produced with zero samples past the end of the stream,
 * like the reference's zero-padded final job
 * (albatros_analysis/scripts/xcorr/helper_gpu_stream_clean.py:163-167). */
int ab_stream_push_final(ab_stream *st, const uint8_t *raw, int64_t ant_stride, const int32_t *spec_map,
                         int64_t map_stride, int64_t chunk, void *stream);
/* Visibilities accumulated so far: device c64 (njobs, M, M, q1-q0), each
 * job divided by nblock once complete (the reference's /K). */
const float *ab_stream_vis(const ab_stream *st);
/* Measurement hooks (no reference counterpart; the reference times whole
 * jobs with CUDA events, scripts/xcorr/helper_gpu_stream.py:113-142):
 * ab_stream_profile(st, 1) times every stage of later pushes with CUDA events
 * (synchronising after each stage), ab_stream_stage_times() returns the
 * accumulated ms and launch counts of the 5 stages
 * (row iFFT, time-axis deconvolution, PFB fold, PFB DFT, correlate). */
int ab_stream_profile(ab_stream *st, int enable);
int ab_stream_stage_times(const ab_stream *st, double *ms, int64_t *launches);
int64_t ab_stream_kernel_launches(const ab_stream *st);
/* Shared per-push scratch (no reference counterpart; the reference's driver
 * holds one buffer set per run, helper_gpu_stream_clean.py:71-167).  A stream
 * with the fused PFB fold (osamp >= 4, ntap = 4) keeps nothing in its scratch
 * between pushes, so several streams whose pushes are serialised on one CUDA
 * stream may share one workspace.  ab_stream_workspace_bytes: bytes needed
 * (-1 when the stream cannot share).  ab_stream_set_workspace: frees the
 * stream's own scratch (after a device synchronise) and uses ws (device,
 * 256-byte aligned, caller-owned, alive until the stream is destroyed).
 * Pushes of streams sharing a workspace must not overlap in time. */
/* Half-length J of the FIR time stage this stream runs (0: another form). */
int64_t ab_stream_fir_taps(const ab_stream *st);
/* Time stage form of this stream: kind 0 = FFT, 1 = FIR (param = J),
 * 2 = IIR (param = rows over which a recursion state is carried). */
int ab_stream_time_filter(const ab_stream *st, int32_t *kind, int32_t *param);
int64_t ab_stream_workspace_bytes(const ab_stream *st);
int ab_stream_set_workspace(ab_stream *st, void *ws, int64_t bytes);

#ifdef __cplusplus
}
#endif
#endif /* ALBATROS_GB300_H */
