/*
 * albatros_oracle.c -- CPU restatement of the ALBATROS packed-baseband
 * arithmetic, used ONLY as a test oracle and as the timed CPU baseline.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only
 * as the checker or the CPU baseline. The product path
 * (albatros_axion_detection_gb300) never calls it.
 *
 * Every function restates one reference function (paths inside the
 * PhilJ0ly/albatros_axion_detection project, under albatros_analysis/):
 *
 *   or_unpack_4bit_float      src/correlations/unpacking.c:155-205
 *   or_unpack_1bit_float      src/correlations/unpacking.c:207-246
 *   or_sortpols               src/correlations/unpacking.c:248-368
 *   or_hist_4bit / _1bit      src/correlations/unpacking.c:7-153
 *   or_avg_xcorr_4bit         src/correlations/correlations_cpu.c:128-186
 *   or_avg_xcorr_4bit_2ant    src/correlations/correlations_cpu.c:188-271
 *   or_avg_xcorr_1bit         src/correlations/correlations_cpu.c:273-433
 *   or_avg_xcorr_1bit_vanvleck(_2ant)
 *                             src/correlations/correlations_cpu.c:435-638
 *   or_xcorr_all_ant_4bit     all-baseline version of the above, the int64
 *                             oracle for the coarse correlator (the matrix
 *                             X X^H of src/correlations/correlations_gpu.py:95-121
 *                             evaluated exactly on the decoded nibbles)
 *
 * Differences from the reference, all deliberate:
 *   - sums are accumulated in int64 (the reference uses per-thread int32
 *     partial sums added into float32), so the oracle is exact for any
 *     length; the Python wrapper converts and divides exactly as the
 *     reference's Python layer does;
 *   - everything is single-threaded unless OR_THREADS>1 is requested through
 *     the *_mt entry points (OpenMP), used only for the timed baseline.
 *
 * Decode rule kept bit-exact (unpacking.c:187-202): a nibble v in [0,15] maps
 * to v-16 when v > 8, else v.  Nibble 0x8 therefore decodes to +8.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline int nib_decode(unsigned v) { return v > 8u ? (int)v - 16 : (int)v; }
static inline int hi_nib(uint8_t b) { return nib_decode((unsigned)(b >> 4)); }
static inline int lo_nib(uint8_t b) { return nib_decode((unsigned)(b & 15u)); }
static inline int bit_pm1(uint8_t b, int shift) { return ((b >> shift) & 1) ? 1 : -1; }

/* Output: interleaved (re, im) float32, (nrows, ncols) per pol.
   Byte 2*c of a spectrum row is pol0 of channel c, byte 2*c+1 is pol1. */
void or_unpack_4bit_float(const uint8_t *data, float *pol0, float *pol1,
                          int64_t rowstart, int64_t rowend,
                          const int64_t *channels, int64_t ncols, int64_t nchan)
{
    const int64_t rowlen = 2 * nchan;
    for (int64_t r = rowstart; r < rowend; r++) {
        const uint8_t *row = data + r * rowlen;
        float *o0 = pol0 + 2 * (r - rowstart) * ncols;
        float *o1 = pol1 + 2 * (r - rowstart) * ncols;
        for (int64_t k = 0; k < ncols; k++) {
            uint8_t b0 = row[2 * channels[k]], b1 = row[2 * channels[k] + 1];
            o0[2 * k] = (float)hi_nib(b0);
            o0[2 * k + 1] = (float)lo_nib(b0);
            o1[2 * k] = (float)hi_nib(b1);
            o1[2 * k + 1] = (float)lo_nib(b1);
        }
    }
}

/* 1-bit: byte j of a spectrum holds channels 2j and 2j+1 with bits (MSB first)
   r0c0 i0c0 r1c0 i1c0 r0c1 i0c1 r1c1 i1c1; a set bit is +1, a clear bit -1.
   Channels [chanstart, chanend) must start even (unpacking.c:220-243). */
void or_unpack_1bit_float(const uint8_t *data, float *pol0, float *pol1,
                          int64_t rowstart, int64_t rowend,
                          int64_t chanstart, int64_t chanend, int64_t nchan)
{
    const int64_t bps = nchan / 2, nc = chanend - chanstart;
    for (int64_t r = rowstart; r < rowend; r++) {
        float *o0 = pol0 + 2 * (r - rowstart) * nc;
        float *o1 = pol1 + 2 * (r - rowstart) * nc;
        for (int64_t j = 0; j < nc / 2; j++) {
            uint8_t b = data[r * bps + chanstart / 2 + j];
            o0[4 * j + 0] = (float)bit_pm1(b, 7);
            o0[4 * j + 1] = (float)bit_pm1(b, 6);
            o1[4 * j + 0] = (float)bit_pm1(b, 5);
            o1[4 * j + 1] = (float)bit_pm1(b, 4);
            o0[4 * j + 2] = (float)bit_pm1(b, 3);
            o0[4 * j + 3] = (float)bit_pm1(b, 2);
            o1[4 * j + 2] = (float)bit_pm1(b, 1);
            o1[4 * j + 3] = (float)bit_pm1(b, 0);
        }
    }
}

/* Separate the pols of packed data without decoding.
   4-bit: one byte per channel per pol.
   1-bit: four channels per output byte per pol; pol0 keeps bits (r,i) of
   channels c..c+3 as r0i0 r1i1 r2i2 r3i3, pol1 the same; the last byte holds
   (chanend-chanstart)%4 channels when that is nonzero (unpacking.c:276-366). */
void or_sortpols(const uint8_t *data, uint8_t *pol0, uint8_t *pol1,
                 int64_t rowstart, int64_t rowend, int64_t ncols, int64_t nchan,
                 int bit_depth, int64_t chanstart, int64_t chanend)
{
    const int64_t nrows = rowend - rowstart;
    memset(pol0, 0, (size_t)(nrows * ncols));
    memset(pol1, 0, (size_t)(nrows * ncols));
    if (bit_depth == 4) {
        for (int64_t i = 0; i < nrows; i++)
            for (int64_t k = chanstart; k < chanend; k++) {
                pol0[i * ncols + k - chanstart] = data[(i + rowstart) * 2 * nchan + 2 * k];
                pol1[i * ncols + k - chanstart] = data[(i + rowstart) * 2 * nchan + 2 * k + 1];
            }
        return;
    }
    if (bit_depth != 1) return;
    const int64_t bps = nchan / 2; /* bytes per spectrum row, integer division as in the reference */
    const int64_t nsel = chanend - chanstart;
    for (int64_t i = 0; i < nrows; i++) {
        const uint8_t *row = data + (i + rowstart) * bps + chanstart / 2;
        for (int64_t j = 0; j < ncols; j++) {
            /* channels handled by this output byte: 4j .. 4j+3 (relative) */
            int64_t left = nsel - 4 * j;
            int nch = left >= 4 ? 4 : (int)left;
            uint8_t p0 = 0, p1 = 0;
            for (int c = 0; c < nch; c++) {
                uint8_t b = row[2 * j + c / 2];
                int sh = (c & 1) ? 0 : 4;          /* channel pair half */
                unsigned bits = (b >> sh) & 15u;   /* r0 i0 r1 i1 for that channel */
                unsigned pol0bits = (bits >> 2) & 3u, pol1bits = bits & 3u;
                p0 |= (uint8_t)(pol0bits << (6 - 2 * c));
                p1 |= (uint8_t)(pol1bits << (6 - 2 * c));
            }
            pol0[i * ncols + j] = p0;
            pol1[i * ncols + j] = p1;
        }
    }
}

/* Histograms of quantisation levels (unpacking.c:7-153). mode 0: pol0, 1: pol1,
   -1: both. histvals is (nbins+1, nchan) uint64; a 4-bit level v counts at
   bin (v & 15) i.e. the raw nibble; a 1-bit level at its bit value. */
void or_hist_4bit(const uint8_t *data, uint64_t *histvals, int64_t rowstart, int64_t rowend,
                  int64_t nchan, int64_t nbins, int mode)
{
    memset(histvals, 0, sizeof(uint64_t) * (size_t)((nbins + 1) * nchan));
    for (int64_t r = rowstart; r < rowend; r++)
        for (int64_t c = 0; c < nchan; c++)
            for (int p = 0; p < 2; p++) {
                if (mode != -1 && mode != p) continue;
                uint8_t b = data[r * 2 * nchan + 2 * c + p];
                histvals[(b >> 4) * nchan + c]++;
                histvals[(b & 15) * nchan + c]++;
            }
}

void or_hist_1bit(const uint8_t *data, uint64_t *histvals, int64_t rowstart, int64_t rowend,
                  int64_t nchan, int64_t nbins, int mode)
{
    memset(histvals, 0, sizeof(uint64_t) * (size_t)((nbins + 1) * nchan));
    for (int64_t r = rowstart; r < rowend; r++)
        for (int64_t j = 0; j < nchan / 2; j++) {
            uint8_t b = data[r * (nchan / 2) + j];
            for (int half = 0; half < 2; half++) {
                int c = (int)(2 * j + half);
                unsigned bits = (b >> (half ? 0 : 4)) & 15u;
                for (int p = 0; p < 2; p++) {
                    if (mode != -1 && mode != p) continue;
                    unsigned pb = p == 0 ? (bits >> 2) & 3u : bits & 3u;
                    histvals[((pb >> 1) & 1u) * nchan + c]++;
                    histvals[(pb & 1u) * nchan + c]++;
                }
            }
        }
}

/* sum over rows of d0 * conj(d1) on sortpols'd 4-bit data (rows, ncol).
   re = r0 r1 + i0 i1, im = r1 i0 - r0 i1 (correlations_cpu.c:172-173). */
void or_avg_xcorr_4bit(const uint8_t *data0, const uint8_t *data1, int64_t *re, int64_t *im,
                       int64_t nrows, int64_t ncol)
{
    for (int64_t k = 0; k < ncol; k++) re[k] = im[k] = 0;
    for (int64_t i = 0; i < nrows; i++)
        for (int64_t k = 0; k < ncol; k++) {
            uint8_t a = data0[i * ncol + k], b = data1[i * ncol + k];
            int r0 = hi_nib(a), i0 = lo_nib(a), r1 = hi_nib(b), i1 = lo_nib(b);
            re[k] += r0 * r1 + i0 * i1;
            im[k] += r1 * i0 - r0 * i1;
        }
}

/* Merge-intersect of two ascending specnum lists (correlations_cpu.c:201-214):
   writes matching row pairs, returns how many. */
int64_t or_specnum_intersect(const int64_t *s0, const int64_t *s1, int64_t off0, int64_t off1,
                             int64_t n0, int64_t n1, int32_t *rows0, int32_t *rows1)
{
    int64_t i = 0, j = 0, n = 0;
    while (i < n0 && j < n1) {
        int64_t a = s0[i] - off0, b = s1[j] - off1;
        if (a == b) { rows0[n] = (int32_t)i; rows1[n] = (int32_t)j; n++; i++; j++; }
        else if (a > b) j++;
        else i++;
    }
    return n;
}

int64_t or_avg_xcorr_4bit_2ant(const uint8_t *data0, const uint8_t *data1, int64_t *re, int64_t *im,
                               const int64_t *specnum0, const int64_t *specnum1,
                               int64_t idxstart0, int64_t idxstart1,
                               int64_t nrows0, int64_t nrows1, int64_t ncol)
{
    int32_t *r0 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nrows0 > 0 ? nrows0 : 1));
    int32_t *r1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nrows1 > 0 ? nrows1 : 1));
    int64_t n = or_specnum_intersect(specnum0, specnum1, idxstart0, idxstart1, nrows0, nrows1, r0, r1);
    for (int64_t k = 0; k < ncol; k++) re[k] = im[k] = 0;
    for (int64_t i = 0; i < n; i++)
        for (int64_t k = 0; k < ncol; k++) {
            uint8_t a = data0[(int64_t)r0[i] * ncol + k], b = data1[(int64_t)r1[i] * ncol + k];
            int x0 = hi_nib(a), y0 = lo_nib(a), x1 = hi_nib(b), y1 = lo_nib(b);
            re[k] += x0 * x1 + y0 * y1;
            im[k] += x1 * y0 - x0 * y1;
        }
    free(r0); free(r1);
    return n;
}

/* 1-bit packed (sortpols layout: 4 channels per byte, bits r,i per channel).
   Product of +-1 values: x*y = 1 - 2*(bx ^ by). Re = rr + ii, Im = r1 i0 - r0 i1
   (correlations_cpu.c:327-334). ncol = bytes per row, nchan = channels. */
void or_avg_xcorr_1bit(const uint8_t *data0, const uint8_t *data1, int64_t *re, int64_t *im,
                       int64_t nchan, int64_t nspec, int64_t ncol)
{
    for (int64_t k = 0; k < nchan; k++) re[k] = im[k] = 0;
    for (int64_t i = 0; i < nspec; i++)
        for (int64_t c = 0; c < nchan; c++) {
            uint8_t a = data0[i * ncol + c / 4], b = data1[i * ncol + c / 4];
            int sh = 6 - 2 * (int)(c % 4);
            int ar = (a >> (sh + 1)) & 1, ai = (a >> sh) & 1;
            int br = (b >> (sh + 1)) & 1, bi = (b >> sh) & 1;
            re[c] += 2 - 2 * ((ar ^ br) + (ai ^ bi));
            im[c] += -2 * ((br ^ ai) - (ar ^ bi));
        }
}

/* Van Vleck partial sums (correlations_cpu.c:490-508): per channel the four
   +-1 products R0 = r0 r1, R1 = i0 i1, IM0 = r0 i1, IM1 = r1 i0. */
static void vv_accum(uint8_t a, uint8_t b, int c, int64_t *R0, int64_t *R1, int64_t *IM0, int64_t *IM1)
{
    int sh = 6 - 2 * (c % 4);
    int ar = (a >> (sh + 1)) & 1, ai = (a >> sh) & 1;
    int br = (b >> (sh + 1)) & 1, bi = (b >> sh) & 1;
    R0[c] += 1 - 2 * (ar ^ br);
    R1[c] += 1 - 2 * (ai ^ bi);
    IM0[c] += 1 - 2 * (ar ^ bi);
    IM1[c] += 1 - 2 * (br ^ ai);
}

/* ncol bytes per row; all 4*ncol channel slots are summed, as the reference
   does (correlations_cpu.c:469-509); results are written for nchan channels. */
void or_avg_xcorr_1bit_vanvleck(const uint8_t *data0, const uint8_t *data1,
                                int64_t *R0, int64_t *R1, int64_t *IM0, int64_t *IM1,
                                int64_t nchan, int64_t nrows, int64_t ncol)
{
    int64_t nslot = 4 * ncol > nchan ? 4 * ncol : nchan;
    int64_t *t = (int64_t *)calloc((size_t)(4 * nslot), sizeof(int64_t));
    for (int64_t i = 0; i < nrows; i++)
        for (int64_t c = 0; c < 4 * ncol; c++)
            vv_accum(data0[i * ncol + c / 4], data1[i * ncol + c / 4], (int)c, t, t + nslot, t + 2 * nslot, t + 3 * nslot);
    for (int64_t c = 0; c < nchan; c++) {
        R0[c] = t[c]; R1[c] = t[nslot + c]; IM0[c] = t[2 * nslot + c]; IM1[c] = t[3 * nslot + c];
    }
    free(t);
}

int64_t or_avg_xcorr_1bit_vanvleck_2ant(const uint8_t *data0, const uint8_t *data1,
                                        int64_t *R0, int64_t *R1, int64_t *IM0, int64_t *IM1,
                                        const int64_t *specnum0, const int64_t *specnum1,
                                        int64_t idxstart0, int64_t idxstart1,
                                        int64_t nrows0, int64_t nrows1, int64_t ncol, int64_t nchan)
{
    int32_t *r0 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nrows0 > 0 ? nrows0 : 1));
    int32_t *r1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nrows1 > 0 ? nrows1 : 1));
    int64_t n = or_specnum_intersect(specnum0, specnum1, idxstart0, idxstart1, nrows0, nrows1, r0, r1);
    int64_t nslot = 4 * ncol > nchan ? 4 * ncol : nchan;
    int64_t *t = (int64_t *)calloc((size_t)(4 * nslot), sizeof(int64_t));
    for (int64_t i = 0; i < n; i++)
        for (int64_t c = 0; c < 4 * ncol; c++)
            vv_accum(data0[(int64_t)r0[i] * ncol + c / 4], data1[(int64_t)r1[i] * ncol + c / 4], (int)c,
                     t, t + nslot, t + 2 * nslot, t + 3 * nslot);
    for (int64_t c = 0; c < nchan; c++) {
        R0[c] = t[c]; R1[c] = t[nslot + c]; IM0[c] = t[2 * nslot + c]; IM1[c] = t[3 * nslot + c];
    }
    free(t); free(r0); free(r1);
    return n;
}

/* All-baseline coarse correlator on raw 4-bit packets, exact int64.
   raw: nant arrays laid out back to back, each (nspec, 2*nchan) bytes.
   Input index m = ant*2 + pol.  For rows [rowstart, rowend) and the ncols
   channel columns in `channels`:
     re[(i*M + j)*ncols + k] = sum_t Re(x_i x_j^*),  im likewise,
   i.e. the unnormalised X X^H per channel.  nthreads>1 uses OpenMP over
   channels (the sums are integers, so the result does not depend on it). */
void or_xcorr_all_ant_4bit(const uint8_t *raw, int64_t nant, int64_t nspec, int64_t nchan,
                           int64_t rowstart, int64_t rowend,
                           const int64_t *channels, int64_t ncols,
                           int64_t *re, int64_t *im, int nthreads)
{
    const int64_t M = 2 * nant, rowlen = 2 * nchan;
    (void)nthreads;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) if (nthreads > 1)
#endif
    for (int64_t k = 0; k < ncols; k++) {
        int64_t *accr = (int64_t *)calloc((size_t)(M * M), sizeof(int64_t));
        int64_t *acci = (int64_t *)calloc((size_t)(M * M), sizeof(int64_t));
        int *xr = (int *)malloc(sizeof(int) * (size_t)M);
        int *xi = (int *)malloc(sizeof(int) * (size_t)M);
        for (int64_t t = rowstart; t < rowend; t++) {
            for (int64_t a = 0; a < nant; a++)
                for (int p = 0; p < 2; p++) {
                    uint8_t b = raw[(a * nspec + t) * rowlen + 2 * channels[k] + p];
                    xr[2 * a + p] = hi_nib(b);
                    xi[2 * a + p] = lo_nib(b);
                }
            for (int64_t i = 0; i < M; i++)
                for (int64_t j = 0; j < M; j++) {
                    accr[i * M + j] += xr[i] * xr[j] + xi[i] * xi[j];
                    acci[i * M + j] += xi[i] * xr[j] - xr[i] * xi[j];
                }
        }
        for (int64_t i = 0; i < M * M; i++) {
            re[i * ncols + k] = accr[i];
            im[i * ncols + k] = acci[i];
        }
        free(accr); free(acci); free(xr); free(xi);
    }
}

/* Multi-threaded 4-bit unpack for the timed CPU baseline (same arithmetic). */
void or_unpack_4bit_float_mt(const uint8_t *data, float *pol0, float *pol1,
                             int64_t rowstart, int64_t rowend,
                             const int64_t *channels, int64_t ncols, int64_t nchan, int nthreads)
{
    (void)nthreads;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for if (nthreads > 1)
#endif
    for (int64_t r = rowstart; r < rowend; r++)
        or_unpack_4bit_float(data, pol0 + 2 * (r - rowstart) * ncols, pol1 + 2 * (r - rowstart) * ncols,
                             r, r + 1, channels, ncols, nchan);
}
