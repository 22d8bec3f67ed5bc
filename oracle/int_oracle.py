"""NumPy-facing wrappers of the C oracle (albatros_oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, ``__graft_entry__.smoke()`` and
the CPU legs of ``bench.py``.
"""
from __future__ import annotations

import numpy as np

from . import c_oracle


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def unpack_4bit(raw2d, rowstart, rowend, channels, nchan):
    """unpack_4bit_float (src/correlations/unpacking.c:155-205): 2 x (rows, ncols) complex64."""
    raw2d = _c(raw2d, np.uint8)
    ch = _c(channels, np.int64)
    p0 = np.empty((rowend - rowstart, ch.size), np.complex64)
    p1 = np.empty_like(p0)
    c_oracle().or_unpack_4bit_float(raw2d.ctypes.data, p0.ctypes.data, p1.ctypes.data, rowstart, rowend,
                                    ch.ctypes.data, ch.size, nchan)
    return p0, p1


def unpack_4bit_mt(raw2d, rowstart, rowend, channels, nchan, nthreads):
    """unpack_4bit (above) split over nthreads host threads (the CPU baseline)."""
    raw2d = _c(raw2d, np.uint8)
    ch = _c(channels, np.int64)
    p0 = np.empty((rowend - rowstart, ch.size), np.complex64)
    p1 = np.empty_like(p0)
    c_oracle().or_unpack_4bit_float_mt(raw2d.ctypes.data, p0.ctypes.data, p1.ctypes.data, rowstart, rowend,
                                       ch.ctypes.data, ch.size, nchan, nthreads)
    return p0, p1


def unpack_1bit(raw2d, rowstart, rowend, chanstart, chanend, nchan):
    """unpack_1bit_float (src/correlations/unpacking.c:207-246) over channels [chanstart, chanend)."""
    raw2d = _c(raw2d, np.uint8)
    p0 = np.empty((rowend - rowstart, chanend - chanstart), np.complex64)
    p1 = np.empty_like(p0)
    c_oracle().or_unpack_1bit_float(raw2d.ctypes.data, p0.ctypes.data, p1.ctypes.data, rowstart, rowend,
                                    chanstart, chanend, nchan)
    return p0, p1


def sortpols(raw2d, nchan, bit_depth, rowstart, rowend, chanstart, chanend):
    """sortpols (src/correlations/unpacking.c:248-368): the pols' bytes, undecoded."""
    raw2d = _c(raw2d, np.uint8)
    nc = (chanend - chanstart) if bit_depth == 4 else int(np.ceil((chanend - chanstart) / 4))
    p0 = np.empty((rowend - rowstart, nc), np.uint8)
    p1 = np.empty_like(p0)
    c_oracle().or_sortpols(raw2d.ctypes.data, p0.ctypes.data, p1.ctypes.data, rowstart, rowend, nc, nchan,
                           bit_depth, chanstart, chanend)
    return p0, p1


def hist(raw2d, rowstart, rowend, nchan, bit_depth, mode):
    """hist_4bit / hist_1bit (src/correlations/unpacking.c:7-153): (2**bit_depth, nchan) uint64 counts."""
    raw2d = _c(raw2d, np.uint8)
    nbins = 2 ** bit_depth - 1
    h = np.empty((nbins + 1, nchan), np.uint64)
    f = c_oracle().or_hist_4bit if bit_depth == 4 else c_oracle().or_hist_1bit
    f(raw2d.ctypes.data, h.ctypes.data, rowstart, rowend, nchan, nbins, mode)
    return h


def avg_xcorr_4bit_sums(d0, d1, nrows):
    """avg_xcorr_4bit (src/correlations/correlations_cpu.c:128-186) as exact int64 sums, not yet / rows."""
    d0, d1 = _c(d0, np.uint8), _c(d1, np.uint8)
    re = np.empty(d0.shape[1], np.int64)
    im = np.empty_like(re)
    c_oracle().or_avg_xcorr_4bit(d0.ctypes.data, d1.ctypes.data, re.ctypes.data, im.ctypes.data, nrows, d0.shape[1])
    return re, im


def avg_xcorr_4bit_2ant_sums(d0, d1, s0, s1, off0, off1):
    """avg_xcorr_4bit_2ant (src/correlations/correlations_cpu.c:188-271): int64 sums over the
    intersected spectrum numbers, and their count."""
    d0, d1 = _c(d0, np.uint8), _c(d1, np.uint8)
    s0, s1 = _c(s0, np.int64), _c(s1, np.int64)
    re = np.empty(d0.shape[1], np.int64)
    im = np.empty_like(re)
    n = c_oracle().or_avg_xcorr_4bit_2ant(d0.ctypes.data, d1.ctypes.data, re.ctypes.data, im.ctypes.data,
                                          s0.ctypes.data, s1.ctypes.data, off0, off1, s0.size, s1.size, d0.shape[1])
    return re, im, int(n)


def avg_xcorr_1bit_sums(d0, d1, nchan, nspec):
    """avg_xcorr_1bit (src/correlations/correlations_cpu.c:273-433) as exact int64 sums."""
    d0, d1 = _c(d0, np.uint8), _c(d1, np.uint8)
    re = np.empty(nchan, np.int64)
    im = np.empty_like(re)
    c_oracle().or_avg_xcorr_1bit(d0.ctypes.data, d1.ctypes.data, re.ctypes.data, im.ctypes.data, nchan, nspec,
                                 d0.shape[1])
    return re, im


def vanvleck_2ant_sums(d0, d1, nchan, s0, s1, off0, off1):
    """avg_xcorr_1bit_vanvleck_2ant (src/correlations/correlations_cpu.c:527-638): the four
    int64 partial sums per channel over the intersected spectra, and their count."""
    d0, d1 = _c(d0, np.uint8), _c(d1, np.uint8)
    s0, s1 = _c(s0, np.int64), _c(s1, np.int64)
    out = [np.empty(nchan, np.int64) for _ in range(4)]
    n = c_oracle().or_avg_xcorr_1bit_vanvleck_2ant(d0.ctypes.data, d1.ctypes.data, *[o.ctypes.data for o in out],
                                                   s0.ctypes.data, s1.ctypes.data, off0, off1, s0.size, s1.size,
                                                   d0.shape[1], nchan)
    return out, int(n)


def vanvleck_sums(d0, d1, nchan, nrows):
    """avg_xcorr_1bit_vanvleck (src/correlations/correlations_cpu.c:435-525): the four int64
    partial sums per channel."""
    d0, d1 = _c(d0, np.uint8), _c(d1, np.uint8)
    out = [np.empty(nchan, np.int64) for _ in range(4)]
    c_oracle().or_avg_xcorr_1bit_vanvleck(d0.ctypes.data, d1.ctypes.data, *[o.ctypes.data for o in out], nchan, nrows,
                                          d0.shape[1])
    return out


def xcorr_all_ant_4bit(raw3d, rowstart, rowend, channels, nchan, nthreads=1):
    """Exact (M, M, ncols) int64 re/im sums of x_i conj(x_j) over rows: the all-baseline form of
    avg_xcorr_4bit (src/correlations/correlations_cpu.c:128-186) for every input pair."""
    raw3d = _c(raw3d, np.uint8)
    ch = _c(channels, np.int64)
    nant, nspec = raw3d.shape[0], raw3d.shape[1]
    M = 2 * nant
    re = np.empty((M, M, ch.size), np.int64)
    im = np.empty_like(re)
    c_oracle().or_xcorr_all_ant_4bit(raw3d.ctypes.data, nant, nspec, nchan, rowstart, rowend, ch.ctypes.data,
                                     ch.size, re.ctypes.data, im.ctypes.data, nthreads)
    return re, im
