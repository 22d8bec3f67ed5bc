"""FP64 NumPy restatement of the ALBATROS re-channelisation arithmetic.

TEST INFRASTRUCTURE. Only tests/, ``__graft_entry__.smoke()`` and the
cpu_baseline / reference legs of ``bench.py`` may import this module, and only
as the checker or as the timed CPU baseline.  The product package
``albatros_axion_detection_gb300`` never imports it.

Each function restates one reference function (paths inside the
PhilJ0ly/albatros_axion_detection project, under ``albatros_analysis/``):

=====================  ============================================================
sinc_hamming           src/utils/pfb_utils.py:4-7
get_matft              src/utils/pfb_gpu_utils.py:123-137 (window kept in FP64 unless
                       ``window_f32``; the reference casts it to float32 at :126)
calculate_filter       src/utils/pfb_gpu_utils.py:29-36
ipfb                   src/utils/pfb_gpu_utils.py:56-91 (cuFFT C2R/R2C conventions of
                       src/utils/pycufft.py:120-161: irfft divides by n)
pfb                    src/utils/pfb_gpu_utils.py:105-121
xcorr_all_ant          src/correlations/correlations_gpu.py:95-121
make_continuous        src/correlations/baseband_data_classes.py:48-73
plan_chunks            scripts/xcorr/helper_gpu_stream_clean.py:233-263
stream_timestream      scripts/xcorr/helper_gpu_stream_clean.py:178-197, :433-438
repfb_xcorr_avg        scripts/xcorr/helper_gpu_stream_clean.py:295-456 (buffer
                       semantics of BufferManager :71-167, original channel mapping
                       of scripts/xcorr/helper_gpu_stream.py:196)
=====================  ============================================================

Everything is complex128/float64.  The FFTs are pocketfft's double-precision
transforms (``scipy.fft`` with all host threads when SciPy is present, else
``numpy.fft``: the same algorithm), with the same normalisation as the
reference's cuFFT wrapper (forward unscaled, inverse divided by n, imaginary
parts of the DC and Nyquist bins ignored by irfft).
"""
from __future__ import annotations

import os

import numpy as np

try:
    import scipy.fft as _sfft

    def _rfft(a, n=None, axis=-1):
        return _sfft.rfft(a, n=n, axis=axis, workers=os.cpu_count() or 1)

    def _irfft(a, n=None, axis=-1):
        return _sfft.irfft(a, n=n, axis=axis, workers=os.cpu_count() or 1)
except ImportError:  # pragma: no cover - SciPy is installed wherever the tests run
    _rfft, _irfft = np.fft.rfft, np.fft.irfft

__all__ = [
    "sinc_hamming", "get_matft", "calculate_filter", "ipfb", "pfb",
    "xcorr_all_ant", "make_continuous", "plan_chunks", "repfb_xcorr_avg", "stream_timestream",
    "decode_4bit", "unpack_4bit_np", "unpack_1bit_np", "band_edges",
]


def sinc_hamming(ntap: int, lblock: int) -> np.ndarray:
    """Hamming window times sinc over ntap blocks (src/utils/pfb_utils.py:4-7)."""
    n = ntap * lblock
    w = np.arange(0, n) - n / 2
    return np.hamming(n) * np.sinc(w / lblock)


def get_matft(nslice: int, nchan: int = 2049, ntap: int = 4, window_f32: bool = False) -> np.ndarray:
    """Window-matrix spectrum, (lblock, nslice//2+1) complex128.

    Column k holds the ntap window taps w[t*lblock+k] at rows t<ntap and zeros
    below; matft is its real FFT along the nslice axis
    (src/utils/pfb_gpu_utils.py:123-137)."""
    nn = 2 * (nchan - 1)
    win = sinc_hamming(ntap, nn)
    if window_f32:
        win = win.astype(np.float32).astype(np.float64)
    mat = np.zeros((nslice, nn))
    mat[:ntap, :] = win.reshape(ntap, nn)
    return _rfft(mat.T, axis=1)


def calculate_filter(matft: np.ndarray, thresh: float) -> np.ndarray:
    """Wiener-regularised inverse (src/utils/pfb_gpu_utils.py:29-36)."""
    filt = 1.0 / np.conj(matft)
    if thresh > 0:
        a2 = np.abs(matft) ** 2
        filt = filt * (a2 / (thresh ** 2 + a2) * (1.0 + thresh ** 2))
    return filt


def ipfb(dat: np.ndarray, filt: np.ndarray) -> np.ndarray:
    """Inverse PFB of (nslice, nchan) spectra -> (nslice, lblock) timestream,
    cupy_ipfb (src/utils/pfb_gpu_utils.py:56-91): irfft along channels, rfft
    along time, times filt, irfft along time.

    Returns the transposed view like the reference (F-ordered result)."""
    dd = _irfft(dat, axis=1)
    ddft = _rfft(dd.T, axis=1)
    ddft *= filt
    res = _irfft(ddft, n=dd.shape[0], axis=1)
    return res.T


def pfb(timestream: np.ndarray, win: np.ndarray, nchan: int = 2049, ntap: int = 4) -> np.ndarray:
    """Forward PFB: tap-fold then real FFT per block (src/utils/pfb_gpu_utils.py:105-121)."""
    lblock = 2 * (nchan - 1)
    ts = np.asarray(timestream, dtype=np.float64).ravel()
    nblock = ts.size // lblock - (ntap - 1)
    ts = ts[: (nblock + ntap - 1) * lblock].reshape(-1, lblock)
    w = np.asarray(win, dtype=np.float64).reshape(ntap, lblock)
    y = ts[0:nblock] * w[0]
    for i in range(1, ntap):
        y += ts[i:nblock + i] * w[i]
    return _rfft(y, axis=1)


def xcorr_all_ant(x: np.ndarray, nant: int, npol: int, ntime: int, nfreq: int) -> np.ndarray:
    """out[i, j, f] = sum_t x[i, t, f] conj(x[j, t, f]) / ntime
    (src/correlations/correlations_gpu.py:95-121)."""
    x = np.asarray(x, dtype=np.complex128).reshape(nant * npol, ntime, nfreq)
    return np.einsum("itf,jtf->ijf", x, np.conj(x)) / ntime


def decode_4bit(b: np.ndarray):
    """(re, im) int arrays of 4-bit packed bytes; nibble v>8 -> v-16
    (src/correlations/unpacking.c:187-202)."""
    b = np.asarray(b, dtype=np.uint8)
    hi = (b >> 4).astype(np.int64)
    lo = (b & 15).astype(np.int64)
    hi[hi > 8] -= 16
    lo[lo > 8] -= 16
    return hi, lo


def unpack_4bit_np(raw2d: np.ndarray, rowstart: int, rowend: int, channels) -> tuple:
    """Pure NumPy 4-bit unpack of (nspec, 2*nchan) bytes -> 2 x (rows, ncols) complex128,
    the decode of unpack_4bit_float (src/correlations/unpacking.c:155-205)."""
    ch = np.asarray(channels, dtype=np.int64)
    r = raw2d[rowstart:rowend]
    out = []
    for p in range(2):
        re, im = decode_4bit(r[:, 2 * ch + p])
        out.append(re + 1j * im)
    return out[0], out[1]


def unpack_1bit_np(raw2d: np.ndarray, rowstart: int, rowend: int, chanstart: int, chanend: int):
    """Pure NumPy 1-bit unpack of (nspec, nchan/2) bytes (src/correlations/unpacking.c:207-246)."""
    r = raw2d[rowstart:rowend, chanstart // 2: chanend // 2].astype(np.int64)
    bit = lambda s: 2 * ((r >> s) & 1) - 1
    n, nb = r.shape
    p0 = np.empty((n, 2 * nb), np.complex128)
    p1 = np.empty((n, 2 * nb), np.complex128)
    p0[:, 0::2] = bit(7) + 1j * bit(6)
    p1[:, 0::2] = bit(5) + 1j * bit(4)
    p0[:, 1::2] = bit(3) + 1j * bit(2)
    p1[:, 1::2] = bit(1) + 1j * bit(0)
    return p0, p1


def unpack_1bit_channels(raw2d: np.ndarray, rowstart: int, rowend: int, channels):
    """1-bit decode of arbitrary channel indices: channel c lives in byte c//2,
    high half-byte for even c, bits (r0, i0, r1, i1) MSB first, set bit = +1
    (src/correlations/unpacking.c:207-246)."""
    ch = np.asarray(channels, dtype=np.int64)
    b = raw2d[rowstart:rowend][:, ch // 2].astype(np.int64)
    v = np.where((ch % 2) == 0, b >> 4, b) & 15
    pm = lambda x: 2 * x - 1
    p0 = pm((v >> 3) & 1) + 1j * pm((v >> 2) & 1)
    p1 = pm((v >> 1) & 1) + 1j * pm(v & 1)
    return p0, p1


def make_continuous(spec, chan_specnum, start_specnum, channels, nspec, nchans=2049):
    """Place rows at (specnum-start) % nspec and columns at absolute channel
    numbers, zeros elsewhere (src/correlations/baseband_data_classes.py:48-73)."""
    spec = np.asarray(spec)
    specnum = (np.asarray(chan_specnum, dtype=np.int64) - start_specnum) % nspec
    out = np.zeros((nspec, nchans), dtype=np.complex128)
    out[np.ix_(specnum, np.asarray(channels, dtype=np.int64))] = spec[: len(specnum)]
    return out


def plan_chunks(nchunks: int, lchunk: int, nblock: int, lblock: int, ntap: int):
    """Job -> chunk ranges (scripts/xcorr/helper_gpu_stream_clean.py:233-263)."""
    ranges = []
    stride, need = nblock * lblock, (nblock + ntap - 1) * lblock
    rem, cur = 0, 0
    while cur < nchunks:
        start = cur
        while rem < need and cur < nchunks:
            rem += lchunk
            cur += 1
        if rem >= need:
            ranges.append((start, cur))
            rem -= stride
        else:
            if rem > 0:
                ranges.append((start, cur))
            break
    return ranges


def band_edges(channels, chanstart: int, chanend: int, osamp: int):
    """Fine band [channels[chanstart]*osamp, channels[chanend]*osamp)
    (scripts/xcorr/helper_gpu_stream_clean.py:342-343); when chanend is the
    last recorded channel, the end is (channels[chanend-1]+1)*osamp."""
    ch = np.asarray(channels, dtype=np.int64)
    q0 = int(ch[chanstart]) * osamp
    q1 = int(ch[chanend]) * osamp if chanend < len(ch) else (int(ch[chanend - 1]) + 1) * osamp
    return q0, q1


def stream_timestream(raw: np.ndarray, a: int, p: int, sel, chan_abs, acclen: int, nchunks: int, cut: int,
                      filt: np.ndarray, spec_present=None, bits: int = 4) -> np.ndarray:
    """The IPFB timestream of input (antenna a, pol p) over the first nchunks
    chunks, float64 (nchunks*acclen*4096 samples): per chunk, the previous
    chunk's last 2*cut placed rows (zeros before the first) and this chunk's
    acclen rows go through the IPFB and the [cut, nslice-cut) rows are kept
    (IPFBProcessor.process_chunk, scripts/xcorr/helper_gpu_stream_clean.py:178-197,
    and the cut_pol refresh :433-438)."""
    nslice = acclen + 2 * cut
    lchunk = acclen * 4096
    ts = np.empty(nchunks * lchunk)
    prev = np.zeros((2 * cut, 2049), np.complex128)
    for j in range(nchunks):
        rows = np.arange(j * acclen, (j + 1) * acclen)
        if bits == 4:
            spec = unpack_4bit_np(raw[a], rows[0], rows[-1] + 1, sel)[p]
        else:
            spec = unpack_1bit_channels(raw[a], rows[0], rows[-1] + 1, sel)[p]
        if spec_present is not None:
            keep = np.asarray(spec_present[a][rows], dtype=bool)
            placed = make_continuous(spec[keep], rows[keep], 0, chan_abs, acclen)
        else:
            placed = make_continuous(spec, rows, 0, chan_abs, acclen)
        x = np.concatenate([prev, placed], axis=0)
        ts[j * lchunk:(j + 1) * lchunk] = ipfb(x, filt)[cut:nslice - cut].ravel()
        prev = placed[acclen - 2 * cut:].copy()
        del x, placed
    return ts


def repfb_xcorr_avg(raw: np.ndarray, channels, acclen: int, nchunks: int, nblock: int,
                    chanstart: int, chanend: int, osamp: int, cut: int = 10,
                    filt_thresh: float = 0.45, ntap: int = 4, spec_present=None,
                    filt=None, bits: int = 4, max_jobs=None):
    """Streaming unpack -> IPFB -> PFB -> xcorr, FP64 restatement of
    repfb_xcorr_avg (scripts/xcorr/helper_gpu_stream_clean.py:295-402).

    raw: (nant, nspec, 2*nchan_raw) uint8 4-bit packets, one spectrum per row
    (bits=4), or (nant, nspec, nchan_raw/2) 1-bit packets (bits=1).
    channels: absolute channel numbers of the raw columns.
    spec_present: optional (nant, nchunks*acclen) bool; False rows are missing
    (zero-filled, as make_continuous does for absent specnums).
    max_jobs: compute only the first max_jobs jobs of the plan (and only the
    chunks they read); None computes every job.
    Returns vis (M, M, nfine, njobs) complex128 and the fine band (q0, q1).

    One input (antenna, pol) is carried at a time, so the working set is one
    input's timestream plus one job's PFB, whatever the number of inputs.
    """
    nant = raw.shape[0]
    npol, M = 2, 2 * raw.shape[0]
    lblock = 4096 * osamp
    nslice = acclen + 2 * cut
    sel = np.arange(chanstart, chanend)
    chan_abs = np.asarray(channels, dtype=np.int64)[sel]
    if filt is None:
        filt = calculate_filter(get_matft(nslice), filt_thresh)
    win = sinc_hamming(ntap, lblock)
    q0, q1 = band_edges(channels, chanstart, chanend, osamp)
    jobs = plan_chunks(nchunks, acclen * 4096, nblock, lblock, ntap)
    if max_jobs is not None:
        jobs = jobs[:max_jobs]
    njobs = len(jobs)
    # samples the jobs read (the last one zero-padded past the stream's end)
    span = (njobs * nblock + ntap - 1) * lblock
    lchunk = acclen * 4096
    nch_used = min(nchunks, -(-span // lchunk))
    xin = np.zeros((M, njobs, nblock, q1 - q0), np.complex128)
    for a in range(nant):
        for p in range(npol):
            ts = np.zeros(max(span, nch_used * lchunk))
            ts[:nch_used * lchunk] = stream_timestream(raw, a, p, sel, chan_abs, acclen, nch_used, cut, filt,
                                                       spec_present, bits)
            for k in range(njobs):
                seg = ts[k * nblock * lblock: k * nblock * lblock + (nblock + ntap - 1) * lblock]
                xin[2 * a + p, k] = pfb(seg, win, nchan=lblock // 2 + 1, ntap=ntap)[:, q0:q1]
            del ts
    vis = np.zeros((M, M, q1 - q0, njobs), np.complex128)
    for k in range(njobs):
        vis[..., k] = xcorr_all_ant(xin[:, k], nant, npol, nblock, q1 - q0)
    return vis, (q0, q1)
