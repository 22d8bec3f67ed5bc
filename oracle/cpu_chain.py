"""CPU re-channelisation chain for the timed CPU baseline.

TEST INFRASTRUCTURE / BASELINE ONLY: imported by ``bench.py`` (cpu_baseline
leg and ``--impl reference``) and tests; never by the product package.

This is the reference's own CPU pipeline restated with the libraries present
here (numba is not installed, so its loops become vectorised NumPy):
  unpack      the reference's C unpack_4bit_float (src/correlations/unpacking.c:155-205),
              from oracle/_ref when it was built in this checkout, else the
              oracle's C restatement of it;
  placement   make_continuous (src/correlations/baseband_data_classes.py:48-73);
  IPFB        cpu_ipfb (src/utils/pfb_cpu_utils.py:90-121): scipy.fft irfft /
              rfft / irfft in float32 with workers = all cores;
  PFB         cpu_pfb (src/utils/pfb_cpu_utils.py:143-172): tap fold then rfft;
  xcorr       avg_xcorr_all_ant_cpu_og (src/correlations/correlations.py:154-178):
              X_f X_f^H / K per frequency.
"""
from __future__ import annotations

import ctypes
import os
import time

import numpy as np
import scipy.fft as sfft

from . import c_oracle, ref_libs
from . import pfb_oracle as po


def unpacker():
    """(function, kind): the reference's compiled C when available, else the port."""
    libs = ref_libs()
    if libs is not None:
        up = libs[0]
        I, P = ctypes.c_int, ctypes.c_void_p
        up.unpack_4bit_float.argtypes = [P, P, P, I, I, P, I, I]

        def f(raw2d, r0, r1, ch, nchan):
            ch = np.ascontiguousarray(ch, np.int64)
            a = np.empty((r1 - r0, ch.size), np.complex64)
            b = np.empty_like(a)
            up.unpack_4bit_float(raw2d.ctypes.data, a.ctypes.data, b.ctypes.data, r0, r1, ch.ctypes.data, ch.size,
                                 nchan)
            return a, b
        return f, "reference"
    lib = c_oracle()

    def g(raw2d, r0, r1, ch, nchan):
        ch = np.ascontiguousarray(ch, np.int64)
        a = np.empty((r1 - r0, ch.size), np.complex64)
        b = np.empty_like(a)
        lib.or_unpack_4bit_float_mt(raw2d.ctypes.data, a.ctypes.data, b.ctypes.data, r0, r1, ch.ctypes.data, ch.size,
                                    nchan, os.cpu_count() or 1)
        return a, b
    return g, "port"


def ipfb_f32(dat, filt, cut, workers):
    """cpu_ipfb (src/utils/pfb_cpu_utils.py:90-121) in float32, then the chunk's [cut, -cut) rows raveled."""
    dd = sfft.irfft(dat, axis=1, workers=workers)
    ddft = sfft.rfft(dd.T, axis=1, workers=workers)
    ddft *= filt
    res = sfft.irfft(ddft, axis=1, workers=workers)
    return np.ascontiguousarray(res.T[cut:res.shape[1] - cut]).ravel()


def pfb_f32(ts, win, lblock, ntap, workers):
    """cpu_pfb (src/utils/pfb_cpu_utils.py:143-172): tap fold, then rfft of each block."""
    nblock = ts.size // lblock - (ntap - 1)
    t = ts[: (nblock + ntap - 1) * lblock].reshape(-1, lblock)
    w = win.reshape(ntap, lblock)
    y = t[0:nblock] * w[0]
    for i in range(1, ntap):
        y += t[i:nblock + i] * w[i]
    return sfft.rfft(y, axis=1, workers=workers)


class CpuChain:
    """One chunk of the streaming chain on the host (float32), per input as
    the reference's driver runs it (scripts/xcorr/helper_gpu_stream_clean.py:295-456)."""

    def __init__(self, channels_abs, acclen, cut, osamp, q0, q1, thresh=0.45, ntap=4, workers=None):
        self.chan_abs = np.asarray(channels_abs, np.int64)
        self.acclen, self.cut, self.osamp, self.ntap = acclen, cut, osamp, ntap
        self.q0, self.q1 = q0, q1
        self.workers = workers or os.cpu_count() or 1
        nslice = acclen + 2 * cut
        self.filt = po.calculate_filter(po.get_matft(nslice), thresh).astype(np.complex64)
        self.lblock = 4096 * osamp
        self.win = po.sinc_hamming(ntap, self.lblock).astype(np.float32)
        self.unpack, self.kind = unpacker()

    def run_chunk(self, raw, cols, nchan_raw, chunk=0):
        """raw: (nant, nspec, 2*nchan_raw) uint8.  Returns the chunk's (M, M, nq)
        visibilities of the fine blocks that lie inside the chunk."""
        nant = raw.shape[0]
        r0, r1 = chunk * self.acclen, (chunk + 1) * self.acclen
        xin = []
        for a in range(nant):
            p0, p1 = self.unpack(raw[a], r0, r1, cols, nchan_raw)
            for p in (p0, p1):
                placed = np.zeros((self.acclen + 2 * self.cut, 2049), np.complex64)
                placed[2 * self.cut:, self.chan_abs] = p
                ts = ipfb_f32(placed, self.filt, self.cut, self.workers)
                spec = pfb_f32(ts, self.win, self.lblock, self.ntap, self.workers)
                xin.append(spec[:, self.q0:self.q1])
        x = np.stack(xin)  # (M, nb, nq)
        K = x.shape[1]
        return np.einsum("itf,jtf->ijf", x, np.conj(x)) / K


def time_sample(raw, cols, chan_abs, nchan_raw, acclen, cut, osamp, q0, q1, reps=1):
    """Seconds per chunk of the CPU chain (both antennas), and its kind."""
    ch = CpuChain(chan_abs, acclen, cut, osamp, q0, q1)
    ch.run_chunk(raw, cols, nchan_raw, 0)  # warm caches / plans
    t0 = time.perf_counter()
    for _ in range(reps):
        ch.run_chunk(raw, cols, nchan_raw, 0)
    return (time.perf_counter() - t0) / reps, ch.kind, ch.workers
