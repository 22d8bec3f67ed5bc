"""IPFB / PFB on the GPU: the call surface of
albatros_analysis/src/utils/pfb_gpu_utils.py (calculate_filter :29-36,
cupy_ipfb :56-91, cupy_pfb :105-121, get_matft :123-137) and
albatros_analysis/src/utils/pfb_utils.py (sinc_hamming :4-7), computed by the
CUDA kernels of csrc/ipfb.cu and csrc/pfb.cu.

The FFTs are this library's own shared-memory mixed-radix transforms:
register butterflies of radix 2, 3, 4, 5, 7, 8; any other prime factor of an
IPFB length runs by Bluestein's method (a chirp convolution through a
7-smooth FFT in shared memory; smaller primes and the rare ones too long for
shared memory as direct DFT passes), so cupy_ipfb runs any even nslice, like
the reference's cuFFT: 10.6 ms for nslice 32788 = 4 * 7 * 1171 (the
reference's default cut on 2^15 spectra) against 1.4 ms for 32928 =
2^5 * 3 * 7^3 on one GB300.  lblock must factor into 2, 3, 5, 7; PFB lengths
must be powers of two (lblock = 4096*osamp).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._arrays import device_array, to_device


def sinc_hamming(ntap, lblock):
    """Hamming window times sinc over ntap blocks, float64 on the host.

    Reference: src/utils/pfb_utils.py:4-7."""
    n = ntap * lblock
    w = np.arange(0, n) - n / 2
    return np.hamming(n) * np.sinc(w / lblock)


def get_matft(nslice, nchan=2049, ntap=4):
    """Spectrum of the zero-padded window matrix, (lblock, nslice//2+1) complex64,
    evaluated directly in FP64 on the GPU (4 nonzero taps per column).

    Reference: src/utils/pfb_gpu_utils.py:123-137."""
    nslice, nchan, ntap = int(nslice), int(nchan), int(ntap)
    lblock = 2 * (nchan - 1)
    out = torch.empty((lblock, nslice // 2 + 1), dtype=torch.complex64, device="cuda")
    _lib.call("ab_get_matft", _lib.ctx(), out.data_ptr(), nslice, nchan, ntap, _lib.stream_ptr(out))
    return out


def calculate_filter(matft, thresh):
    """Wiener-regularised inverse 1/conj(m) * |m|^2/(t^2+|m|^2) * (1+t^2), in FP64.

    Reference: src/utils/pfb_gpu_utils.py:29-36."""
    m = device_array(matft, torch.complex64, "matft").contiguous()
    out = torch.empty_like(m)
    _lib.call("ab_calculate_filter", m.data_ptr(), out.data_ptr(), m.numel(), float(thresh), _lib.stream_ptr(m))
    return out


def build_filter(nslice, thresh, nchan=2049, ntap=4):
    """calculate_filter(get_matft(nslice, nchan, ntap), thresh) in one FP64 pass.

    Reference: scripts/xcorr/helper_gpu_stream_clean.py:281-292 (get_matft then calculate_filter)."""
    lblock = 2 * (int(nchan) - 1)
    out = torch.empty((lblock, int(nslice) // 2 + 1), dtype=torch.complex64, device="cuda")
    _lib.call("ab_build_filter", _lib.ctx(), out.data_ptr(), int(nslice), int(nchan), int(ntap), float(thresh),
              _lib.stream_ptr(out))
    return out


def cupy_ipfb(dat, filt):
    """Inverse PFB of (nslice, nchan) complex64 spectra with filter
    (lblock, nslice//2+1) -> (nslice, lblock) float32.

    Like the reference, the result is the transpose of a C-ordered
    (lblock, nslice) array (an F-ordered view).

    Reference: src/utils/pfb_gpu_utils.py:56-91."""
    d = device_array(dat, torch.complex64, "dat").contiguous()
    f = device_array(filt, torch.complex64, "filt").contiguous()
    if d.dim() != 2:
        raise ValueError("dat must be 2-D (nslice, nchan)")
    nslice, nchan = d.shape
    lblock = 2 * (nchan - 1)
    if tuple(f.shape) != (lblock, nslice // 2 + 1):
        raise ValueError(f"filt must have shape {(lblock, nslice // 2 + 1)}, got {tuple(f.shape)}")
    out = torch.empty((lblock, nslice), dtype=torch.float32, device=d.device)
    _lib.call("ab_ipfb", _lib.ctx(d.device.index), d.data_ptr(), f.data_ptr(), out.data_ptr(), nslice, nchan,
              _lib.stream_ptr(d))
    return out.T


def _pfb_args(timestream, win, nchan, ntap):
    ts = device_array(timestream, torch.float32, "timestream").contiguous()
    w = to_device(win, torch.float32, ts.device)
    lblock = 2 * (int(nchan) - 1)
    if w.numel() != int(ntap) * lblock:
        raise ValueError(f"win must hold ntap*lblock = {int(ntap) * lblock} samples")
    nblock = ts.numel() // lblock - (int(ntap) - 1)
    return ts, w, lblock, nblock


def cupy_pfb(timestream, win, out=None, nchan=2049, ntap=4):
    """Forward PFB: tap-fold the timestream with `win` and real-FFT each block of
    lblock = 2*(nchan-1) samples -> (nblock, nchan) complex64.  As in the
    reference, `out` is only checked for shape.

    Reference: src/utils/pfb_gpu_utils.py:105-121."""
    ts, w, lblock, nblock = _pfb_args(timestream, win, nchan, ntap)
    if out is not None:
        assert tuple(out.shape) == (nblock, nchan)
    res = torch.empty((max(nblock, 0), int(nchan)), dtype=torch.complex64, device=ts.device)
    if nblock > 0:
        _lib.call("ab_pfb", _lib.ctx(ts.device.index), ts.data_ptr(), ts.numel(), w.data_ptr(), int(nchan), int(ntap),
                  res.data_ptr(), _lib.stream_ptr(ts))
    return res


def cupy_pfb_band(timestream, win, q0, q1, nchan=2049, ntap=4):
    """cupy_pfb(...)[:, q0:q1] without forming the other bins (q0, q1 multiples
    of osamp = lblock/4096).

    Reference: src/utils/pfb_gpu_utils.py:105-121 with the band slice of
    scripts/xcorr/helper_gpu_stream_clean.py:342-346."""
    ts, w, lblock, nblock = _pfb_args(timestream, win, nchan, ntap)
    res = torch.empty((max(nblock, 0), int(q1) - int(q0)), dtype=torch.complex64, device=ts.device)
    if nblock > 0:
        _lib.call("ab_pfb_band", _lib.ctx(ts.device.index), ts.data_ptr(), ts.numel(), w.data_ptr(), int(nchan),
                  int(ntap), int(q0), int(q1), res.data_ptr(), _lib.stream_ptr(ts))
    return res
