"""Correlators on the GPU: the call surface of
albatros_analysis/src/correlations/correlations.py (avg_xcorr_4bit :296-327,
avg_xcorr_4bit_2ant :330-383, avg_xcorr_1bit :386-408,
avg_xcorr_1bit_vanvleck(_2ant) :411-489, van_vleck_correction :491-497,
avg_xcorr_4bit_float_gpu :180-207) and
albatros_analysis/src/correlations/correlations_gpu.py (avg_xcorr_all_ant_gpu :95-121),
plus the exact all-baseline coarse correlator on raw 4-bit packets.

Integer correlators sum exactly in int64 on the device and then convert and
divide like the reference's Python layer (complex64 / rowcount), so results
equal the reference's whenever its float32 partial sums are exact.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._arrays import device_array, host_int64, to_device


def _dev_u8(a, name):
    return to_device(a, torch.uint8)


def _intersect(specnum0, specnum1, off0, off1):
    """Matched row pairs of two ascending specnum lists, as the merge loop of
    correlations_cpu.c:201-214."""
    a = host_int64(specnum0) - int(off0)
    b = host_int64(specnum1) - int(off1)
    _, i0, i1 = np.intersect1d(a, b, assume_unique=False, return_indices=True)
    return i0.astype(np.int32), i1.astype(np.int32)


def _pairs4(d0, d1, r0, r1, nmatch, ncol):
    re = torch.empty(ncol, dtype=torch.int64, device=d0.device)
    im = torch.empty(ncol, dtype=torch.int64, device=d0.device)
    tr0 = None if r0 is None else torch.from_numpy(r0).to(d0.device)
    tr1 = None if r1 is None else torch.from_numpy(r1).to(d0.device)
    _lib.call("ab_avg_xcorr_4bit_pairs", d0.data_ptr(), d1.data_ptr(), _lib.ptr(tr0), _lib.ptr(tr1), int(nmatch),
              int(ncol), re.data_ptr(), im.data_ptr(), _lib.stream_ptr(d0))
    return re.cpu().numpy(), im.cpu().numpy()


def avg_xcorr_4bit(data0, data1, specnums):
    """Time-averaged d0 * conj(d1) per channel of sortpols'd 4-bit data
    (rows, ncol); the first len(specnums) rows are used.  complex64 (ncol,),
    or nan for an empty block.

    Reference: src/correlations/correlations.py:296-327 (C correlations_cpu.c:128-186)."""
    assert data0.shape[1] == data1.shape[1]
    assert data0.shape[0] == data1.shape[0]
    rowcount = len(specnums)
    if rowcount == 0:
        return np.nan
    if rowcount > data0.shape[0]:
        raise ValueError("more specnums than rows")
    d0, d1 = _dev_u8(data0, "data0"), _dev_u8(data1, "data1")
    re, im = _pairs4(d0, d1, None, None, rowcount, d0.shape[1])
    xc = (re.astype(np.float32) + 1j * im.astype(np.float32)).astype(np.complex64)
    return xc / rowcount


def avg_xcorr_4bit_2ant(data0, data1, specnum0, specnum1, start_idx0, start_idx1):
    """Cross-correlation of two antennas over the spectra present in both
    (specnum - start_idx equal).  complex64 (ncol,) / rowcount, or nan.

    Reference: src/correlations/correlations.py:330-383 (C correlations_cpu.c:188-271)."""
    assert data0.shape[1] == data1.shape[1]
    if len(specnum0) == 0 or len(specnum1) == 0:
        return np.nan
    r0, r1 = _intersect(specnum0, specnum1, start_idx0, start_idx1)
    if r0.size == 0:
        return np.nan
    if r0.max() >= data0.shape[0] or r1.max() >= data1.shape[0]:
        raise ValueError("specnum rows beyond data")
    d0, d1 = _dev_u8(data0, "data0"), _dev_u8(data1, "data1")
    re, im = _pairs4(d0, d1, r0, r1, r0.size, d0.shape[1])
    xc = (re.astype(np.float32) + 1j * im.astype(np.float32)).astype(np.complex64)
    return xc / r0.size


def _pairs1(data0, data1, r0, r1, nmatch, nchannels):
    d0, d1 = _dev_u8(data0, "data0"), _dev_u8(data1, "data1")
    ncol = d0.shape[1]
    if nchannels > 4 * ncol:
        raise ValueError("nchannels exceeds 4 * bytes per row")
    sums = torch.empty((6, int(nchannels)), dtype=torch.int64, device=d0.device)
    tr0 = None if r0 is None else torch.from_numpy(r0).to(d0.device)
    tr1 = None if r1 is None else torch.from_numpy(r1).to(d0.device)
    _lib.call("ab_avg_xcorr_1bit_pairs", d0.data_ptr(), d1.data_ptr(), _lib.ptr(tr0), _lib.ptr(tr1), int(nmatch),
              ncol, int(nchannels), sums.data_ptr(), _lib.stream_ptr(d0))
    return sums.cpu().numpy()


def avg_xcorr_1bit(data0, data1, specnums, nchannels):
    """1-bit (sortpols layout) time-averaged d0 * conj(d1), complex64 (nchannels,).

    Reference: src/correlations/correlations.py:386-408 (C correlations_cpu.c:273-433)."""
    assert data0.shape[0] == data1.shape[0]
    assert data0.shape[1] == data1.shape[1]
    rowcount = len(specnums)
    if rowcount == 0:
        return np.nan
    s = _pairs1(data0, data1, None, None, rowcount, nchannels)
    xc = (s[0].astype(np.float32) + 1j * s[1].astype(np.float32)).astype(np.complex64)
    return xc / rowcount


def avg_xcorr_1bit_vanvleck(data0, data1, specnums, nchannels):
    """Van Vleck partial sums [R0, R1, IM0, IM1] (float32, / rowcount).

    Reference: src/correlations/correlations.py:411-443 (C correlations_cpu.c:435-525)."""
    assert data0.shape[0] == data1.shape[0]
    assert data0.shape[1] == data1.shape[1]
    rowcount = len(specnums)
    if rowcount == 0:
        return [np.full(nchannels, np.nan, np.float32) for _ in range(4)]
    s = _pairs1(data0, data1, None, None, rowcount, nchannels)
    return [s[q].astype(np.float32) / rowcount for q in (2, 3, 4, 5)]


def avg_xcorr_1bit_vanvleck_2ant(data0, data1, nchannels, specnum0, specnum1, idxstart0, idxstart1):
    """Two-antenna Van Vleck partial sums ([R0, R1, IM0, IM1] float32, rowcount).

    Reference: src/correlations/correlations.py:446-489 (C correlations_cpu.c:527-638)."""
    assert data0.shape[0] == data1.shape[0]
    assert data0.shape[1] == data1.shape[1]
    nanv = [np.full(nchannels, np.nan, np.float32) for _ in range(4)]
    if len(specnum0) == 0 or len(specnum1) == 0:
        return nanv, 0
    r0, r1 = _intersect(specnum0, specnum1, idxstart0, idxstart1)
    if r0.size == 0:
        return nanv, 0
    s = _pairs1(data0, data1, r0, r1, r0.size, nchannels)
    return [s[q].astype(np.float32) for q in (2, 3, 4, 5)], int(r0.size)


def van_vleck_correction(R0, R1, I0, I1, rowcount):
    """Arcsine-law correction of 1-bit partial sums (correlations.py:491-497)."""
    k = np.pi / 2 / rowcount
    return np.sin(R0 * k) + np.sin(R1 * k) + 1j * (np.sin(I1 * k) - np.sin(I0 * k))


def _f_order_ok(t: torch.Tensor, shape) -> bool:
    return tuple(t.shape) == tuple(shape) and t.permute(*reversed(range(t.dim()))).is_contiguous()


def avg_xcorr_all_ant_gpu(x, nant: int, npol: int, ntime: int, nfreq: int, split: int = 1, scratch=None, out=None):
    """All antenna-pol pairs, out[i, j, f] = sum_t x[i, t, f] conj(x[j, t, f]) / ntime.

    x: complex64 F-ordered (nant*npol, ntime, nfreq) device array (a torch
    tensor with those strides, or any contiguous buffer of that many
    elements read in F order).  Returns F-ordered (M, M, nfreq) complex64.

    Reference: src/correlations/correlations_gpu.py:95-121 (cuBLAS, cgemm_batch.cu:8-53)."""
    M = int(nant) * int(npol)
    K = int(ntime)
    if K % split != 0:
        raise ValueError("split should be a divisor of ntime")
    xt = device_array(x, torch.complex64, "x")
    if xt.numel() != M * K * int(nfreq):
        raise ValueError("x does not hold nant*npol*ntime*nfreq elements")
    if xt.dim() == 3 and not _f_order_ok(xt, (M, K, int(nfreq))):
        raise ValueError("x must be F-ordered (nant*npol, ntime, nfreq)")
    if xt.dim() != 3 and not xt.is_contiguous():
        raise ValueError("flat x must be contiguous")
    if out is None:
        out = torch.empty((int(nfreq), M, M), dtype=torch.complex64, device=xt.device).permute(2, 1, 0)
    elif not isinstance(out, torch.Tensor) or not _f_order_ok(out, (M, M, int(nfreq))) or out.dtype != xt.dtype:
        raise ValueError("invalid out buffer")
    if split > 1:
        raise NotImplementedError()
    _lib.call("ab_avg_xcorr_all_ant", xt.data_ptr(), int(nant), int(npol), K, int(nfreq), out.data_ptr(),
              _lib.stream_ptr(xt))
    return out


def avg_xcorr_4bit_float_gpu(data0, data1, specnum0, specnum1):
    """Single-baseline average of unpacked complex64 data (rows, nchan).

    Same specnum array (same antenna): mean of data0 * conj(data1) over the
    first len(specnum0) rows, returned with that count, as the reference.
    Different antennas: over the rows whose specnums match.

    Reference: src/correlations/correlations.py:180-207."""
    d0 = device_array(data0, torch.complex64, "data0")
    d1 = device_array(data1, torch.complex64, "data1")
    same = specnum0 is specnum1 or (hasattr(specnum0, "__array_interface__") and hasattr(specnum1, "__array_interface__")
                                    and specnum0.__array_interface__["data"][0] == specnum1.__array_interface__["data"][0])
    if same:
        n = len(specnum0)
        a, b = d0[:n], d1[:n]
    else:
        r0, r1 = _intersect(specnum0, specnum1, 0, 0)
        n = int(r0.size)
        a = d0[torch.from_numpy(r0.astype(np.int64)).to(d0.device)]
        b = d1[torch.from_numpy(r1.astype(np.int64)).to(d1.device)]
    if n == 0:
        return np.nan, 0
    nchan = a.shape[1]
    # F-ordered (2, n, nchan): element (i, t, f) at i + 2 (t + n f)
    x = torch.stack([a, b]).permute(2, 1, 0).contiguous().permute(2, 1, 0)
    out = avg_xcorr_all_ant_gpu(x, 2, 1, n, nchan)
    return out[0, 1, :].contiguous(), n


def xcorr_coarse_4bit(raw, rowstart, rowend, channels, length_channels, chunk=None, rows=None, average=True):
    """Exact all-baseline coarse correlation of raw 4-bit packets.

    raw: device uint8 (nant, nspec, 2*length_channels) (or one antenna 2-D);
    rows [rowstart, rowend) (or per-antenna row indices `rows` (nant, nrows)),
    channels: channel indices; chunk: spectra per average (None = all).
    Returns complex64 (nchunks, M, M, ncols) averages (average=True, /rows per
    chunk) or the exact int64 (re, im) sums.  M = 2*nant, input 2a+p.

    Reference: no single counterpart: every input pair of avg_xcorr_4bit (correlations_cpu.c:128-186)."""
    r = device_array(raw, torch.uint8, "raw")
    if r.dim() == 2:
        r = r.unsqueeze(0)
    if r.dim() != 3 or not r.is_contiguous():
        raise ValueError("raw must be contiguous (nant, nspec, 2*nchan)")
    nant, nspec, rb = r.shape
    length_channels = int(length_channels)
    if rb != 2 * length_channels:
        raise ValueError("raw rows must be 2*length_channels bytes")
    ch = host_int64(channels)
    if ch.size == 0 or ch.min() < 0 or ch.max() >= length_channels:
        raise ValueError("channel index out of range")
    trows = None
    if rows is not None:
        rr = np.ascontiguousarray(np.asarray(rows, dtype=np.int32))
        if rr.ndim != 2 or rr.shape[0] != nant or rr.min() < 0 or rr.max() >= nspec:
            raise ValueError("rows must be (nant, nrows) valid row indices")
        nrows = rr.shape[1]
        trows = torch.from_numpy(rr).to(r.device)
        rowstart = 0
    else:
        rowstart, rowend = int(rowstart), int(rowend)
        if rowstart < 0 or rowend > nspec or rowend <= rowstart:
            raise ValueError("bad row range")
        nrows = rowend - rowstart
    chunk = nrows if chunk is None else int(chunk)
    nchunks = -(-nrows // chunk)
    M = 2 * nant
    re = torch.empty((nchunks, M, M, ch.size), dtype=torch.int64, device=r.device)
    im = torch.empty_like(re)
    dch = torch.from_numpy(ch).to(r.device)
    _lib.call("ab_xcorr_coarse_4bit", _lib.ctx(r.device.index), r.data_ptr(), nspec * rb, nant, nspec,
              length_channels, rowstart, nrows, _lib.ptr(trows), dch.data_ptr(), ch.size, chunk, re.data_ptr(),
              im.data_ptr(), _lib.stream_ptr(r))
    if not average:
        return re, im
    counts = torch.tensor([min(chunk, nrows - k * chunk) for k in range(nchunks)], dtype=torch.float64,
                          device=r.device).view(-1, 1, 1, 1)
    return (torch.complex(re.to(torch.float64), im.to(torch.float64)) / counts).to(torch.complex64)
