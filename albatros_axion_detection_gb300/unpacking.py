"""Packed-baseband unpacking on the GPU: the call surface of
albatros_analysis/src/correlations/unpacking.py (unpack_4bit :193-245,
unpack_1bit :248-302, sortpols :305-377, hist :82-138), computed by the CUDA kernels of
csrc/unpack.cu through the C-ABI."""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._arrays import device_array, host_int64


def _rows_view(data: torch.Tensor, bytes_per_spectrum: int, rowend: int, name: str = "data"):
    n = data.numel()
    if not data.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if bytes_per_spectrum <= 0 or n % bytes_per_spectrum:
        raise ValueError(f"{name} size {n} is not a multiple of {bytes_per_spectrum} bytes per spectrum")
    if rowend > n // bytes_per_spectrum:
        raise ValueError(f"rowend {rowend} beyond the {n // bytes_per_spectrum} spectra in {name}")


def unpack_4bit(data, rowstart, rowend, channels, length_channels, dtype=torch.complex64):
    """4-bit baseband -> (pol0, pol1) complex64 (rowend-rowstart, len(channels)).

    data: device uint8 array holding spectra of 2*length_channels bytes (pol0
    byte then pol1 byte per channel; real = high nibble, imag = low nibble,
    nibble v > 8 decodes to v - 16). channels: channel INDICES (host).
    dtype=torch.int8 returns the same levels as int8 complex instead,
    (rows, len(channels), 2) with (re, im) last.

    Reference: src/correlations/unpacking.py:193-245 (GPU :140-155; C unpacking.c:155-205)."""
    d = device_array(data, torch.uint8, "data")
    rowstart, rowend, length_channels = int(rowstart), int(rowend), int(length_channels)
    ch = host_int64(channels, "channels")
    if rowstart < 0 or rowend < rowstart:
        raise ValueError(f"bad row range [{rowstart}, {rowend})")
    _rows_view(d, 2 * length_channels, rowend)
    if ch.size and (ch.min() < 0 or ch.max() >= length_channels):
        raise ValueError("channel index out of range")
    nrows, ncols = rowend - rowstart, ch.size
    if dtype == torch.int8:
        pol0 = torch.empty((nrows, ncols, 2), dtype=torch.int8, device=d.device)
        pol1 = torch.empty((nrows, ncols, 2), dtype=torch.int8, device=d.device)
        if nrows and ncols:
            dch = torch.from_numpy(ch).to(d.device)
            _lib.call("ab_unpack_4bit_i8", d.data_ptr(), pol0.data_ptr(), pol1.data_ptr(), rowstart, rowend,
                      dch.data_ptr(), ncols, length_channels, _lib.stream_ptr(d))
        return pol0, pol1
    if dtype != torch.complex64:
        raise ValueError("dtype must be torch.complex64 or torch.int8")
    pol0 = torch.empty((nrows, ncols), dtype=torch.complex64, device=d.device)
    pol1 = torch.empty((nrows, ncols), dtype=torch.complex64, device=d.device)
    if nrows == 0 or ncols == 0:
        return pol0, pol1
    s = _lib.stream_ptr(d)
    contiguous = ncols % 4 == 0 and ch[0] % 4 == 0 and length_channels % 4 == 0 and \
        np.array_equal(ch, np.arange(ch[0], ch[0] + ncols)) and d.data_ptr() % 8 == 0
    if contiguous:
        _lib.call("ab_unpack_4bit_range", d.data_ptr(), pol0.data_ptr(), pol1.data_ptr(), rowstart, rowend,
                  int(ch[0]), ncols, length_channels, s)
    else:
        dch = torch.from_numpy(ch).to(d.device)
        _lib.call("ab_unpack_4bit", d.data_ptr(), pol0.data_ptr(), pol1.data_ptr(), rowstart, rowend,
                  dch.data_ptr(), ncols, length_channels, s)
    return pol0, pol1


def unpack_1bit(data, rowstart, rowend, channels, length_channels, dtype=torch.complex64):
    """1-bit baseband -> (pol0, pol1) complex64 (rows, len(channels)), values +-1
    (dtype=torch.int8: int8 complex, (rows, len(channels), 2)).

    Like the reference's GPU path, byte columns channels[::2]//2 are decoded and
    each byte fills two consecutive output channels (the channel list must be
    made of (even, even+1) pairs: contiguous and starting even)."""
    d = device_array(data, torch.uint8, "data")
    rowstart, rowend, length_channels = int(rowstart), int(rowend), int(length_channels)
    ch = host_int64(channels, "channels")
    if ch.size % 2:
        raise ValueError("1-bit unpack needs an even number of channels")
    if ch.size and (ch.min() < 0 or ch.max() >= length_channels):
        raise ValueError("channel index out of range")
    if rowstart < 0 or rowend < rowstart:
        raise ValueError(f"bad row range [{rowstart}, {rowend})")
    _rows_view(d, length_channels // 2, rowend)
    cols = ch[::2] // 2
    nrows = rowend - rowstart
    if dtype == torch.int8:
        pol0 = torch.empty((nrows, ch.size, 2), dtype=torch.int8, device=d.device)
        pol1 = torch.empty((nrows, ch.size, 2), dtype=torch.int8, device=d.device)
        if nrows and ch.size:
            dcols = torch.from_numpy(np.ascontiguousarray(cols)).to(d.device)
            _lib.call("ab_unpack_1bit_i8", d.data_ptr(), pol0.data_ptr(), pol1.data_ptr(), rowstart, rowend,
                      dcols.data_ptr(), cols.size, length_channels, _lib.stream_ptr(d))
        return pol0, pol1
    if dtype != torch.complex64:
        raise ValueError("dtype must be torch.complex64 or torch.int8")
    pol0 = torch.empty((nrows, ch.size), dtype=torch.complex64, device=d.device)
    pol1 = torch.empty((nrows, ch.size), dtype=torch.complex64, device=d.device)
    if nrows == 0 or ch.size == 0:
        return pol0, pol1
    dcols = torch.from_numpy(np.ascontiguousarray(cols)).to(d.device)
    _lib.call("ab_unpack_1bit", d.data_ptr(), pol0.data_ptr(), pol1.data_ptr(), rowstart, rowend,
              dcols.data_ptr(), cols.size, length_channels, _lib.stream_ptr(d))
    return pol0, pol1


def sortpols(data, length_channels, bit_mode, rowstart, rowend, chanstart, chanend):
    """Separate the pols of packed data without decoding (device uint8 out).

    4-bit: (rows, chanend-chanstart) bytes per pol. 1-bit: four channels per
    byte, (rows, ceil((chanend-chanstart)/4)) bytes per pol.

    Reference: src/correlations/unpacking.py:305-377 (C unpacking.c:248-408)."""
    d = device_array(data, torch.uint8, "data")
    length_channels, rowstart, rowend = int(length_channels), int(rowstart), int(rowend)
    if chanend is None:
        chanstart, chanend = 0, length_channels
    elif chanend > length_channels:
        raise ValueError("ERROR: Trying to unpack more channels than present. Check chanend.")
    chanstart, chanend = int(chanstart), int(chanend)
    if bit_mode == 4:
        ncols = chanend - chanstart
        _rows_view(d, 2 * length_channels, rowend)
    elif bit_mode == 1:
        if chanstart % 2 > 0:
            raise ValueError("ERROR: Start channel index must be even.")
        ncols = int(np.ceil((chanend - chanstart) / 4))
        _rows_view(d, length_channels // 2, rowend)
    else:
        raise ValueError("bit_mode must be 1 or 4")
    nrows = rowend - rowstart
    pol0 = torch.empty((nrows, ncols), dtype=torch.uint8, device=d.device)
    pol1 = torch.empty((nrows, ncols), dtype=torch.uint8, device=d.device)
    if nrows > 0 and ncols > 0:
        _lib.call("ab_sortpols", d.data_ptr(), pol0.data_ptr(), pol1.data_ptr(), rowstart, rowend, ncols,
                  length_channels, int(bit_mode), chanstart, chanend, _lib.stream_ptr(d))
    return pol0, pol1


def hist(data, rowstart, rowend, length_channels, bit_depth, mode):
    """Histogram of quantisation levels: device uint64 (2**bit_depth, length_channels).

    hist[v, c] counts the real and imaginary levels of channel c in rows
    [rowstart, rowend) equal to v (the raw nibble for 4-bit data, the bit for
    1-bit data), over pol0 (mode 0), pol1 (mode 1) or both (mode -1).  The
    reference asserts on a bad bit_depth or mode; here they raise ValueError.

    Reference: src/correlations/unpacking.py:82-138 (C unpacking.c:7-153)."""
    d = device_array(data, torch.uint8, "data")
    rowstart, rowend, length_channels = int(rowstart), int(rowend), int(length_channels)
    if bit_depth not in (1, 4):
        raise ValueError(f"bit_depth set to {bit_depth}, only takes values 1 or 4")
    if mode not in (0, 1, -1):
        raise ValueError(f"mode set to {mode}, only takes values 0,1,-1")
    if rowstart < 0 or rowend < rowstart:
        raise ValueError(f"bad row range [{rowstart}, {rowend})")
    if bit_depth == 1 and length_channels % 2:
        raise ValueError("1-bit data needs an even number of channels")
    _rows_view(d, 2 * length_channels if bit_depth == 4 else length_channels // 2, rowend)
    out = torch.empty((2 ** bit_depth, length_channels), dtype=torch.uint64, device=d.device)
    _lib.call("ab_hist", d.data_ptr(), out.data_ptr(), rowstart, rowend, length_channels, int(bit_depth), int(mode),
              _lib.stream_ptr(d))
    return out
