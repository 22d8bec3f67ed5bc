"""Data placement on the GPU: make_continuous_gpu
(albatros_analysis/src/correlations/baseband_data_classes.py:48-73)."""
from __future__ import annotations

import torch

from . import _lib
from ._arrays import device_array, host_int64


def make_continuous_gpu(spec, chan_specnum, start_specnum, channels, nspec, nchans=2049, out=None):
    """Scatter the rows of `spec` to (specnum - start_specnum) % nspec and its
    columns to the absolute channel numbers `channels` of a zero
    (nspec, nchans) complex64 grid.  When nothing is missing and all nchans
    channels are present, `spec` itself is returned (or copied into `out`).

    Reference: src/correlations/baseband_data_classes.py:48-73."""
    s = device_array(spec, torch.complex64, "spec")
    sn = host_int64(chan_specnum, "chan_specnum")
    ch = host_int64(channels, "channels")
    nspec, nchans = int(nspec), int(nchans)
    if sn.size == nspec and ch.size == nchans:
        if out is not None:
            out.copy_(s)
            return out
        return s
    if out is None:
        out = torch.empty((nspec, nchans), dtype=torch.complex64, device=s.device)
    elif tuple(out.shape) != (nspec, nchans) or out.dtype != torch.complex64 or not out.is_contiguous():
        raise ValueError("invalid out buffer")
    if s.dim() != 2 or s.shape[1] != ch.size or s.shape[0] < sn.size or not s.is_contiguous():
        raise ValueError("spec must be contiguous (>= len(specnum), len(channels))")
    if ch.size and (ch.min() < 0 or ch.max() >= nchans):
        raise ValueError("channel number out of range")
    dsn = torch.from_numpy(sn).to(s.device)
    dch = torch.from_numpy(ch).to(s.device)
    _lib.call("ab_make_continuous", s.data_ptr(), sn.size, ch.size, dsn.data_ptr(), int(start_specnum),
              dch.data_ptr(), nspec, nchans, out.data_ptr(), _lib.stream_ptr(s))
    return out
