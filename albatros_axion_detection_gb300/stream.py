"""Streaming unpack -> IPFB -> PFB(osamp) -> fine cross-correlation on the GPU.

Host-side mirror of the reference's streaming driver
(albatros_analysis/scripts/xcorr/helper_gpu_stream_clean.py): the same
ProcessingConfig fields, the same job planner (JobChunkPlanner.plan_chunks
:233-263), the same band [channels[chanstart]*osamp, channels[chanend]*osamp)
(:342-343) and visibility layout (M, M, nchan, njobs) F-ordered (:347).  The
per-chunk work and all overlap state live on the device in an ``ab_stream``
object (csrc/chain.cu).  Inputs are 4-bit or 1-bit packets on the device
(``ingest`` builds them, with their spectrum map, from baseband files), or
pinned host packets streamed in chunk by chunk (``run_from_host``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np
import torch

from . import _lib, output
from ._arrays import device_array, host_int64


@dataclass
class ProcessingConfig:
    """Configuration of one streaming run (helper_gpu_stream_clean.py:38-51)."""
    acclen: int          # new coarse spectra per IPFB chunk
    pfb_size: int        # unused, kept for signature parity
    nchunks: int         # IPFB chunks to process
    nblock: int          # fine PFB blocks per job
    chanstart: int
    chanend: int
    osamp: int
    cut: int = 10
    filt_thresh: float = 0.45
    ntap: int = 4
    npol: int = 2


class JobChunkPlanner:
    """Reference: scripts/xcorr/helper_gpu_stream_clean.py:229-263."""

    @staticmethod
    def plan_chunks(nchunks: int, lchunk: int, nblock: int, lblock: int, ntap: int) -> List[Tuple[int, Optional[int]]]:
        """Job -> chunk ranges: a job needs (nblock + ntap - 1) * lblock samples,
        and advances by nblock * lblock (helper_gpu_stream_clean.py:233-263)."""
        ranges = []
        stride, need = nblock * lblock, (nblock + ntap - 1) * lblock
        have, cur = 0, 0
        while cur < nchunks:
            start = cur
            while have < need and cur < nchunks:
                have += lchunk
                cur += 1
            if have >= need:
                ranges.append((start, cur))
                have -= stride
            else:
                if have > 0:
                    ranges.append((start, cur))
                break
        return ranges


def band_edges(channels, chanstart: int, chanend: int, osamp: int) -> Tuple[int, int]:
    """Fine band [channels[chanstart]*osamp, channels[chanend]*osamp); when
    chanend is one past the last recorded channel, (channels[-1]+1)*osamp.

    Reference: scripts/xcorr/helper_gpu_stream_clean.py:342-343."""
    ch = host_int64(channels)
    q0 = int(ch[chanstart]) * osamp
    q1 = int(ch[chanend]) * osamp if chanend < ch.size else (int(ch[chanend - 1]) + 1) * osamp
    return q0, q1


class StreamCorrelator:
    """Device state of one streaming run; push chunks in order, read vis.

    Reference: scripts/xcorr/helper_gpu_stream_clean.py:295-456 (the per-chunk loop and its overlap state)."""

    def __init__(self, nant: int, channels, chanstart: int, chanend: int, acclen: int, nchunks: int, nblock: int,
                 osamp: int, cut: int = 10, filt_thresh: float = 0.45, ntap: int = 4, nchan_raw: Optional[int] = None,
                 bits: int = 4):
        ch = host_int64(channels)
        if bits not in (1, 4):
            raise ValueError("bits must be 1 or 4")
        self.bits = int(bits)
        self.nant, self.M = int(nant), 2 * int(nant)
        self.nchan_raw = int(nchan_raw if nchan_raw is not None else ch.size)
        self.acclen, self.nchunks, self.nblock = int(acclen), int(nchunks), int(nblock)
        self.osamp, self.cut, self.ntap, self.filt_thresh = int(osamp), int(cut), int(ntap), float(filt_thresh)
        self.lblock = 4096 * self.osamp
        self.jobs = JobChunkPlanner.plan_chunks(self.nchunks, self.acclen * 4096, self.nblock, self.lblock, self.ntap)
        self.q0, self.q1 = band_edges(ch, chanstart, chanend, self.osamp)
        cols = np.arange(chanstart, chanend, dtype=np.int64)
        absch = np.ascontiguousarray(ch[chanstart:chanend])
        self._cols, self._abs = cols, absch
        out = ctypes.c_void_p()
        _lib.call("ab_stream_create", _lib.ctx(), self.nant, self.nchan_raw, self.bits, cols.ctypes.data, absch.ctypes.data,
                  cols.size, self.acclen, self.cut, self.osamp, self.ntap, self.filt_thresh, self.nblock,
                  len(self.jobs), self.q0, self.q1, ctypes.byref(out))
        self._h = out.value
        self.nq = self.q1 - self.q0

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().ab_stream_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        _lib.call("ab_stream_reset", self._h, _lib.stream_ptr())

    def push(self, raw: torch.Tensor, chunk: int, spec_map: Optional[torch.Tensor] = None, final: bool = False):
        """Process chunk `chunk` of raw packets (nant, nspec, 2*nchan_raw) uint8
        on the device: spectra [chunk*acclen - 2*cut, (chunk+1)*acclen) are
        read (row g of antenna a is spec_map[a, g] when given, <0 = missing)."""
        need = (int(chunk) + 1) * self.acclen
        if spec_map is None and raw.shape[1] < need:
            raise ValueError(f"raw holds {raw.shape[1]} spectra, chunk {chunk} needs {need}")
        row_bytes = 2 * self.nchan_raw if self.bits == 4 else self.nchan_raw // 2
        if raw.shape[0] != self.nant or raw.shape[2] != row_bytes or not raw.is_contiguous():
            raise ValueError(f"raw must be contiguous (nant, nspec, {row_bytes}) uint8")
        mp, mstride = 0, 0
        if spec_map is not None:
            if spec_map.dtype != torch.int32 or spec_map.shape[0] != self.nant or spec_map.shape[1] < need \
                    or not spec_map.is_contiguous():
                raise ValueError("spec_map must be contiguous int32 (nant, >= (chunk+1)*acclen)")
            mp, mstride = spec_map.data_ptr(), spec_map.shape[1]
        fn = "ab_stream_push_final" if final else "ab_stream_push"
        _lib.call(fn, self._h, raw.data_ptr(), raw.shape[1] * raw.shape[2], mp, mstride, int(chunk),
                  _lib.stream_ptr(raw))

    def run_from_host(self, host: torch.Tensor, dev: torch.Tensor, spec_map: Optional[torch.Tensor] = None,
                      copy_stream: Optional[torch.cuda.Stream] = None):
        """Process every chunk from pinned host packets: chunk j's spectra are
        copied from ``host`` into the device buffer ``dev`` (same shape) on a
        side stream, ahead of the push that reads them, so the transfers
        overlap the chain; each push waits only for its own chunk's copy
        (its 2*cut earlier rows came with the previous chunk)."""
        if host.shape != dev.shape or host.dtype != torch.uint8 or not host.is_pinned():
            raise ValueError("host must be a pinned uint8 tensor shaped like dev")
        if not dev.is_cuda or not dev.is_contiguous() or not host.is_contiguous():
            raise ValueError("dev must be a contiguous device tensor")
        cur = torch.cuda.current_stream(dev.device)
        cs = copy_stream if copy_stream is not None else torch.cuda.Stream(device=dev.device)
        cs.wait_stream(cur)  # earlier work on dev is done before it is overwritten
        nspec = host.shape[1]
        events = []
        with torch.cuda.stream(cs):
            for j in range(self.nchunks):
                lo = j * self.acclen
                hi = nspec if j == self.nchunks - 1 else min((j + 1) * self.acclen, nspec)
                for a in range(host.shape[0]):
                    dev[a, lo:hi].copy_(host[a, lo:hi], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                events.append(ev)
        for j, ev in enumerate(events):
            cur.wait_event(ev)
            self.push(dev, j, spec_map, final=(j == self.nchunks - 1))
        dev.record_stream(cs)

    def vis_device(self) -> torch.Tensor:
        """Device view (njobs, M, M, nq) complex64 of the accumulated visibilities."""
        n = max(len(self.jobs), 1) * self.M * self.M * self.nq
        addr = _lib.load().ab_stream_vis(self._h)
        t = _device_view(addr, n)
        return t.view(max(len(self.jobs), 1), self.M, self.M, self.nq)[: len(self.jobs)]

    def fir_taps(self) -> int:
        """Half-length J of the FIR time stage (0: the IIR or FFT form runs)."""
        return int(_lib.load().ab_stream_fir_taps(self._h))

    def time_filter(self):
        """("fft", 0), ("fir", J) or ("iir", rows a state is carried): the form of the
        IPFB time stage this stream runs."""
        kind, param = ctypes.c_int32(), ctypes.c_int32()
        _lib.call("ab_stream_time_filter", self._h, ctypes.byref(kind), ctypes.byref(param))
        return ("fft", "fir", "iir")[kind.value], int(param.value)

    def workspace_bytes(self) -> int:
        """Bytes of per-push scratch this stream can take from a shared
        workspace (-1: it keeps state there and cannot share)."""
        return int(_lib.load().ab_stream_workspace_bytes(self._h))

    def set_workspace(self, ws: torch.Tensor):
        """Use ``ws`` (a device uint8 tensor, kept alive here) as this stream's
        per-push scratch.  Streams sharing one workspace must push in turn on
        one CUDA stream."""
        if ws.dtype != torch.uint8 or not ws.is_cuda or not ws.is_contiguous():
            raise ValueError("workspace must be a contiguous uint8 CUDA tensor")
        _lib.call("ab_stream_set_workspace", self._h, ws.data_ptr(), ws.numel())
        self._ws = ws

    def kernel_launches(self) -> int:
        return int(_lib.load().ab_stream_kernel_launches(self._h))

    STAGES = ("row_ifft", "time_deconv", "pfb_fold", "pfb_dft", "xcorr")

    def profile(self, enable: bool = True):
        """Time each stage of later pushes with CUDA events (serialising)."""
        _lib.call("ab_stream_profile", self._h, 1 if enable else 0)

    def stage_times(self) -> dict:
        ms = np.zeros(5, np.float64)
        n = np.zeros(5, np.int64)
        _lib.call("ab_stream_stage_times", self._h, ms.ctypes.data, n.ctypes.data)
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.STAGES)}


def _device_view(addr: int, n: int) -> torch.Tensor:
    """Wrap n complex64 at device address `addr` (owned by the library)."""
    class _CAI:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<c8", "data": (addr, False), "version": 3,
                                    "strides": None}
    return torch.as_tensor(_CAI(), device="cuda")


def repfb_xcorr_avg(raw, channels, acclen: int, nchunks: int, nblock: int, chanstart: int, chanend: int, osamp: int,
                    cut: int = 10, filt_thresh: float = 0.45, ntap: int = 4, spec_map=None, bits: int = 4,
                    with_missing: bool = False):
    """Streaming unpack -> IPFB -> PFB -> xcorr over device-resident packets.

    raw: (nant, nspec, 2*nchan_raw) uint8 device array of 4-bit packets, or
    (nant, nspec, nchan_raw/2) of 1-bit packets with bits=1; channels: absolute
    channel numbers of the raw columns; [chanstart, chanend) selects the
    coarse channels.  Returns (vis, freqs): vis (M, M, nchan, njobs) complex64
    F-ordered (numpy, NaNs masked as the reference does) and the fine
    channel numbers; with_missing=True returns (vis, missing_fraction, freqs)
    like the reference (helper_gpu_stream_clean.py:402), missing_fraction
    (nant, njobs) the per-job missing-spectrum percentage of each antenna."""
    r = device_array(raw, torch.uint8, "raw")
    ch = host_int64(channels)
    nchan_raw = r.shape[2] // 2 if bits == 4 else r.shape[2] * 2
    sc = StreamCorrelator(r.shape[0], ch, chanstart, chanend, acclen, nchunks, nblock, osamp, cut, filt_thresh, ntap,
                          nchan_raw=nchan_raw, bits=bits)
    try:
        for j in range(nchunks):
            sc.push(r, j, spec_map, final=(j == nchunks - 1))
        v = sc.vis_device().permute(1, 2, 3, 0).cpu().numpy()  # (M, M, nq, njobs)
    finally:
        sc.close()
    vis = output.mask_invalid(np.asfortranarray(v))
    freqs = np.arange(sc.q0, sc.q1)
    if not with_missing:
        return vis, freqs
    present = output.chunk_presence(spec_map, r.shape[0], nchunks, acclen)
    return vis, output.missing_fraction(present, acclen, nblock, osamp, ntap), freqs
