"""Many baseband files of uneven size through the streaming chain, as one
captured CUDA graph.

The reference processes one file set at a time through its streaming driver
(albatros_analysis/scripts/xcorr/helper_gpu_stream_clean.py:295-456, called
once per run from scripts/xcorr/xcorr_gpu_cpu.py).  A batch here is a list of
files, each with its own packet format (4-bit or 1-bit), channel selection,
length, chunk size (acclen) and oversampling; every file gets its own
``StreamCorrelator`` (device overlap state and visibilities), and the files are
spread over a few CUDA streams ("lanes", longest-first onto the least-loaded
lane).  Files on one lane run in turn and share one per-push workspace, so
device memory grows with the number of lanes, not the number of files.  The
whole batch (optionally with the host->device copies of the packets and the
device->host copies of the visibilities) is captured once into a CUDA graph
and replayed.  The time stage of each (acclen, cut, osamp) comes from the
autotuner (``autotune.tune_configs``: IIR / FIR row tile, or FFT radix order).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import autotune
from .stream import StreamCorrelator


@dataclass
class BatchFile:
    """One file of the batch.

    raw: device packets (nant, nspec, row_bytes) uint8, row_bytes = 2*nchan
    (4-bit) or nchan/2 (1-bit); channels: absolute channel numbers of the raw
    columns; [chanstart, chanend) the selected ones (default all).  nchunks
    chunks of acclen spectra are processed (default: all whole chunks).
    host: optional pinned host copy of raw, copied in at every run."""
    raw: torch.Tensor
    channels: np.ndarray
    bits: int
    acclen: int
    cut: int
    osamp: int
    nblock: int
    nchunks: Optional[int] = None
    chanstart: int = 0
    chanend: Optional[int] = None
    spec_map: Optional[torch.Tensor] = None
    host: Optional[torch.Tensor] = None
    filt_thresh: float = 0.45
    ntap: int = 4
    name: str = ""

    def __post_init__(self):
        self.channels = np.asarray(self.channels, dtype=np.int64)
        if self.chanend is None:
            self.chanend = int(self.channels.size)
        if self.nchunks is None:
            self.nchunks = int(self.raw.shape[1]) // int(self.acclen)
        if self.nchunks < 1:
            raise ValueError(f"file {self.name!r}: fewer spectra than one chunk of {self.acclen}")

    @property
    def nant(self) -> int:
        return int(self.raw.shape[0])

    @property
    def nchan_raw(self) -> int:
        return int(self.raw.shape[2]) * 2 if self.bits == 1 else int(self.raw.shape[2]) // 2

    @property
    def spectra(self) -> int:
        """Input spectra consumed (all antennas)."""
        return self.nant * self.nchunks * self.acclen


def assign_lanes(work: Sequence[int], lanes: int) -> List[List[int]]:
    """Greedy longest-first assignment of items (by work) to at most `lanes`
    lanes, each item onto the currently least-loaded lane (ties: lowest lane)."""
    nl = max(1, min(int(lanes), len(work)))
    load = [0] * nl
    out: List[List[int]] = [[] for _ in range(nl)]
    for i in sorted(range(len(work)), key=lambda i: (-work[i], i)):
        k = min(range(nl), key=lambda k: (load[k], k))
        out[k].append(i)
        load[k] += work[i]
    return out


class BatchCorrelator:
    """Run a list of ``BatchFile`` through unpack -> IPFB -> PFB -> xcorr.

    lanes: concurrent CUDA streams; tune: run the FFT radix autotuner for the
    time-axis lengths of the batch first; vis_to_host: also copy every file's
    visibilities into pinned host tensors at the end of each run."""

    def __init__(self, files: Sequence[BatchFile], lanes: int = 4, tune: bool = True, vis_to_host: bool = False):
        if not files:
            raise ValueError("empty batch")
        self.files: List[BatchFile] = list(files)
        self.tuned = autotune.tune_configs((f.acclen, f.cut, f.osamp) for f in self.files) if tune else {}
        self.lanes = assign_lanes([f.spectra for f in self.files], lanes)
        # create the streams lane by lane, moving each onto the lane's shared
        # workspace right away (only one stream's own scratch exists at a time)
        self.sc: List[Optional[StreamCorrelator]] = [None] * len(self.files)
        self.workspaces: List[Optional[torch.Tensor]] = []
        for lane in self.lanes:
            ws, members = None, []
            for i in lane:
                f = self.files[i]
                choice = self.tuned.get((f.acclen, f.cut, f.osamp))
                if choice is not None:
                    autotune.apply(choice)
                sc = StreamCorrelator(f.nant, f.channels, f.chanstart, f.chanend, f.acclen, f.nchunks, f.nblock,
                                      f.osamp, f.cut, f.filt_thresh, f.ntap, nchan_raw=f.nchan_raw, bits=f.bits)
                self.sc[i] = sc
                need = sc.workspace_bytes()
                if need < 0:
                    continue  # keeps state in its scratch: stays on its own buffers
                if ws is None or ws.numel() < need:
                    ws = torch.empty(need, dtype=torch.uint8, device=f.raw.device)
                    for j in members:
                        self.sc[j].set_workspace(ws)
                sc.set_workspace(ws)
                members.append(i)
            self.workspaces.append(ws)
        if self.tuned:
            autotune.set_time_filter(autotune.DEFAULT_MODE, autotune.DEFAULT_ROW_TILE)  # defaults for later streams
        self.streams = [torch.cuda.Stream(device=self.files[0].raw.device) for _ in self.lanes]
        self.vis_host = None
        if vis_to_host:
            self.vis_host = [torch.empty(sc.vis_device().shape, dtype=torch.complex64, pin_memory=True)
                             for sc in self.sc]
        self.graph: Optional[torch.cuda.CUDAGraph] = None

    # ------------------------------------------------------------------
    @property
    def spectra(self) -> int:
        return sum(f.spectra for f in self.files)

    @property
    def h2d_bytes(self) -> int:
        return sum(f.host.numel() for f in self.files if f.host is not None)

    @property
    def d2h_bytes(self) -> int:
        return 0 if self.vis_host is None else sum(v.numel() * 8 for v in self.vis_host)

    def kernel_launches(self) -> int:
        """Kernels of the last eager run (a graph replays the same set)."""
        return sum(sc.kernel_launches() for sc in self.sc)

    def _enqueue(self, io: bool):
        """Issue one pass over every file, lanes forked from and joined back
        into the current stream; io adds the host copies (packets in from
        each file's pinned ``host`` tensor, visibilities out)."""
        cur = torch.cuda.current_stream()
        for lane, s in zip(self.lanes, self.streams):
            s.wait_stream(cur)
            with torch.cuda.stream(s):
                for i in lane:
                    f, sc = self.files[i], self.sc[i]
                    if io and f.host is not None:
                        f.raw.copy_(f.host, non_blocking=True)
                    sc.reset()
                    for j in range(f.nchunks):
                        sc.push(f.raw, j, f.spec_map, final=(j == f.nchunks - 1))
                    if io and self.vis_host is not None:
                        self.vis_host[i].copy_(sc.vis_device(), non_blocking=True)
        for s in self.streams:
            cur.wait_stream(s)

    def capture(self):
        """Run once eagerly (tables, attributes, launch counts), then capture
        the pass into CUDA graphs used by later ``run`` calls: one on the
        device-resident packets, and one with the host copies when any file
        has a host tensor or vis_to_host was asked for."""
        self._enqueue(io=True)
        torch.cuda.synchronize()
        self._launches = self.kernel_launches()
        self.graphs = {}
        modes = [False] + ([True] if self.h2d_bytes or self.vis_host is not None else [])
        for io in modes:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._enqueue(io)
            self.graphs[io] = g
        torch.cuda.synchronize()
        self.graph = self.graphs[False]
        return self

    def run(self, io: bool = True):
        """One pass over the batch on the current stream (graph replay once
        captured).  io=False skips the host copies."""
        io = bool(io) and bool(self.h2d_bytes or self.vis_host is not None)
        g = getattr(self, "graphs", {}).get(io)
        if g is not None:
            g.replay()
        else:
            self._enqueue(io)

    def launches_per_run(self) -> int:
        return getattr(self, "_launches", None) or self.kernel_launches()

    def vis(self, i: int) -> torch.Tensor:
        """Device visibilities of file i: (njobs, M, M, nq) complex64."""
        return self.sc[i].vis_device()

    def close(self):
        self.graph = None
        self.graphs = {}
        for sc in self.sc:
            sc.close()
        self.workspaces = []


# ---------------------------------------------------------------------------
# The uneven synthetic batch: files of mixed formats and sizes.

@dataclass
class FileSpec:
    name: str
    bits: int
    nchan: int
    chan0: int
    nspec: int
    osamp: int
    acclen: int
    cut: int
    seed: int
    nant: int = 2

    @property
    def nblock(self) -> int:
        """One job per chunk: acclen*4096 samples / (4096*osamp) per block."""
        return max(self.acclen // self.osamp, 1)


def uneven_batch_specs(seed: int = 2024, nfiles: int = 24, n1bit: int = 8, nchans=(32, 64, 128, 512),
                       log2_len=(14, 19), osamps=(16, 64), acclens=((1 << 14, 40), (1 << 15, 80))) -> List[FileSpec]:
    """Seeded file list: nfiles files, n1bit of them 1-bit, channel counts
    drawn from nchans, lengths uniform in [2^lo, 2^hi] spectra, osamp from
    osamps.  Chunking: the larger (acclen, cut) of `acclens` whose acclen
    leaves at least two chunks, else the smallest."""
    rng = np.random.default_rng(seed)
    bits = np.array([1] * n1bit + [4] * (nfiles - n1bit))
    rng.shuffle(bits)
    acc = sorted(acclens)
    out = []
    for k in range(nfiles):
        nchan = int(rng.choice(nchans))
        chan0 = 2 * int(rng.integers(0, (2048 - nchan) // 2 + 1))
        nspec = int(rng.integers(1 << log2_len[0], (1 << log2_len[1]) + 1))
        osamp = int(rng.choice(osamps))
        a, c = acc[0]
        for aa, cc in acc:
            if nspec >= 2 * aa:
                a, c = aa, cc
        out.append(FileSpec(f"file{k:02d}_{int(bits[k])}bit_{nchan}ch", int(bits[k]), nchan, chan0, nspec, osamp, a,
                            c, seed * 1000 + k))
    return out


def synth_packets(spec: FileSpec, device) -> torch.Tensor:
    """(nant, nspec, row_bytes) uint8 packets of `spec` made on `device`:
    4-bit = clip(rint(N(0, 2.5)), -7, 7) nibbles (real high, imag low, pol0
    then pol1 per channel); 1-bit = independent random sign bits."""
    g = torch.Generator(device=device)
    g.manual_seed(spec.seed)
    if spec.bits == 4:
        shape = (spec.nant, spec.nspec, spec.nchan, 2)

        def nib():
            v = torch.randn(shape, generator=g, device=device, dtype=torch.float32) * 2.5
            return torch.clamp(torch.round(v), -7, 7).to(torch.int16) & 15
        re, im = nib(), nib()
        return ((re << 4) | im).to(torch.uint8).reshape(spec.nant, spec.nspec, 2 * spec.nchan).contiguous()
    return torch.randint(0, 256, (spec.nant, spec.nspec, spec.nchan // 2), generator=g, device=device,
                         dtype=torch.uint8)


def files_from_specs(specs: Sequence[FileSpec], device, host_copies: bool = False) -> List[BatchFile]:
    """BatchFile per spec with synthetic packets (and pinned host copies)."""
    files = []
    for sp in specs:
        raw = synth_packets(sp, device)
        host = None
        if host_copies:
            host = torch.empty(raw.shape, dtype=torch.uint8, pin_memory=True)
            host.copy_(raw)
        files.append(BatchFile(raw=raw, channels=np.arange(sp.chan0, sp.chan0 + sp.nchan), bits=sp.bits,
                               acclen=sp.acclen, cut=sp.cut, osamp=sp.osamp, nblock=sp.nblock, host=host,
                               name=sp.name))
    return files
