"""The reference's plain GPU path of the streaming chain, for the comparator arm.

BASELINE ONLY: ``bench.py`` times it beside the library, and a GPU test checks
that it computes the same visibilities as the FP64 oracle; the product package
never imports it.

The reference runs this chain as CuPy array operations around cuFFT and
cuBLAS.  CuPy cannot be installed here, so every CuPy operation is restated as
the same torch operation on the same dtypes, with the same temporaries, in the
same order, and the library calls go through ``plain_gpu_shim.cu`` (cuFFT
R2C/C2R plans with one shared work area, a cuBLAS strided-batched CGEMM with a
handle per call), the calls the reference's own wrappers make.  Paths are
inside the PhilJ0ly/albatros_axion_detection project, under
``albatros_analysis/``:

==========================  ===================================================
``unpack_4bit``             src/correlations/unpacking.py:140-155 (GPU branch
                            of unpack_4bit :193-245)
``bfi_chunk``               BasebandFileIterator.__next__
                            src/correlations/baseband_data_classes.py:614-715
                            (contiguous spectra: one read per chunk)
``make_continuous_gpu``     src/correlations/baseband_data_classes.py:48-73
``rfft`` / ``irfft``        src/utils/pycufft.py:120-161
``get_matft``               src/utils/pfb_gpu_utils.py:123-137
``calculate_filter``        src/utils/pfb_gpu_utils.py:29-36
``cupy_ipfb``               src/utils/pfb_gpu_utils.py:56-91
``cupy_pfb``                src/utils/pfb_gpu_utils.py:105-121
``avg_xcorr_all_ant_gpu``   src/correlations/correlations_gpu.py:95-121
``PlainGpuChain``           scripts/xcorr/helper_gpu_stream_clean.py:71-197
                            (BufferManager, IPFBProcessor), :233-263 (planner),
                            :295-456 (repfb_xcorr_avg, _process_antenna_pol)
==========================  ===================================================

Two departures, both forced: the fine band ends at (channels[-1]+1)*osamp when
the selection runs to the last recorded channel (the reference indexes
channels[chanend], one past the end, and raises there); and the channel map is
the original driver's (all recorded channels selected, where the two agree).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libplain_gpu.so")
SRC = os.path.join(HERE, "plain_gpu_shim.cu")


def build(arch: str = "103a") -> str:
    """Compile the cuFFT / cuBLAS shim (nvcc, host code only)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["nvcc", "-O2", "-shared", "-Xcompiler", "-fPIC", f"-gencode=arch=compute_{arch},code=sm_{arch}", SRC,
           "-o", LIB, "-lcufft", "-lcublas"]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is not built (baseline.plain_gpu.build())")
        L = ctypes.CDLL(LIB)
        P, I = ctypes.c_void_p, ctypes.c_int
        L.pg_fft_plan.argtypes = [I, I, I, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_size_t)]
        L.pg_fft_set_work.argtypes = [P, P]
        L.pg_fft_exec.argtypes = [P, P, P, P]
        L.pg_fft_destroy.argtypes = [P]
        L.pg_cgemm_strided_batched.argtypes = [P, P, P, I, I, I, I, P]
        for f in ("pg_fft_plan", "pg_fft_set_work", "pg_fft_exec", "pg_fft_destroy", "pg_cgemm_strided_batched"):
            getattr(L, f).restype = I
        _lib = L
    return _lib


def _ok(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with library status {rc}")


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class PlanCache:
    """Plans per (batch, n, type) and one work area as large as the largest
    plan's, set on a plan every time it is fetched
    (src/utils/pycufft.py:27-81)."""

    def __init__(self):
        self._plans = {}
        self._work = None
        self._work_bytes = 0

    def get(self, batch, n, kind):
        key = (int(batch), int(n), kind)
        plan = self._plans.get(key)
        if plan is None:
            h, size = ctypes.c_void_p(), ctypes.c_size_t()
            _ok(lib().pg_fft_plan(0 if kind == "R2C" else 1, key[0], key[1], ctypes.byref(h), ctypes.byref(size)),
                f"cuFFT plan {key}")
            plan = h.value
            self._plans[key] = plan
            if size.value > self._work_bytes:
                self._work_bytes = size.value
                self._work = torch.empty(max(size.value, 1), dtype=torch.uint8, device="cuda")
        _ok(lib().pg_fft_set_work(plan, self._work.data_ptr()), "cuFFT work area")
        return plan

    def close(self):
        for p in self._plans.values():
            lib().pg_fft_destroy(p)
        self._plans.clear()


_cache = PlanCache()


def rfft(inp: torch.Tensor, axis: int = 1) -> torch.Tensor:
    """Real -> complex along `axis`, unscaled (src/utils/pycufft.py:120-137)."""
    if axis != inp.dim() - 1:
        inp = inp.transpose(axis, -1)
    if not inp.is_contiguous():
        inp = inp.contiguous()
    n = inp.shape[-1]
    out = torch.empty(inp.shape[:-1] + (n // 2 + 1,), dtype=torch.complex64, device=inp.device)
    batch = inp.numel() // n
    _ok(lib().pg_fft_exec(_cache.get(batch, n, "R2C"), inp.data_ptr(), out.data_ptr(), _stream()), "R2C")
    if axis != inp.dim() - 1:
        out = out.transpose(axis, -1)
    return out


def irfft(inp: torch.Tensor, axis: int = 1) -> torch.Tensor:
    """Complex -> real along `axis`, then divided by n (src/utils/pycufft.py:139-161)."""
    if axis != inp.dim() - 1:
        inp = inp.transpose(axis, -1)
    if not inp.is_contiguous():
        inp = inp.contiguous()
    n = 2 * (inp.shape[-1] - 1)
    out = torch.empty(inp.shape[:-1] + (n,), dtype=torch.float32, device=inp.device)
    batch = out.numel() // n
    _ok(lib().pg_fft_exec(_cache.get(batch, n, "C2R"), inp.data_ptr(), out.data_ptr(), _stream()), "C2R")
    out /= n
    if axis != inp.dim() - 1:
        out = out.transpose(axis, -1)
    return out


def sinc_hamming(ntap, lblock):
    """src/utils/pfb_utils.py:4-7 (float64 on the host)."""
    n = ntap * lblock
    w = np.arange(0, n) - n / 2
    return np.hamming(n) * np.sinc(w / lblock)


def get_matft(nslice, nchan=2049, ntap=4):
    """Window matrix spectrum, float32 window (src/utils/pfb_gpu_utils.py:123-137)."""
    nn = 2 * (nchan - 1)
    win = torch.from_numpy(sinc_hamming(ntap, nn).astype(np.float32)).cuda().reshape(ntap, -1)
    mat = torch.zeros((nslice, nn), dtype=torch.float32, device="cuda")
    mat[:ntap, :] = win
    mat = mat.T.contiguous()
    return rfft(mat, axis=1)


def calculate_filter(matft, thresh):
    """src/utils/pfb_gpu_utils.py:29-36, in complex64 like the CuPy arrays."""
    filt = 1 / torch.conj(matft)
    if thresh > 0:
        a2 = torch.abs(matft) ** 2
        filt *= a2 / (thresh ** 2 + a2) * (1. + thresh ** 2)
    return filt


def cupy_ipfb(dat, filt):
    """src/utils/pfb_gpu_utils.py:56-91; returns the transposed view."""
    dd = irfft(dat, axis=1)
    dd2 = dd.T.contiguous()
    ddft = rfft(dd2, axis=1)
    ddft = ddft * filt
    res = irfft(ddft, axis=1)
    return res.T


def cupy_pfb(timestream, win, nchan=2049, ntap=4):
    """src/utils/pfb_gpu_utils.py:105-121."""
    lblock = 2 * (nchan - 1)
    nblock = timestream.numel() // lblock - (ntap - 1)
    ts = timestream.reshape(-1, lblock)
    w = win.reshape(ntap, lblock)
    y = ts[0:nblock] * w[0]
    for i in range(1, ntap):
        y += ts[i:nblock + i] * w[i]
    return rfft(y, axis=1)


def unpack_4bit(data, rowstart, rowend, channels_dev, length_channels):
    """4-bit decode with CuPy's ops and temporaries (src/correlations/unpacking.py:140-155):
    gathers, masked fix-ups (nibble > 8 -> v - 16), complex128 sum, complex64 cast."""
    d = data.reshape(-1, 2 * length_channels)
    rows = d[rowstart:rowend]

    def nib(col, hi):
        g = rows[:, col]
        v = torch.bitwise_right_shift(torch.bitwise_and(g, 0xF0), 4) if hi else torch.bitwise_and(g, 0x0F)
        v = v.to(torch.int8)
        m = v > 8
        v[m] = v[m] - 16
        return v
    c0, c1 = 2 * channels_dev, 2 * channels_dev + 1
    p0re, p0im, p1re, p1im = nib(c0, True), nib(c0, False), nib(c1, True), nib(c1, False)
    d_pol0 = (p0re.to(torch.complex128) + 1j * p0im.to(torch.complex128)).to(torch.complex64)
    d_pol1 = (p1re.to(torch.complex128) + 1j * p1im.to(torch.complex128)).to(torch.complex64)
    return d_pol0, d_pol1


def make_continuous_gpu(spec, chan_specnum, start_specnum, channels_dev, nspec, nchans=2049):
    """Zero grid, rows by (specnum - start) % nspec, columns by channel number
    (src/correlations/baseband_data_classes.py:48-73)."""
    specnum = torch.from_numpy(np.asarray(chan_specnum) - start_specnum).cuda() % nspec
    if specnum.shape[0] == nspec and channels_dev.numel() == nchans:
        return spec
    out = torch.zeros((nspec, nchans), dtype=spec.dtype, device=spec.device)
    out[specnum[:, None], channels_dev[None, :]] = spec[: len(specnum)]
    return out


def avg_xcorr_all_ant_gpu(x, nant, npol, ntime, nfreq):
    """X_f X_f^H / K per frequency via a strided-batched CGEMM, output
    (M, M, nfreq) F-ordered (src/correlations/correlations_gpu.py:95-121)."""
    M = nant * npol
    out = torch.empty((nfreq, M, M), dtype=torch.complex64, device=x.device).permute(2, 1, 0)
    _ok(lib().pg_cgemm_strided_batched(x.data_ptr(), x.data_ptr(), out.data_ptr(), M, M, ntime, nfreq, _stream()),
        "cgemm_strided_batched")
    out /= ntime
    return out


def plan_chunks(nchunks, lchunk, nblock, lblock, ntap):
    """scripts/xcorr/helper_gpu_stream_clean.py:233-263."""
    ranges, stride, need = [], nblock * lblock, (nblock + ntap - 1) * lblock
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


class PlainGpuChain:
    """repfb_xcorr_avg of scripts/xcorr/helper_gpu_stream_clean.py:295-456 over
    device-resident 4-bit packets (nant, nspec, 2*nchan_raw), all recorded
    channels selected, no missing spectra."""

    def __init__(self, nant, channels, acclen, nchunks, nblock, osamp, cut=10, filt_thresh=0.45, ntap=4):
        self.nant, self.npol = int(nant), 2
        self.channels = np.asarray(channels, dtype=np.int64)
        self.nchan_raw = self.channels.size
        self.acclen, self.nchunks, self.nblock, self.osamp = int(acclen), int(nchunks), int(nblock), int(osamp)
        self.cut, self.ntap = int(cut), int(ntap)
        self.lblock = 4096 * self.osamp
        self.szblock = (self.nblock + self.ntap - 1) * self.lblock
        self.lchunk = 4096 * self.acclen
        self.q0 = int(self.channels[0]) * self.osamp
        self.q1 = (int(self.channels[-1]) + 1) * self.osamp
        self.nchan = self.q1 - self.q0
        self.jobs = plan_chunks(self.nchunks, self.lchunk, self.nblock, self.lblock, self.ntap)
        # setup_filters_and_windows (:281-292), outside any timed region
        self.win = torch.from_numpy(sinc_hamming(self.ntap, self.lblock).astype(np.float32)).cuda()
        self.filt = calculate_filter(get_matft(self.acclen + 2 * self.cut), filt_thresh)
        self.idx_dev = torch.arange(self.nchan_raw, device="cuda")     # channel indices (BFI channel_idxs)
        self.abs_dev = torch.from_numpy(self.channels).cuda()          # channel numbers (make_continuous)
        M = self.nant * self.npol
        # BufferManager (:71-88)
        self.cut_pol = torch.zeros((self.nant, self.npol, 2 * self.cut, 2049), dtype=torch.complex64, device="cuda")
        self.pfb_buf = torch.zeros((self.nant, self.npol, self.nblock + self.ntap - 1, self.lblock),
                                   dtype=torch.float32, device="cuda")
        self.rem_buf = torch.empty((self.nant, self.npol, self.lchunk), dtype=torch.float32, device="cuda")
        self.xin = torch.empty((self.nchan, self.nblock, M), dtype=torch.complex64, device="cuda").permute(2, 1, 0)
        self.vis = np.zeros((M, M, self.nchan, len(self.jobs)), dtype=np.complex64, order="F")

    def reset(self):
        self.cut_pol.zero_()
        self.pfb_buf.zero_()
        self.rem_idx = np.zeros((self.nant, self.npol), dtype=np.int64)
        self.pfb_idx = np.zeros((self.nant, self.npol), dtype=np.int64)
        self._first = True

    # --- BasebandFileIterator.__next__ for contiguous spectra (:614-715)
    def bfi_chunk(self, raw_a, j):
        pol0 = torch.zeros((self.acclen, self.nchan_raw), dtype=torch.complex64, device="cuda")
        pol1 = torch.zeros((self.acclen, self.nchan_raw), dtype=torch.complex64, device="cuda")
        r0 = j * self.acclen
        specnums = np.arange(r0, r0 + self.acclen, dtype=np.int64)
        a, b = unpack_4bit(raw_a, r0, r0 + self.acclen, self.idx_dev, self.nchan_raw)
        pol0[0:self.acclen], pol1[0:self.acclen] = a, b
        return {"pol0": pol0, "pol1": pol1, "specnums": specnums}

    # --- IPFBProcessor.process_chunk (:178-197)
    def process_chunk(self, chunk, p, cut_pol_data):
        pol_data = torch.empty((self.acclen + 2 * self.cut, 2049), dtype=torch.complex64, device="cuda")
        pol_data[:2 * self.cut] = cut_pol_data
        pol_data[2 * self.cut:] = make_continuous_gpu(chunk[f"pol{p}"], chunk["specnums"], 0, self.abs_dev,
                                                      self.acclen)
        res = cupy_ipfb(pol_data, self.filt)[self.cut:-self.cut]
        return res.reshape(-1)  # ravel of the transposed view: a copy

    # --- BufferManager (:90-167)
    def _add_remaining(self, a, p):
        rem, pos = int(self.rem_idx[a, p]), int(self.pfb_idx[a, p])
        flat = self.pfb_buf[a, p].view(-1)
        if pos + rem > self.szblock:
            avail = self.szblock - pos
            flat[pos:] = self.rem_buf[a, p, :avail]
            over = rem - avail
            self.rem_buf[a, p, :over] = self.rem_buf[a, p, avail:rem].clone()
            self.rem_idx[a, p] = over
            self.pfb_idx[a, p] = self.szblock
            return True
        flat[pos:pos + rem] = self.rem_buf[a, p, :rem]
        self.pfb_idx[a, p] += rem
        self.rem_idx[a, p] = 0
        return False

    def _add_chunk(self, a, p, chunk):
        n, pos = chunk.numel(), int(self.pfb_idx[a, p])
        flat = self.pfb_buf[a, p].view(-1)
        if pos + n > self.szblock:
            avail = self.szblock - pos
            flat[pos:] = chunk[:avail]
            self.rem_buf[a, p, :n - avail] = chunk[avail:]
            self.rem_idx[a, p] = n - avail
            self.pfb_idx[a, p] = self.szblock
            return True
        flat[pos:pos + n] = chunk
        self.pfb_idx[a, p] = pos + n
        return pos + n == self.szblock

    # --- _process_antenna_pol (:404-456)
    def _process_antenna_pol(self, a, p, subjobs):
        if self._add_remaining(a, p):
            return
        for chunks in subjobs:
            chunk = chunks[a]
            processed = self.process_chunk(chunk, p, self.cut_pol[a, p])
            pol_data = torch.empty((self.acclen + 2 * self.cut, 2049), dtype=torch.complex64, device="cuda")
            pol_data[2 * self.cut:] = make_continuous_gpu(chunk[f"pol{p}"], chunk["specnums"], 0, self.abs_dev,
                                                          self.acclen)
            self.cut_pol[a, p] = pol_data[-2 * self.cut:]
            if self._add_chunk(a, p, processed):
                break
        if self.pfb_idx[a, p] != self.szblock:
            self.pfb_buf[a, p].view(-1)[int(self.pfb_idx[a, p]):] = 0.0

    def run(self, raw):
        """One pass over raw (nant, nspec, 2*nchan_raw) uint8 on the device;
        returns vis (M, M, nchan, njobs) complex64 on the host."""
        self.reset()
        # jobs = list(zip(*antenna_objs)): every chunk of every antenna read up front
        chunks = [[self.bfi_chunk(raw[a], j) for a in range(self.nant)] for j in range(self.nchunks)]
        for k, (c0, c1) in enumerate(self.jobs):
            if not self._first:  # reset_overlap_region (:90-98)
                tail = self.pfb_buf[:, :, -(self.ntap - 1):, :]
                if self.nblock < self.ntap - 1:  # the two row ranges overlap
                    tail = tail.clone()
                self.pfb_buf[:, :, :self.ntap - 1, :] = tail
                self.pfb_idx[:, :] = (self.ntap - 1) * self.lblock
            self._first = False
            subjobs = chunks[c0:c1]
            for a in range(self.nant):
                for p in range(self.npol):
                    self._process_antenna_pol(a, p, subjobs)
                    self.xin[a * self.npol + p, :, :] = cupy_pfb(self.pfb_buf[a, p], self.win,
                                                                 nchan=2048 * self.osamp + 1,
                                                                 ntap=self.ntap)[:, self.q0:self.q1]
            self.vis[:, :, :, k] = avg_xcorr_all_ant_gpu(self.xin, self.nant, self.npol, self.nblock,
                                                         self.nchan).cpu().numpy()
        return self.vis

    def close(self):
        _cache.close()
