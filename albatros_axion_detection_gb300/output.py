"""Output side of a streaming correlation run: the per-job missing-data
percentage, NaN masking of the visibilities and the ``.npz`` product.

Reference: MissingDataTracker (albatros_analysis/scripts/xcorr/
helper_gpu_stream_clean.py:200-226) fed from _process_antenna_pol (:405-456)
while BufferManager (:71-167) fills the PFB buffer job by job (jobs from
JobChunkPlanner.plan_chunks :233-263); the masking of repfb_xcorr_avg
(:399-402); the writer of scripts/xcorr/xcorr_gpu_cpu.py:115-118.

The tracker's result depends only on how many spectra of each chunk were
present and on the buffer geometry, never on sample values, so it is
computed here on the host from per-chunk counts (the device run reads the
same gaps through its spectrum map).  Host logic only: no GPU work.
"""
from __future__ import annotations

import os
from typing import List, Optional, Sequence, Tuple

import numpy as np


def _plan(nchunks: int, lchunk: int, nblock: int, lblock: int, ntap: int) -> List[Tuple[int, int]]:
    from .stream import JobChunkPlanner
    return [(a, nchunks if b is None else b) for a, b in JobChunkPlanner.plan_chunks(nchunks, lchunk, nblock,
                                                                                    lblock, ntap)]


def missing_fraction(present, acclen: int, nblock: int, osamp: int, ntap: int = 4) -> np.ndarray:
    """Missing-data percentage per (antenna, job), as the reference's tracker.

    present: (nant, nchunks) spectra present in each acclen-spectrum chunk.
    A chunk enters the tracker with 100 * (1 - present / acclen) and a life
    of ((fill + lchunk) // lblock) % nblock + 1 jobs, fill being the PFB
    buffer's fill position (samples) when the chunk arrives; each job's value
    is the mean over the live entries, after which every entry loses one job
    of life.  A job whose buffer is already full from the previous job's
    overflow takes no chunk and keeps 0 (the reference returns early there,
    :416-419), its entries keeping their life.
    """
    pres = np.asarray(present, dtype=np.float64)
    if pres.ndim != 2:
        raise ValueError("present must be (nant, nchunks)")
    nant, nchunks = pres.shape
    lblock, lchunk = 4096 * int(osamp), 4096 * int(acclen)
    szblock = (int(nblock) + int(ntap) - 1) * lblock
    jobs = _plan(nchunks, lchunk, int(nblock), lblock, int(ntap))
    pct = (1.0 - pres / float(acclen)) * 100.0
    out = np.zeros((nant, len(jobs)), dtype=np.float64)
    live: List[List[int]] = []  # [chunk, jobs of life left], the same for every antenna
    fill, rem = 0, 0
    for j, (c0, c1) in enumerate(jobs):
        if j > 0:
            fill = (int(ntap) - 1) * lblock  # the overlap blocks kept from the previous job
        if fill + rem > szblock:  # the carried overflow alone fills the buffer
            rem -= szblock - fill
            fill = szblock
            continue
        fill, rem = fill + rem, 0
        for c in range(c0, c1):
            live.append([c, (fill + lchunk) // lblock % int(nblock) + 1])
            end = fill + lchunk
            if end >= szblock:
                rem, fill = end - szblock, szblock
                break
            fill = end
        if live:
            out[:, j] = pct[:, [c for c, _ in live]].mean(axis=1)
            for e in live:
                e[1] -= 1
            live = [e for e in live if e[1] > 0]
    return out


def chunk_presence(spec_map, nant: int, nchunks: int, acclen: int) -> np.ndarray:
    """(nant, nchunks) spectra present per chunk from a device or host
    spectrum map (row g of antenna a present when spec_map[a, g] >= 0);
    None means every spectrum is present.

    Reference: the per-chunk counts MissingDataTracker keeps (scripts/xcorr/helper_gpu_stream_clean.py:200-226)."""
    if spec_map is None:
        return np.full((nant, nchunks), acclen, dtype=np.int64)
    m = spec_map[:, : nchunks * acclen]
    if hasattr(m, "cpu"):  # torch tensor: count on its device, bring back nant*nchunks numbers
        return (m >= 0).reshape(nant, nchunks, acclen).sum(-1).cpu().numpy().astype(np.int64)
    return (np.asarray(m) >= 0).reshape(nant, nchunks, acclen).sum(-1).astype(np.int64)


def mask_invalid(vis) -> np.ma.MaskedArray:
    """NaN/inf-masked visibilities (numpy.ma.masked_invalid, as :399)."""
    return np.ma.masked_invalid(vis)


def xcorr_npz_name(init_t, acclen: int, osamp: int, nchunks: int, chanstart: int, chanend: int) -> str:
    """File name of the streaming product (xcorr_gpu_cpu.py:113)."""
    return f"stream_xcorr_all_ant_4bit_{init_t}_{acclen}_{osamp}_{nchunks}_{chanstart}_{chanend}.npz"


def save_xcorr_npz(path: str, vis, missing: np.ndarray, chans: Sequence[int]) -> str:
    """Write data / mask / missing_fraction / chans as xcorr_gpu_cpu.py:116
    does; vis may be a masked array or a plain one (then NaNs are masked)."""
    v = vis if isinstance(vis, np.ma.MaskedArray) else mask_invalid(vis)
    mask = np.ma.getmaskarray(v)
    np.savez(path, data=np.ma.getdata(v), mask=mask, missing_fraction=np.asarray(missing), chans=np.asarray(chans))
    return path if path.endswith(".npz") else path + ".npz"


def load_xcorr_npz(path: str) -> Tuple[np.ma.MaskedArray, np.ndarray, np.ndarray]:
    """(vis as a masked array, missing_fraction, chans) from a saved product.

    Reference: the product of scripts/xcorr/xcorr_gpu_cpu.py:113-118."""
    with np.load(path) as f:
        return np.ma.MaskedArray(f["data"], mask=f["mask"]), f["missing_fraction"], f["chans"]


def write_run(outdir: str, init_t, acclen: int, osamp: int, nchunks: int, chanstart: int, chanend: int, vis,
              missing: np.ndarray, chans: Sequence[int], name: Optional[str] = None) -> str:
    """Save a run under outdir with the reference's file name; returns the path.

    Reference: scripts/xcorr/xcorr_gpu_cpu.py:113-118."""
    path = os.path.join(outdir, name or xcorr_npz_name(init_t, acclen, osamp, nchunks, chanstart, chanend))
    return save_xcorr_npz(path, vis, missing, chans)
