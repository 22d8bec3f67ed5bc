"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own code.

Run with the reference checkout at $ALBATROS_REFERENCE (or in a directory
``reference`` beside this repository's checkout).  It
  1. compiles the reference's C (src/correlations/unpacking.c,
     src/correlations/correlations_cpu.c) with oracle/build.py into oracle/_ref/
     and calls it through ctypes with the reference's own argument types
     (src/correlations/unpacking.py:25-79, src/correlations/correlations.py:22-105);
  2. imports the reference's CPU PFB module src/utils/pfb_cpu_utils.py with a
     stand-in ``numba`` module (njit = identity, prange = range; numba is not
     installed) and runs get_matft_cpu / compute_filter / cpu_ipfb / cpu_pfb.

Fixture inputs are the reference tests' hand-made arrays (built here from their
description) or seeded ``numpy.random.default_rng`` draws; seeded inputs are
regenerated by the tests from the seed and checked against a stored checksum.
The fixtures are read by tests/test_oracle_golden.py (CPU) and the GPU parity
tests; nothing reads the reference at test time.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from tests.golden import gen  # noqa: E402

REF = obuild.REF

P, I, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_short


def ref_c():
    assert obuild.build_ref(), "reference sources not found"
    up = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "lib_unpacking.so"))
    co = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "lib_correlations_cpu.so"))
    up.unpack_4bit_float.argtypes = [P, P, P, I, I, P, I, I]
    up.unpack_1bit_float.argtypes = [P, P, P, I, I, I, I, I]
    up.sortpols.argtypes = [P, P, P, I, I, I, I, S, I, I]
    up.hist_4bit.argtypes = [P, P, I, I, I, I, I]
    up.hist_1bit.argtypes = [P, P, I, I, I, I, I]
    co.avg_xcorr_4bit.argtypes = [P, P, P, I, I]
    co.avg_xcorr_4bit_2ant.argtypes = [P, P, P, P, P, ctypes.c_int64, ctypes.c_int64, I, I, I]
    co.avg_xcorr_4bit_2ant.restype = I
    co.avg_xcorr_1bit.argtypes = [P, P, P, I, ctypes.c_uint32, ctypes.c_uint32]
    co.avg_xcorr_1bit_vanvleck_2ant.argtypes = [P, P, P, P, P, P, P, P, ctypes.c_int64, ctypes.c_int64,
                                                ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, I]
    co.avg_xcorr_1bit_vanvleck_2ant.restype = I
    return up, co


def ref_unpack4(up, raw2d, r0, r1, ch, nchan):
    ch = np.ascontiguousarray(ch, dtype=np.int64)
    a = np.empty((r1 - r0, len(ch)), np.complex64)
    b = np.empty_like(a)
    up.unpack_4bit_float(raw2d.ctypes.data, a.ctypes.data, b.ctypes.data, r0, r1, ch.ctypes.data, len(ch), nchan)
    return a, b


def ref_unpack1(up, raw2d, r0, r1, c0, c1, nchan):
    a = np.empty((r1 - r0, c1 - c0), np.complex64)
    b = np.empty_like(a)
    up.unpack_1bit_float(raw2d.ctypes.data, a.ctypes.data, b.ctypes.data, r0, r1, c0, c1, nchan)
    return a, b


def ref_sortpols(up, raw2d, r0, r1, nchan, bits, c0, c1):
    nc = (c1 - c0) if bits == 4 else int(np.ceil((c1 - c0) / 4))
    a = np.empty((r1 - r0, nc), np.uint8)
    b = np.empty_like(a)
    up.sortpols(raw2d.ctypes.data, a.ctypes.data, b.ctypes.data, r0, r1, nc, nchan, bits, c0, c1)
    return a, b


def unpack_cases(up):
    out = {}
    packed = gen.fixture_4bit_packed()
    for name, ch in (("all", np.arange(10)), ("one", np.arange(3, 4)), ("two", np.array([2, 5]))):
        a, b = ref_unpack4(up, packed.reshape(-1, 20), 0, 2, ch, 10)
        out[f"u4_fix_{name}_ch"] = ch
        out[f"u4_fix_{name}_p0"], out[f"u4_fix_{name}_p1"] = a, b
    raw = gen.raw_4bit(seed=11, nspec=300, nchan=64)
    ch = np.array([0, 1, 5, 17, 18, 40, 63], dtype=np.int64)
    a, b = ref_unpack4(up, raw, 7, 291, ch, 64)
    out["u4_rand_ch"], out["u4_rand_p0"], out["u4_rand_p1"] = ch, a, b
    out["u4_rand_sum"] = gen.checksum(raw)

    p1 = gen.fixture_1bit_packed()
    a, b = ref_unpack1(up, p1.reshape(-1, 4), 0, 2, 2, 6, 8)
    out["u1_fix_p0"], out["u1_fix_p1"] = a, b
    raw1 = gen.raw_1bit(seed=12, nspec=300, nchan=64)
    a, b = ref_unpack1(up, raw1, 3, 299, 6, 40, 64)
    out["u1_rand_p0"], out["u1_rand_p1"], out["u1_rand_sum"] = a, b, gen.checksum(raw1)

    for (c0, c1) in ((2, 7), (0, 8)):
        a, b = ref_sortpols(up, p1.reshape(-1, 4), 0, 2, 8, 1, c0, c1)
        out[f"sp1_fix_{c0}_{c1}_p0"], out[f"sp1_fix_{c0}_{c1}_p1"] = a, b
    for (c0, c1) in ((0, 64), (6, 31), (10, 12)):
        a, b = ref_sortpols(up, raw1, 3, 299, 64, 1, c0, c1)
        out[f"sp1_rand_{c0}_{c1}_p0"], out[f"sp1_rand_{c0}_{c1}_p1"] = a, b
    a, b = ref_sortpols(up, raw, 7, 291, 64, 4, 5, 45)
    out["sp4_rand_p0"], out["sp4_rand_p1"] = a, b
    return out


def ref_hist(up, raw2d, r0, r1, nchan, bits, mode):
    """The reference's hist_4bit / hist_1bit (unpacking.c:7-153).  Its final
    merge loop runs k <= hist_len, one element past the histogram, so the
    buffer gets one spare element, dropped here."""
    nbins = 2 ** bits - 1
    h = np.zeros((nbins + 1) * nchan + 1, dtype=np.uint64)
    raw2d = np.ascontiguousarray(raw2d)
    fn = up.hist_4bit if bits == 4 else up.hist_1bit
    fn(raw2d.ctypes.data, h.ctypes.data, r0, r1, nchan, nbins, mode)
    return h[:-1].reshape(nbins + 1, nchan)


def hist_cases(up):
    out = {}
    packed, p1 = gen.fixture_4bit_packed(), gen.fixture_1bit_packed()
    raw, raw1 = gen.raw_4bit(seed=11, nspec=300, nchan=64), gen.raw_1bit(seed=12, nspec=300, nchan=64)
    for mode in (0, 1, -1):
        m = "b" if mode == -1 else str(mode)
        out[f"h4_fix_{m}"] = ref_hist(up, packed.reshape(-1, 20), 0, 2, 10, 4, mode)
        out[f"h4_rand_{m}"] = ref_hist(up, raw, 7, 291, 64, 4, mode)
        out[f"h1_fix_{m}"] = ref_hist(up, p1.reshape(-1, 4), 0, 2, 8, 1, mode)
        out[f"h1_rand_{m}"] = ref_hist(up, raw1, 3, 299, 64, 1, mode)
    return out


def missing_cases():
    """missing_fraction of the reference's streaming driver
    (scripts/xcorr/helper_gpu_stream_clean.py): its own ProcessingConfig,
    BufferSizes, BufferManager, MissingDataTracker, JobChunkPlanner and
    _process_antenna_pol, taken from the source with ``cupy`` bound to NumPy,
    driven by the job loop of its repfb_xcorr_avg (:355-372) with the IPFB
    and make_continuous_gpu stubbed out (they do not touch the bookkeeping).
    Chunks carry only their present spectrum numbers."""
    import ast
    from dataclasses import dataclass
    from typing import List, Optional, Tuple
    path = os.path.join(REF, "albatros_analysis", "scripts", "xcorr", "helper_gpu_stream_clean.py")
    tree = ast.parse(open(path).read())
    keep = {"ProcessingConfig", "BufferSizes", "BufferManager", "MissingDataTracker", "JobChunkPlanner",
            "_process_antenna_pol"}
    mod = ast.Module(body=[n for n in tree.body if getattr(n, "name", None) in keep], type_ignores=[])

    class _Bdc:
        @staticmethod
        def make_continuous_gpu(pol, specnums, start, channels, nspec, nchans=2049):
            return np.zeros((nspec, nchans), np.complex64)

    ns = dict(np=np, cp=np, dataclass=dataclass, List=List, Tuple=Tuple, Optional=Optional, bdc=_Bdc)
    exec(compile(mod, path, "exec"), ns)
    out = {}
    rng = np.random.default_rng(77)
    for k, (nant, acclen, nblock, osamp, nchunks) in enumerate([(2, 64, 5, 4, 13), (3, 16, 8, 16, 20),
                                                                (2, 32, 3, 64, 17), (1, 128, 40, 4, 9)]):
        cfg = ns["ProcessingConfig"](acclen=acclen, pfb_size=0, nchunks=nchunks, nblock=nblock, chanstart=0,
                                     chanend=4, osamp=osamp, cut=2)
        sizes = ns["BufferSizes"].from_config(cfg)
        present = rng.integers(acclen // 2, acclen + 1, (nant, nchunks))
        present[:, rng.random(nchunks) < 0.3] = acclen  # some complete chunks
        jobs = [tuple({"specnums": np.arange(present[a, c]), "pol0": None, "pol1": None} for a in range(nant))
                for c in range(nchunks)]

        class _Ipfb:
            def process_chunk(self, chunk, pol_idx, start_specnum, cut_pol):
                return np.zeros(sizes.lchunk, np.float32)

        bm = ns["BufferManager"](cfg, sizes, nant)
        plan = ns["JobChunkPlanner"].plan_chunks(nchunks, sizes.lchunk, nblock, sizes.lblock, cfg.ntap)
        tracker = ns["MissingDataTracker"](nant, len(plan))
        for job_idx, (c0, c1) in enumerate(plan):
            bm.reset_overlap_region()
            sub = jobs[c0:c1] if c1 is not None else jobs[c0:]
            for a in range(nant):
                for p in range(cfg.npol):
                    ns["_process_antenna_pol"](a, p, sub, bm, _Ipfb(), tracker, job_idx, 0, np.arange(4), cfg,
                                               sizes, False)
        out[f"mf{k}_cfg"] = np.array([nant, acclen, nblock, osamp, nchunks])
        out[f"mf{k}_present"] = present
        out[f"mf{k}_out"] = tracker.missing_fraction
    return out


def ingest_cases():
    """Baseband / BasebandFileIterator of the reference
    (src/correlations/baseband_data_classes.py), taken from the source with
    xp = NumPy and numba's njit / prange as identity / range, run on the
    scenario files of gen.baseband_scenarios().  The iterator's float loader
    unpacks nothing here: each chunk row it fills is tagged (row in file,
    file index), so the fixture records which file row serves each present
    spectrum, beside the chunk's spectrum numbers.  Also each file's header
    fields and wrap-fixed per-packet spectrum numbers as Baseband reads them."""
    import ast
    import contextlib
    import io as _io
    import struct
    import time
    import types
    path = os.path.join(REF, "albatros_analysis", "src", "correlations", "baseband_data_classes.py")
    tree = ast.parse(open(path).read())
    keep = {"fill_arr_cpu", "fill_arr", "add_constant_cpu", "add_constant", "get_rows_from_specnum", "Baseband",
            "BasebandFloat", "BasebandFileIterator"}
    mod = ast.Module(body=[n for n in tree.body if getattr(n, "name", None) in keep], type_ignores=[])
    nb = types.SimpleNamespace(njit=lambda *a, **k: (lambda f: f), prange=range)
    ns = dict(np=np, xp=np, nb=nb, os=os, struct=struct, time=time, unpk=None)
    exec(compile(mod, path, "exec"), ns)
    files_by_name = {}

    class TaggedFloat(ns["BasebandFloat"]):
        def __init__(self, file_name, *a, **k):
            super().__init__(file_name, *a, **k)
            self._fid = files_by_name[file_name]

        def _unpack(self, rowstart, rowend):
            rows = np.arange(rowstart, rowend, dtype=np.float32)[:, None] + 1j * np.float32(self._fid)
            v = np.broadcast_to(rows, (rowend - rowstart, len(self.channel_idxs))).astype(np.complex64)
            return v, v

    ns["BasebandFloat"] = TaggedFloat
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, sc in gen.baseband_scenarios().items():
            paths = gen.write_scenario(sc, d, name)
            files_by_name.clear()
            files_by_name.update({p: k for k, p in enumerate(paths)})
            with contextlib.redirect_stdout(_io.StringIO()):
                for k, p in enumerate(paths):
                    b = ns["Baseband"](p)
                    out[f"bb_{name}_{k}_hdr"] = np.array([b.header_bytes, b.bytes_per_packet, b.length_channels,
                                                          b.spectra_per_packet, b.bit_mode, b.num_packets])
                    out[f"bb_{name}_{k}_chans"] = np.asarray(b.channels, np.int64)
                    out[f"bb_{name}_{k}_specnum"] = np.asarray(b.spec_num, np.int64)
                    out[f"bb_{name}_{k}_overflowed"] = np.array(b._overflowed)
                it = ns["BasebandFileIterator"](paths, 0, sc["idxstart"], sc["acclen"], nchunks=sc["nchunks"],
                                                type="float")
                start0 = int(it.spec_num_start)
                sn, rows, fid, counts = [], [], [], []
                for chunk in it:
                    n = len(chunk["specnums"])
                    counts.append(n)
                    sn.append(chunk["specnums"])
                    rows.append(chunk["pol0"][:n, 0].real.astype(np.int64))
                    fid.append(chunk["pol0"][:n, 0].imag.astype(np.int64))
                    assert not chunk["pol0"][n:].any()
            out[f"bfi_{name}_start"] = np.array(start0)
            out[f"bfi_{name}_counts"] = np.array(counts)
            out[f"bfi_{name}_specnums"] = np.concatenate(sn)
            out[f"bfi_{name}_rows"] = np.concatenate(rows)
            out[f"bfi_{name}_files"] = np.concatenate(fid)
    return out


def xcorr_cases(co):
    out = {}
    d0, d1 = gen.sorted_4bit_pair(seed=21, nrows=2000, ncol=33)
    x = np.empty(33, np.complex64)
    co.avg_xcorr_4bit(d0.ctypes.data, d1.ctypes.data, x.ctypes.data, 2000, 33)
    out["x4_sum"] = x.copy()
    s0, s1 = gen.specnum_pair(seed=22, n=2000, span=2600)
    n = co.avg_xcorr_4bit_2ant(d0.ctypes.data, d1.ctypes.data, x.ctypes.data, s0.ctypes.data, s1.ctypes.data,
                               0, 0, 2000, 2000, 33)
    out["x4_2ant_sum"], out["x4_2ant_rows"] = x.copy(), n
    for nch in (32, 29):
        nb = int(np.ceil(nch / 4))
        e0, e1 = gen.sorted_1bit_pair(seed=23 + nch, nrows=1500, nbytes=nb)
        y = np.empty(nch, np.complex64)
        co.avg_xcorr_1bit(e0.ctypes.data, e1.ctypes.data, y.ctypes.data, nch, 1500, nb)
        out[f"x1_{nch}_sum"] = y
    e0, e1 = gen.sorted_1bit_pair(seed=31, nrows=2000, nbytes=8)
    F = [np.empty(32, np.float32) for _ in range(4)]
    n = co.avg_xcorr_1bit_vanvleck_2ant(e0.ctypes.data, e1.ctypes.data, *[f.ctypes.data for f in F],
                                        s0.ctypes.data, s1.ctypes.data, 0, 0, 2000, 2000, 8, 32)
    out["vv_2ant"] = np.stack(F)
    out["vv_2ant_rows"] = n
    return out


def pfb_cases():
    stub = tempfile.mkdtemp()
    os.makedirs(os.path.join(stub, "numba"))
    with open(os.path.join(stub, "numba", "__init__.py"), "w") as f:
        f.write("def njit(*a, **k):\n    return a[0] if a and callable(a[0]) else (lambda f: f)\n"
                "jit = njit\nprange = range\n")
    sys.path.insert(0, stub)
    spec = importlib.util.spec_from_file_location(
        "ref_pfb_cpu_utils", os.path.join(REF, "albatros_analysis", "src", "utils", "pfb_cpu_utils.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    out = {}
    nslice, cut = 12, 2
    matft = m.get_matft_cpu(nslice, n_workers=1)
    filt = m.compute_filter(matft, 0.45)
    dat = gen.ipfb_input(seed=41, nslice=nslice)
    res = np.empty((nslice - 2 * cut) * 4096, np.float32)
    m.cpu_ipfb(dat, res, filt.astype(np.complex64), cut=cut, n_workers=1)
    out["matft_12"], out["ipfb_12_cut2"] = matft.astype(np.complex64), res
    out["ipfb_in_sum"] = gen.checksum(dat)
    osamp, nblock = 2, 4
    win = m.sinc_hamming(4, 4096 * osamp).astype(np.float32)
    ts = gen.timestream(seed=42, n=4096 * osamp * (nblock + 3))
    out["pfb_os2"] = m.cpu_pfb(ts, win, nchan=2048 * osamp + 1, n_workers=1).astype(np.complex64)
    out["pfb_in_sum"] = gen.checksum(ts)
    return out


def main():
    up, co = ref_c()
    fx = {}
    fx.update(unpack_cases(up))
    fx.update(xcorr_cases(co))
    fx.update(hist_cases(up))
    fx.update(missing_cases())
    fx.update(ingest_cases())
    np.savez_compressed(os.path.join(HERE, "golden_int.npz"), **fx)
    np.savez_compressed(os.path.join(HERE, "golden_pfb.npz"), **pfb_cases())
    print("wrote golden_int.npz, golden_pfb.npz")


if __name__ == "__main__":
    main()
