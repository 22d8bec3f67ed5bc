"""Seeded synthetic inputs and the reference tests' hand-made fixtures.

Shared by tests/golden/make_golden.py (which runs the reference on them), the
CPU oracle tests and the GPU parity tests.  Rules follow the workload
description of the ALBATROS baseband benchmark: 4-bit values are
clip(rint(N(0, 2.5)), -7, 7) packed as ((re & 15) << 4) | (im & 15), one
byte per channel per pol with pol0 first; 1-bit values are signs packed as in
src/correlations/unpacking.c:207-246.
"""
from __future__ import annotations

import hashlib

import numpy as np


def checksum(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def pack_4bit(re, im) -> np.ndarray:
    re = np.asarray(re, dtype=np.int64)
    im = np.asarray(im, dtype=np.int64)
    return (((re & 15) << 4) | (im & 15)).astype(np.uint8)


def gaussian_4bit(rng, shape, sigma=2.5):
    return np.clip(np.rint(rng.normal(0.0, sigma, shape)), -7, 7).astype(np.int64)


def raw_4bit(seed: int, nspec: int, nchan: int, sigma: float = 2.5, nant: int | None = None) -> np.ndarray:
    """(nspec, 2*nchan) bytes (or (nant, nspec, 2*nchan)), Gaussian nibbles."""
    rng = np.random.default_rng(seed)
    shape = (nspec, nchan, 2) if nant is None else (nant, nspec, nchan, 2)
    b = pack_4bit(gaussian_4bit(rng, shape, sigma), gaussian_4bit(rng, shape, sigma))
    return b.reshape(shape[:-2] + (2 * nchan,))


def raw_4bit_uniform(seed: int, nspec: int, nchan: int, nant: int | None = None) -> np.ndarray:
    """Uniform random bytes: every nibble value, 0x8 included."""
    rng = np.random.default_rng(seed)
    shape = (nspec, 2 * nchan) if nant is None else (nant, nspec, 2 * nchan)
    return rng.integers(0, 256, shape, dtype=np.uint8)


def raw_1bit(seed: int, nspec: int, nchan: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(0, 256, (nspec, nchan // 2), dtype=np.uint8)


def sorted_4bit_pair(seed: int, nrows: int, ncol: int):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 256, (nrows, ncol), dtype=np.uint8),
            rng.integers(0, 256, (nrows, ncol), dtype=np.uint8))


def sorted_1bit_pair(seed: int, nrows: int, nbytes: int):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 256, (nrows, nbytes), dtype=np.uint8),
            rng.integers(0, 256, (nrows, nbytes), dtype=np.uint8))


def specnum_pair(seed: int, n: int, span: int):
    rng = np.random.default_rng(seed)
    return (np.sort(rng.choice(span, n, replace=False)).astype(np.int64),
            np.sort(rng.choice(span, n, replace=False)).astype(np.int64))


def ipfb_input(seed: int, nslice: int, nchan: int = 2049) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((nslice, nchan)) + 1j * rng.standard_normal((nslice, nchan))).astype(np.complex64)


def timestream(seed: int, n: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal(n).astype(np.float32)


def fixture_4bit_packed() -> np.ndarray:
    """Two spectra of 10 channels (src/correlations/tests/test_4bit_float_unpack.py:28-79):
    pol0 = 1-1j in row 0, 0 in row 1 except channel 3 = 4; pol1 = 7-7j in row 0,
    0 in row 1 except channel 3 = -4.  Returns (1, 40) bytes, pol0/pol1 interleaved."""
    r0 = np.vstack([np.ones(10, np.int64), np.zeros(10, np.int64)]); r0[1, 3] = 4
    i0 = np.vstack([-np.ones(10, np.int64), np.zeros(10, np.int64)])
    r1 = np.vstack([7 * np.ones(10, np.int64), np.zeros(10, np.int64)]); r1[1, 3] = -4
    i1 = np.vstack([-7 * np.ones(10, np.int64), np.zeros(10, np.int64)])
    out = np.zeros((1, 40), np.uint8)
    out[0, 0::2] = pack_4bit(r0, i0).ravel()
    out[0, 1::2] = pack_4bit(r1, i1).ravel()
    return out


def fixture_4bit_expected():
    r0 = np.vstack([np.ones(10), np.zeros(10)]); r0[1, 3] = 4
    i0 = np.vstack([-np.ones(10), np.zeros(10)])
    r1 = np.vstack([7 * np.ones(10), np.zeros(10)]); r1[1, 3] = -4
    i1 = np.vstack([-7 * np.ones(10), np.zeros(10)])
    return r0 + 1j * i0, r1 + 1j * i1


def fixture_1bit_values():
    """8 channels x 2 spectra of +-1 (src/correlations/tests/test_1bit_unpack_gpu.py:10-37)."""
    r0 = np.vstack([np.ones(8, np.int64), -np.ones(8, np.int64)]); r0[1, 3] = 1
    i0 = np.vstack([-np.ones(8, np.int64), np.ones(8, np.int64)])
    r1 = np.vstack([-np.ones(8, np.int64), np.ones(8, np.int64)]); r1[1, 3] = -1
    i1 = np.vstack([np.ones(8, np.int64), -np.ones(8, np.int64)])
    return r0, i0, r1, i1


def pack_1bit(r0, i0, r1, i1) -> np.ndarray:
    """(nspec, nchan) +-1 arrays -> (nspec, nchan/2) bytes, bit 1 <-> +1."""
    b = [(np.asarray(x) > 0).astype(np.uint8) for x in (r0, i0, r1, i1)]
    ev = (b[0][:, 0::2] << 7) | (b[1][:, 0::2] << 6) | (b[2][:, 0::2] << 5) | (b[3][:, 0::2] << 4)
    od = (b[0][:, 1::2] << 3) | (b[1][:, 1::2] << 2) | (b[2][:, 1::2] << 1) | b[3][:, 1::2]
    return (ev | od).astype(np.uint8)


def fixture_1bit_packed() -> np.ndarray:
    return pack_1bit(*fixture_1bit_values()).reshape(1, -1)


# ---------------------------------------------------------------------------
# Baseband files.  Layout of the reference's file writer
# (src/correlations/tests/generate_test_baseband.py:54-101): big-endian uint64
# [80 + 8*len(chans), bytes_per_packet, len(chans), spectra_per_packet, bits,
# have_trimble], the channel list (one entry per spectrum byte) as uint64,
# [gps_week, gps_time] uint64, [lat, lon, elev] float64; then packets of a
# big-endian uint32 spectrum number and the spectra bytes.

def header_channels(chan0: int, nchan: int, bits: int) -> np.ndarray:
    """Channel list of a contiguous band as the digitiser writes it: each
    4-bit channel twice (pol0 and pol1 bytes), every other 1-bit channel."""
    if bits == 4:
        c = np.arange(chan0, chan0 + nchan)
        return np.ravel(np.column_stack((c, c)))
    return np.arange(chan0, chan0 + nchan, 2)


def write_baseband(path: str, specnums, spp: int, chans, bits: int, payload: np.ndarray, gps_time: int = 1721800000):
    """payload: (npkt, spp * len(chans)) uint8; specnums: per packet (taken mod 2^32)."""
    chans = np.asarray(chans)
    bpp = spp * len(chans) + 4
    payload = np.asarray(payload, np.uint8).reshape(len(specnums), bpp - 4)
    pk = np.zeros(len(specnums), dtype=[("spec_num", ">u4"), ("spectra", f"{bpp - 4}u1")])
    pk["spec_num"] = np.asarray(specnums, dtype=np.int64) % (1 << 32)
    pk["spectra"] = payload
    with open(path, "wb") as f:
        np.asarray([80 + 8 * len(chans), bpp, len(chans), spp, bits, 0], dtype=">u8").tofile(f)
        np.asarray(chans, dtype=">u8").tofile(f)
        np.asarray([0, gps_time], dtype=">u8").tofile(f)
        np.asarray([0.0, 0.0, 0.0], dtype=">f8").tofile(f)
        pk.tofile(f)


def baseband_scenarios():
    """name -> dict(files=[(specnums, spp, chan0, nchan, bits, seed)], acclen, nchunks, idxstart).
    wrap: the reference's spectrum-number wrap trio (generate_test_baseband.py:
    171-179: a wrap inside file 1 with a dropped packet, file 2 continuing
    after it, a second wrap inside file 3); gaps4 / gaps1: dropped packets
    inside files and gaps between them, 4-bit and 1-bit."""
    rng = np.random.default_rng(2024)

    def drop(sn, frac):
        keep = rng.random(len(sn)) > frac
        keep[0] = True
        return np.asarray(sn)[keep]
    s1 = (1 << 32) - 10 + 5 * np.arange(7)
    wrap = dict(files=[(np.delete(s1, 2), 5, 452, 2, 4, 1), (25 + 5 * np.arange(3), 5, 452, 2, 4, 2),
                       (np.array([40, 5, 10]), 5, 452, 2, 4, 3)], acclen=10, nchunks=6, idxstart=0)
    a = 1000 + 7 * np.arange(60)
    b = a[-1] + 7 * 9 + 7 * np.arange(50)
    c = b[-1] + 7 * 3 + 7 * np.arange(70)
    gaps4 = dict(files=[(drop(a, 0.15), 7, 100, 6, 4, 4), (drop(b, 0.1), 7, 100, 6, 4, 5),
                        (drop(c, 0.2), 7, 100, 6, 4, 6)], acclen=50, nchunks=20, idxstart=13)
    d = 77 + 4 * np.arange(45)
    e = d[-1] + 4 * 5 + 4 * np.arange(40)
    gaps1 = dict(files=[(drop(d, 0.1), 4, 200, 8, 1, 7), (drop(e, 0.2), 4, 200, 8, 1, 8)], acclen=24, nchunks=12,
                 idxstart=3)
    return {"wrap": wrap, "gaps4": gaps4, "gaps1": gaps1}


def write_scenario(sc: dict, dirpath: str, name: str):
    """Write a scenario's files; returns their paths."""
    paths = []
    for k, (sn, spp, chan0, nchan, bits, seed) in enumerate(sc["files"]):
        chans = header_channels(chan0, nchan, bits)
        pay = np.random.default_rng(seed).integers(0, 256, (len(sn), spp * len(chans)), dtype=np.uint8)
        p = f"{dirpath}/{name}_{k}.raw"
        write_baseband(p, sn, spp, chans, bits, pay)
        paths.append(p)
    return paths
