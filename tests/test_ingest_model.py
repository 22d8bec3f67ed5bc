"""CPU model of the device ingest (csrc/ingest.cu) against the reference's
BasebandFileIterator (golden fixtures from
albatros_analysis/src/correlations/baseband_data_classes.py:522-715).

The host plan (ingest.plan_antenna: files, their rows in the antenna's block,
wrap-fixed spectrum numbers, the run's start) runs as in the product; the
kernels are restated in NumPy: packets_to_rows (drop each packet's 4-byte
spectrum number), spec_map_scatter (spec_map[s + j - start] = min row, the
earliest row winning like the reference's in-order read) and
unset_to_missing (unset entries become -1).  The result must give the
reference iterator's chunks: the spectrum numbers present, and for each the
file and row it came from.
"""
import numpy as np
import pytest

from oracle import ingest_oracle as ig
from tests.golden import gen

UNSET = np.iinfo(np.int32).max


def spec_map_model(af, nmap):
    m = np.full(nmap, UNSET, np.int64)
    spp = af.header.spectra_per_packet
    for row0, sn in zip(af.row0, af.specnums):
        g = (np.asarray(sn, np.int64)[:, None] + np.arange(spp)[None, :] - af.start).ravel()
        rows = row0 + np.arange(g.size)
        ok = (g >= 0) & (g < nmap)
        np.minimum.at(m, g[ok], rows[ok])
    m[m == UNSET] = -1
    return m


@pytest.mark.parametrize("name", ["wrap", "gaps4", "gaps1"])
def test_spec_map_model_gives_the_reference_chunks(golden_int, name, tmp_path):
    from albatros_axion_detection_gb300 import ingest
    sc = gen.baseband_scenarios()[name]
    paths = gen.write_scenario(sc, str(tmp_path), name)
    acclen, nchunks = sc["acclen"], sc["nchunks"]
    af = ingest.plan_antenna(paths, 0, sc["idxstart"], acclen * nchunks)
    assert af.start == int(golden_int[f"bfi_{name}_start"])
    sm = spec_map_model(af, acclen * nchunks)
    counts = golden_int[f"bfi_{name}_counts"]
    ends = np.cumsum(counts)
    for k, n in enumerate(counts):
        w = sm[k * acclen:(k + 1) * acclen]
        g = np.flatnonzero(w >= 0)
        sel = slice(ends[k] - n, ends[k])
        np.testing.assert_array_equal(af.start + k * acclen + g, golden_int[f"bfi_{name}_specnums"][sel])
        rows = np.asarray(af.row0)[golden_int[f"bfi_{name}_files"][sel]] + golden_int[f"bfi_{name}_rows"][sel]
        np.testing.assert_array_equal(w[g], rows)
    # packets_to_rows: the rows are each packet's payload, spectrum after spectrum
    for k, p in enumerate(paths):
        _, _, _, _, body = ig.read_file(p)
        pk = af.packets[k].numpy() if af.packets else None
        if pk is not None:
            np.testing.assert_array_equal(pk[:, 4:].reshape(-1), body.reshape(-1))


def test_duplicate_spectrum_numbers_keep_the_earliest_row():
    """A repeated packet maps to its first occurrence (atomicMin)."""
    from types import SimpleNamespace
    af = SimpleNamespace(header=SimpleNamespace(spectra_per_packet=3), start=0, row0=[0],
                         specnums=[np.array([0, 3, 6, 6, 12, 15])])
    sm = spec_map_model(af, 30)
    expect = np.full(30, -1)
    for pk, s in enumerate(af.specnums[0]):
        for j in range(3):
            if expect[s + j] < 0:
                expect[s + j] = 3 * pk + j
    np.testing.assert_array_equal(sm, expect)
