"""GPU parity of the baseband file ingest: device spectrum rows and spectrum
map vs the reference's BasebandFileIterator (golden fixtures) and the CPU
oracle, and a file-driven streaming run vs the FP64 chain oracle."""
import numpy as np
import pytest
import torch

from oracle import ingest_oracle as ig
from oracle import pfb_oracle as po
from tests.golden import gen
from tests.test_gpu_stream import check

pytestmark = pytest.mark.gpu


def global_rows(af, files, rows):
    """(file index, row in file) -> row of the antenna's block."""
    return np.asarray(af.row0)[files] + rows


@pytest.mark.parametrize("name", ["wrap", "gaps4", "gaps1"])
def test_ingest_vs_reference_iterator(golden_int, name, tmp_path):
    from albatros_axion_detection_gb300 import ingest
    sc = gen.baseband_scenarios()[name]
    paths = gen.write_scenario(sc, str(tmp_path), name)
    acclen, nchunks = sc["acclen"], sc["nchunks"]
    raw, spec_map, ants = ingest.ingest([paths], [sc["idxstart"]], acclen * nchunks)
    af = ants[0]
    sm = spec_map[0].cpu().numpy()
    counts = golden_int[f"bfi_{name}_counts"]
    ends = np.cumsum(counts)
    for k, n in enumerate(counts):  # the chunks the reference delivered
        w = sm[k * acclen:(k + 1) * acclen]
        g = np.flatnonzero(w >= 0)
        sel = slice(ends[k] - n, ends[k])
        np.testing.assert_array_equal(af.start + k * acclen + g, golden_int[f"bfi_{name}_specnums"][sel])
        np.testing.assert_array_equal(w[g], global_rows(af, golden_int[f"bfi_{name}_files"][sel],
                                                        golden_int[f"bfi_{name}_rows"][sel]))
    # rows hold the packets' spectra bytes
    rb = raw.cpu().numpy()[0]
    for k, p in enumerate(paths):
        _, _, _, _, body = ig.read_file(p)
        n = body.size // af.header.row_bytes
        np.testing.assert_array_equal(rb[af.row0[k]: af.row0[k] + n], body.reshape(n, af.header.row_bytes))


def test_ingest_unaligned_packets_and_duplicates(tmp_path):
    """A packet size that is not a multiple of 4 (byte copy path), a repeated
    packet (the earlier row wins) and a spectrum map longer than the data."""
    from albatros_axion_detection_gb300 import ingest
    chans = gen.header_channels(10, 6, 1)  # 3 bytes per spectrum
    sn = np.array([0, 3, 6, 6, 12, 15])   # packet 3 repeats packet 2; 9..11 missing
    pay = np.random.default_rng(0).integers(0, 256, (len(sn), 3 * 3), dtype=np.uint8)
    p = str(tmp_path / "odd.raw")
    gen.write_baseband(p, sn, 3, chans, 1, pay)
    raw, spec_map, ants = ingest.ingest([[p]], [0], 30)
    assert ants[0].header.bytes_per_packet % 4 == 1
    sm = spec_map[0].cpu().numpy()
    expect = np.full(30, -1)
    for pk, s in enumerate(sn):
        for j in range(3):
            if expect[s + j] < 0:
                expect[s + j] = 3 * pk + j
    np.testing.assert_array_equal(sm, expect)
    np.testing.assert_array_equal(raw.cpu().numpy()[0][:18], pay.reshape(18, 3))


def test_file_iterator_chunks(golden_int, tmp_path):
    """The device-backed iterator yields the reference's chunks: present rows
    first (unpacked from the same bytes), zeros after, same spectrum numbers."""
    from albatros_axion_detection_gb300 import ingest
    from albatros_axion_detection_gb300.unpacking import unpack_4bit
    sc = gen.baseband_scenarios()["gaps4"]
    paths = gen.write_scenario(sc, str(tmp_path), "gaps4")
    it = ingest.BasebandFileIterator(paths, 0, sc["idxstart"], sc["acclen"], nchunks=sc["nchunks"], type="float")
    bodies = [ig.read_file(p)[4] for p in paths]
    counts, ends = golden_int["bfi_gaps4_counts"], np.cumsum(golden_int["bfi_gaps4_counts"])
    for k, chunk in enumerate(it):
        sel = slice(ends[k] - counts[k], ends[k])
        np.testing.assert_array_equal(chunk["specnums"], golden_int["bfi_gaps4_specnums"][sel])
        rows = np.stack([bodies[f].reshape(-1, 12)[r] for f, r in zip(golden_int["bfi_gaps4_files"][sel],
                                                                       golden_int["bfi_gaps4_rows"][sel])]) \
            if counts[k] else np.zeros((0, 12), np.uint8)
        e0, e1 = unpack_4bit(torch.from_numpy(rows).cuda(), 0, len(rows), np.arange(6), 6)
        n = counts[k]
        assert torch.equal(chunk["pol0"][:n], e0) and torch.equal(chunk["pol1"][:n], e1)
        assert not chunk["pol0"][n:].any()
    assert k == sc["nchunks"] - 1


def test_file_driven_stream_vs_oracle(tmp_path):
    """repfb_xcorr_avg(idxs, files, ...) from baseband files on disk vs the
    FP64 chain oracle on the same spectra placed by spectrum number."""
    from albatros_axion_detection_gb300 import ingest
    sc = gen.baseband_scenarios()["gaps4"]
    paths = gen.write_scenario(sc, str(tmp_path), "gaps4")
    acclen, nchunks, idxs = 50, 6, [13, 40]
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=8, chanstart=1, chanend=5, osamp=4, cut=10)
    vis, mf, freqs = ingest.repfb_xcorr_avg(idxs, [paths, paths], **kw)
    nspec = acclen * nchunks
    dense = np.zeros((2, nspec, 12), np.uint8)
    present = np.zeros((2, nspec), bool)
    bodies = [ig.read_file(p)[4].reshape(-1, 12) for p in paths]
    for a, i0 in enumerate(idxs):
        chunks = ig.iterate(paths, 0, i0, acclen, nchunks)
        start = i0 + ig.read_file(paths[0])[2][0]
        for s, f, r in chunks:
            dense[a, s - start] = np.stack([bodies[ff][rr] for ff, rr in zip(f, r)]) if len(s) else dense[a, :0]
            present[a, s - start] = True
    ref, (q0, q1) = po.repfb_xcorr_avg(dense, np.arange(100, 106), spec_present=present, **kw)
    assert freqs[0] == q0 and len(freqs) == q1 - q0
    check(np.asarray(vis), ref)
    from albatros_axion_detection_gb300 import output
    np.testing.assert_array_equal(mf, output.missing_fraction(present.reshape(2, nchunks, acclen).sum(-1), acclen,
                                                              8, 4))
