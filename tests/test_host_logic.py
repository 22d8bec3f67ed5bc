"""Host-side logic of the streaming driver: job planner, band edges, and the
FP64 oracle's streaming semantics.  CPU only."""
import numpy as np
import pytest

from albatros_axion_detection_gb300.stream import JobChunkPlanner, band_edges
from oracle import pfb_oracle as po
from tests.golden import gen


@pytest.mark.parametrize("nchunks,lchunk,nblock,lblock", [
    (32, 512 * 262144, 512, 262144), (5, 3, 2, 1), (7, 10, 3, 4), (1, 100, 10, 16), (3, 1, 4, 2), (10, 7, 1, 5)])
def test_plan_chunks_matches_oracle(nchunks, lchunk, nblock, lblock):
    assert JobChunkPlanner.plan_chunks(nchunks, lchunk, nblock, lblock, 4) == po.plan_chunks(nchunks, lchunk, nblock, lblock, 4)


def test_plan_chunks_config3():
    jobs = JobChunkPlanner.plan_chunks(32, 2 ** 15 * 4096, 512, 4096 * 64, 4)
    assert len(jobs) == 31 and jobs[0] == (0, 2) and jobs[-1] == (31, 32)


def test_band_edges():
    ch = np.arange(100, 164)
    assert band_edges(ch, 0, 64, 64) == (100 * 64, 164 * 64)
    assert band_edges(ch, 3, 10, 4) == (103 * 4, 110 * 4)
    assert band_edges(ch, 0, 64, 64) == po.band_edges(ch, 0, 64, 64)


def test_oracle_chain_is_linear_in_inputs():
    """Streaming FP64 chain: antenna-0 autos do not depend on antenna 1's data."""
    raw = gen.raw_4bit(seed=9, nspec=2 * 96, nchan=4, nant=2)
    kw = dict(acclen=96, nchunks=2, nblock=4, chanstart=0, chanend=4, osamp=1, cut=8)
    v1, _ = po.repfb_xcorr_avg(raw, np.arange(10, 14), **kw)
    raw2 = raw.copy()
    raw2[1] = gen.raw_4bit(seed=10, nspec=2 * 96, nchan=4)
    v2, _ = po.repfb_xcorr_avg(raw2, np.arange(10, 14), **kw)
    np.testing.assert_allclose(v1[:2, :2], v2[:2, :2], rtol=1e-12, atol=1e-12)
    assert not np.allclose(v1[2:, 2:], v2[2:, 2:])


def test_candidate_radix_orders():
    from albatros_axion_detection_gb300 import autotune
    for n in (8232, 576, 16464, 4096, 1000):
        c = autotune.candidate_orders(n, limit=40)
        assert c and len(c) == len(set(c)) and len(c) <= 40
        assert all(int(np.prod(r)) == n and set(r) <= {2, 3, 4, 5, 7, 8} for r in c)
        assert len(c[0]) == min(len(r) for r in c)  # fewest passes first
    assert autotune.candidate_orders(11 * 64) == []
    assert autotune.factorise(8232) == {2: 3, 3: 1, 5: 0, 7: 3}


def test_uneven_batch_specs():
    from albatros_axion_detection_gb300 import batch
    specs = batch.uneven_batch_specs(seed=2024)
    assert specs == batch.uneven_batch_specs(seed=2024)  # seeded
    assert len(specs) == 24 and sum(s.bits == 1 for s in specs) == 8
    for s in specs:
        assert s.nchan in (32, 64, 128, 512) and s.osamp in (16, 64)
        assert 2 ** 14 <= s.nspec <= 2 ** 19 and s.chan0 % 2 == 0 and s.chan0 + s.nchan <= 2048
        assert (s.acclen, s.cut) in ((2 ** 14, 40), (2 ** 15, 80)) and s.nspec >= s.acclen
        assert s.nblock * s.osamp == s.acclen


def test_assign_lanes_balances_work():
    from albatros_axion_detection_gb300 import batch
    work = [10, 3, 7, 7, 2, 9, 1]
    lanes = batch.assign_lanes(work, 3)
    assert sorted(i for l in lanes for i in l) == list(range(len(work)))
    loads = [sum(work[i] for i in l) for l in lanes]
    assert max(loads) - min(loads) <= max(work)
    assert batch.assign_lanes([5, 5], 8) == [[0], [1]]


@pytest.mark.parametrize("k", range(4))
def test_missing_fraction_matches_reference(golden_int, k):
    """Per-job missing percentage vs the reference's own tracker and buffer
    bookkeeping run on the same per-chunk counts (tests/golden/make_golden.py:
    missing_cases), including jobs filled by the carried overflow alone."""
    from albatros_axion_detection_gb300.output import missing_fraction
    nant, acclen, nblock, osamp, nchunks = golden_int[f"mf{k}_cfg"]
    got = missing_fraction(golden_int[f"mf{k}_present"], int(acclen), int(nblock), int(osamp))
    np.testing.assert_allclose(got, golden_int[f"mf{k}_out"], rtol=0, atol=1e-12)


def test_chunk_presence_and_npz_roundtrip(tmp_path):
    import torch
    from albatros_axion_detection_gb300 import output
    sm = np.arange(3 * 40, dtype=np.int32).reshape(3, 40)
    sm[0, 5:9] = -1
    sm[2, 30:] = -1
    for m in (sm, torch.from_numpy(sm)):
        np.testing.assert_array_equal(output.chunk_presence(m, 3, 4, 10), [[6, 10, 10, 10], [10] * 4, [10, 10, 10, 0]])
    assert output.chunk_presence(None, 2, 3, 8).tolist() == [[8] * 3] * 2
    assert output.missing_fraction(np.full((2, 5), 64), 64, 5, 4).max() == 0.0
    vis = (np.arange(2 * 2 * 3 * 4) + 1j).astype(np.complex64).reshape(2, 2, 3, 4)
    vis[0, 1, 2, 3] = np.nan
    path = output.write_run(str(tmp_path), 1721800000, 2048, 64, 7, 10, 20, vis, np.ones((1, 4)), np.arange(3))
    assert path.endswith("stream_xcorr_all_ant_4bit_1721800000_2048_64_7_10_20.npz")
    v, mf, ch = output.load_xcorr_npz(path)
    assert v.mask.sum() == 1 and v.mask[0, 1, 2, 3]
    np.testing.assert_array_equal(v.filled(0), np.nan_to_num(vis, nan=0))
    with np.load(path) as f:
        assert sorted(f.files) == ["chans", "data", "mask", "missing_fraction"]


@pytest.mark.parametrize("name", ["wrap", "gaps4", "gaps1"])
def test_ingest_host_side_matches_reference(golden_int, name, tmp_path):
    """Header fields, wrap-fixed spectrum numbers, the overflow counter across
    files and the run's start, as the reference's Baseband and iterator."""
    from albatros_axion_detection_gb300 import ingest
    sc = gen.baseband_scenarios()[name]
    paths = gen.write_scenario(sc, str(tmp_path), name)
    for k, p in enumerate(paths):
        h, pk, sn, over = ingest.read_packets(p)
        g = golden_int[f"bb_{name}_{k}_hdr"]
        assert (h.header_bytes, h.bytes_per_packet, h.length_channels, h.spectra_per_packet, h.bit_mode,
                h.num_packets) == tuple(int(x) for x in g)
        np.testing.assert_array_equal(h.channels, golden_int[f"bb_{name}_{k}_chans"])
        np.testing.assert_array_equal(sn, golden_int[f"bb_{name}_{k}_specnum"])
        assert over == bool(golden_int[f"bb_{name}_{k}_overflowed"])
        assert pk.shape == (h.num_packets, h.bytes_per_packet)
        assert ingest.get_header(p)["spectra_per_packet"] == h.spectra_per_packet
    af = ingest.plan_antenna(paths, 0, sc["idxstart"], sc["acclen"] * sc["nchunks"])
    assert af.start == int(golden_int[f"bfi_{name}_start"])
    ctr = np.cumsum([0] + [int(golden_int[f"bb_{name}_{k}_overflowed"]) for k in range(len(paths))])
    for k, sn in enumerate(af.specnums):
        np.testing.assert_array_equal(sn, golden_int[f"bb_{name}_{k}_specnum"] + ctr[k] * (1 << 32))


def test_plan_antenna_reads_only_files_in_the_run(tmp_path, monkeypatch):
    """A file whose first spectrum lies past the run is only peeked at: its
    packets are not read and it is not part of the antenna's rows."""
    from albatros_axion_detection_gb300 import ingest
    chans = gen.header_channels(100, 4, 4)
    rng = np.random.default_rng(1)
    paths = []
    for k, s0 in enumerate((1000, 1030, 5000)):  # the run [1000, 1060) ends inside a gap before the third file
        p = str(tmp_path / f"f{k}.raw")
        gen.write_baseband(p, s0 + 3 * np.arange(8), 3, chans, 4,
                           rng.integers(0, 256, (8, 3 * len(chans)), dtype=np.uint8))
        paths.append(p)
    assert ingest.first_specnum(paths[2]) == 5000
    read = []
    real = ingest.read_packets
    monkeypatch.setattr(ingest, "read_packets", lambda p, *a, **k: (read.append(p), real(p, *a, **k))[1])
    af = ingest.plan_antenna(paths, 0, 0, 60)
    assert read == paths[:2] and af.paths == paths[:2]
    assert af.row0 == [0, 24] and af.rows == 48 and af.npkt == [8, 8]
    empty = str(tmp_path / "empty.raw")
    gen.write_baseband(empty, np.zeros(0, np.int64), 3, chans, 4, np.zeros((0, 3 * len(chans)), np.uint8))
    assert ingest.first_specnum(empty) is None


def test_fix_wraps_rejects_two_wraps():
    from albatros_axion_detection_gb300 import ingest
    s, over = ingest.fix_wraps(np.array([5, 9, 2, 6]))
    assert over and s.tolist() == [5, 9, 2 + (1 << 32), 6 + (1 << 32)]
    with pytest.raises(ValueError):
        ingest.fix_wraps(np.array([5, 1, 7, 2]))


def test_ingest_header_errors_and_readlen(tmp_path):
    """Malformed headers raise ValueError; readlen follows the reference
    (>= 1 packets, (0, 1) a fraction, 0 none, -1 all)."""
    from albatros_axion_detection_gb300 import ingest
    chans = gen.header_channels(100, 4, 4)
    pay = np.random.default_rng(0).integers(0, 256, (10, 3 * len(chans)), dtype=np.uint8)
    p = str(tmp_path / "ok.raw")
    gen.write_baseband(p, 10 + 3 * np.arange(10), 3, chans, 4, pay)
    for rl, n in ((-1, 10), (4, 4), (0.5, 5), (0, 0), (25, 10)):
        _, pk, sn, _ = ingest.read_packets(p, readlen=rl)
        assert pk.shape[0] == n and len(sn) == n
    blob = open(p, "rb").read()
    bad = tmp_path / "bad.raw"
    bad.write_bytes(blob[:30])  # truncated header
    with pytest.raises(ValueError):
        ingest.read_header(str(bad))
    b = bytearray(blob)
    b[32:40] = (2).to_bytes(8, "big")  # bit_mode 2
    bad.write_bytes(bytes(b))
    with pytest.raises(ValueError):
        ingest.read_header(str(bad))
    b = bytearray(blob)
    b[8:16] = (len(chans) * 3 + 5).to_bytes(8, "big")  # packet size not holding whole spectra
    bad.write_bytes(bytes(b))
    with pytest.raises(ValueError):
        ingest.read_header(str(bad))


def _replica_rank(rank, port, times, out_path):
    import os
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=len(times))
    try:
        ms = bench.replica_ms(times[rank], dist, "cpu")
        with open(f"{out_path}.{rank}", "w") as f:
            f.write(repr(ms))
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks_gloo(tmp_path):
    """bench.py's multi-replica timing on two gloo ranks: every rank reports
    the slowest rank's step time, and the job throughput counts both ranks'
    spectra."""
    import socket
    import torch.multiprocessing as mp
    import bench
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    times = [120.5, 131.25]
    out = str(tmp_path / "ms")
    mp.start_processes(_replica_rank, args=(port, times, out), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        assert float(open(f"{out}.{r}").read()) == max(times)
    assert bench.replica_ms(7.0, None, "cpu") == 7.0
    assert bench.job_throughput(2, 2 ** 21, 131.25) == pytest.approx(2 * 2 ** 21 / 0.13125)
