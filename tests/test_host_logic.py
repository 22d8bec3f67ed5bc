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
