"""CPU model of the fused time stage's block bookkeeping, swept over many
stream geometries.

Restates, from csrc/chain.cu (stream_push) and csrc/fir.cu (launch_iir_t,
fir_item, fold_item_blocks, y_edges), which fine blocks a push completes,
how a column's kept rows are cut into segments (items), which segment folds
which block, and which y rows (staged in shared memory) each fold reads.
Checks, for every push of every geometry:
  * the segments fold each completed block exactly once;
  * every y row a fold reads is one the item holds: the previous chunk's
    tail (first segment), a row the item computed, or the zero padding after
    the stream's end (last segment of the final push);
  * the tail kept for the next chunk is made of rows the item holds;
  * blocks of a push that is not the final one only read rows that exist;
  * no push produces more blocks than the stream's W buffer holds (the final
    push skips the all-zero blocks that start past the end of the data).
The fine blocks follow the reference's PFB buffer (ntap = 4 blocks of osamp
rows each; albatros_analysis/scripts/xcorr/helper_gpu_stream_clean.py:71-167).
"""
import numpy as np
import pytest

NTHREADS, NTAP = 256, 4
TILES = [(21, 2), (21, 4), (41, 1), (41, 2)]  # (rows per thread U, exchanged states D)


def segment_rows(U, D, O):
    """New kept rows per item (launch_iir_t): whole fold rounds when one fits."""
    R = (NTHREADS - 2 * D) * U
    smax, rnd = R - 4 * O, NTHREADS * O
    return R, (smax // rnd * rnd if smax >= rnd else smax)


def items(acclen, S, O):
    nseg = max(1, -(-acclen // S))
    for seg in range(nseg):
        s0 = seg * S
        s1 = min(s0 + S, acclen)
        first, last = seg == 0, s0 + S >= acclen
        ylo = 0 if first else s0 - 4 * O
        yield dict(s0=s0, s1=s1, first=first, last=last, ylo=ylo, nrows=s1 - ylo)


def fold_range(it, S, O, row0, nb):
    def first_ending_at_or_after(r):
        num = r - 4 * O + 1 - row0
        b = 0 if num <= 0 else -(-num // O)
        return min(b, nb)
    b0 = 0 if it["first"] else first_ending_at_or_after(it["s0"])
    b1 = nb if it["last"] else first_ending_at_or_after(it["s0"] + S)
    return b0, b1


def check_stream(U, D, O, acclen, nchunks, total_blocks):
    R, S = segment_rows(U, D, O)
    assert S > 0
    blocks_done = 0
    for c in range(nchunks):
        final = c == nchunks - 1
        b_end = (c + 1) * acclen // O - NTAP + 1
        if final:  # blocks starting at or past the end of the data are all zeros: not produced
            b_end = min(total_blocks, -(-(c + 1) * acclen // O))
        b_end = max(min(b_end, total_blocks), blocks_done)
        nb = b_end - blocks_done
        assert nb <= acclen // O + NTAP + 1  # the stream's W buffer (nb_max in ab_stream_create)
        row0 = blocks_done * O - c * acclen  # local row of the first block
        assert c == 0 or row0 >= -4 * O
        owner = np.zeros(nb, np.int64)
        for it in items(acclen, S, O):
            assert it["nrows"] <= R
            yoff = it["ylo"] - it["s0"] + 4 * O  # y row of the item's first computed row
            held = [(yoff, yoff + it["nrows"])]
            if it["first"]:
                held.append((0, 4 * O))  # previous chunk's tail
            if it["last"]:
                held.append((yoff + it["nrows"], yoff + it["nrows"] + 4 * O))  # zeros past the end
            b0, b1 = fold_range(it, S, O, row0, nb)
            owner[b0:b1] += 1
            for b in range(b0, b1):
                rfirst = row0 + b * O
                if rfirst >= it["s1"]:
                    assert it["last"]  # wholly past the stream: written as zeros, reads nothing
                    continue
                q0 = 4 * O - it["s0"] + rfirst
                rows = np.arange(q0, q0 + 4 * O)
                ok = np.zeros(rows.size, bool)
                for lo, hi in held:
                    ok |= (rows >= lo) & (rows < hi)
                assert ok.all(), (c, b, q0, held)
                if not final:  # a block completed before the end reads only rows that exist
                    assert rfirst + 4 * O <= acclen
            if it["last"]:  # tail for the next chunk: kept rows [acclen - 4O, acclen)
                q = acclen - it["s0"] + np.arange(4 * O)
                ok = np.zeros(q.size, bool)
                for lo, hi in held[:2] if it["first"] else held[:1]:
                    ok |= (q >= lo) & (q < hi)
                assert ok.all()
        assert (owner == 1).all(), (c, np.nonzero(owner != 1)[0][:5])
        blocks_done = b_end


@pytest.mark.parametrize("U,D", TILES)
@pytest.mark.parametrize("O", [4, 8, 16, 32, 64])
def test_fold_bookkeeping_bench_geometry(U, D, O):
    """2^15-spectrum chunks, 512-block jobs, planned as the reference's planner
    does (the last job zero-padded)."""
    acclen, nchunks, nblock = 1 << 15, 5, 512
    nb_stream = nchunks * acclen // O - (NTAP - 1)
    total = -(-nb_stream // nblock) * nblock
    check_stream(U, D, O, acclen, nchunks, total)


@pytest.mark.parametrize("U,D", TILES)
def test_fold_bookkeeping_random_geometries(U, D):
    rng = np.random.default_rng(U * 10 + D)
    for _ in range(60):
        O = int(rng.choice([4, 8, 16, 32, 64]))
        acclen = int(rng.integers(NTAP * O, 40000))  # ab_stream_create needs acclen >= ntap * osamp
        nchunks = int(rng.integers(1, 5))
        nblock = int(rng.integers(1, 600))
        nb_stream = max(nchunks * acclen // O - (NTAP - 1), 1)
        total = -(-nb_stream // nblock) * nblock
        check_stream(U, D, O, acclen, nchunks, total)
