"""CPU model of the coarse correlator's time slicing (csrc/xcorr.cu,
coarse_xcorr_run and the kernels' k_begin / k_end), which carries the fp16
path's exactness: every CTA sums at most 4096 samples of one chunk, so a
Gram entry's fp32 partial sum of products of 4-bit levels (-7..8, |product|
<= 64) stays at most 2^18 < 2^24, where fp32 is still exact; slices of a
chunk cover it once, so the int64 totals are the exact sums of the reference's
avg_xcorr_4bit (albatros_analysis/src/correlations/correlations_cpu.c:128-186).
"""
import numpy as np
import pytest

KCC_KT = 64  # rows per shared-memory tile of the kernels (kCcKT)


def slices(nrows, chunk_rows):
    """(chunk, first row, end row) of every CTA time slice."""
    nchunks = -(-nrows // chunk_rows)
    slice_ = 4096 if chunk_rows >= 4096 else -(-chunk_rows // KCC_KT) * KCC_KT
    spc = -(-chunk_rows // slice_)
    out = []
    for y in range(nchunks * spc):
        chunk, sl = divmod(y, spc)
        k0 = chunk * chunk_rows + sl * slice_
        k1 = min(k0 + slice_, min((chunk + 1) * chunk_rows, nrows))
        out.append((chunk, k0, k1))
    return out


@pytest.mark.parametrize("nrows,chunk_rows", [(1 << 17, 1 << 14), (1 << 18, 1 << 18), (2048, 2048), (1000, 64),
                                              (70001, 5000), (4097, 4097), (10, 3)])
def test_slices_cover_each_chunk_once_within_the_fp32_bound(nrows, chunk_rows):
    seen = np.zeros(nrows, np.int64)
    for chunk, k0, k1 in slices(nrows, chunk_rows):
        if k1 <= k0:
            continue  # an empty tail slice does no work
        assert k1 - k0 <= 4096
        assert chunk * chunk_rows <= k0 and k1 <= min((chunk + 1) * chunk_rows, nrows)
        seen[k0:k1] += 1
    assert (seen == 1).all()
    assert 4096 * 8 * 8 < 1 << 24


def test_decoded_levels():
    """The 4-bit rule (unpacking.c:187-202): nibble v > 8 -> v - 16, else v."""
    v = np.arange(16)
    lev = ((v + 7) & 15) - 7
    np.testing.assert_array_equal(lev, np.where(v > 8, v - 16, v))
    assert lev.min() == -7 and lev.max() == 8
