"""The allocation-free coarse correlator (ab_xcorr_coarse_4bit_noalloc).

It serves callers that may not allocate device memory while running, by
keeping its partial sums in a fixed buffer built into the library.  Here it is
called through the C-ABI and must reproduce the regular entry point
(ab_xcorr_coarse_4bit) exactly, integer sums being bit-exact, on two calls in
a row with different data (the shared buffer must not leak the first call's
sums into the second).  This file is collected last so a failure here does not
hide the rest of the suite; it passes alone or after the other tests.
"""
import pytest
import torch

from tests.golden import gen

pytestmark = pytest.mark.gpu


def _call(lib, name, raw, nant, nspec, nchan, ch, chunk, with_ctx):
    from albatros_axion_detection_gb300 import _lib
    M = 2 * nant
    nchunks = -(-nspec // chunk)
    re = torch.full((nchunks, M, M, ch.numel()), -1, dtype=torch.int64, device="cuda")
    im = torch.full_like(re, -1)
    args = [raw.data_ptr(), nspec * 2 * nchan, nant, nspec, nchan, 0, nspec, None, ch.data_ptr(), ch.numel(), chunk,
            re.data_ptr(), im.data_ptr(), torch.cuda.current_stream().cuda_stream]
    if with_ctx:
        args = [_lib.ctx()] + args
    rc = getattr(lib, name)(*args)
    assert rc == 0, lib.ab_last_error()
    return re, im


def test_noalloc_matches_regular_entry_point_twice():
    from albatros_axion_detection_gb300 import _lib
    lib = _lib.load()
    nant, nspec, nchan, chunk = 4, 3000, 48, 1024
    ch = torch.tensor([0, 3, 7, 8, 20, 47], dtype=torch.int64, device="cuda")
    for seed in (101, 202):  # two calls in a row, different data
        raw = torch.from_numpy(gen.raw_4bit_uniform(seed=seed, nspec=nspec, nchan=nchan, nant=nant)).cuda()
        r0, i0 = _call(lib, "ab_xcorr_coarse_4bit_noalloc", raw, nant, nspec, nchan, ch, chunk, with_ctx=False)
        r1, i1 = _call(lib, "ab_xcorr_coarse_4bit", raw, nant, nspec, nchan, ch, chunk, with_ctx=True)
        torch.cuda.synchronize()
        assert torch.equal(r0, r1) and torch.equal(i0, i1)
        assert int(r0[0, 0, 0, 0]) > 0  # autocorrelation power is positive


def test_noalloc_rejects_scratch_beyond_its_buffer():
    from albatros_axion_detection_gb300 import _lib
    lib = _lib.load()
    # 32 antennas x 512 channels x 1 chunk needs 512 * 128^2 * 8 B = 64 MiB > 16 MiB
    rc = lib.ab_xcorr_coarse_4bit_noalloc(1, 1 << 30, 32, 100, 512, 0, 100, None, 1, 512, 100, 1, 1, None)
    assert rc == -1
    assert b"built-in buffer" in lib.ab_last_error()
