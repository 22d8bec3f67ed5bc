"""The plain-GPU comparator arm of the benchmark (baseline/plain_gpu.py: the
reference's CuPy glue restated in torch around cuFFT and cuBLAS) computes the
chain's visibilities: it agrees with the FP64 streaming oracle to the float32
rounding of the reference's own code (1e-4 norm-wise, the reference's compare
scripts use rtol 1e-3), with several jobs per chunk, a job spanning chunks and
the reference's default cut (nslice without a smooth factorisation)."""
import numpy as np
import pytest
import torch

from oracle import pfb_oracle as po
from tests.golden import gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("acclen,cut,osamp,nblock,nchunks", [
    (1024, 64, 16, 16, 3),   # several jobs per chunk
    (1024, 10, 4, 300, 3),   # job spanning chunks, nslice 1044 = 4*9*29
    (2048, 10, 64, 24, 3),   # osamp 64 (4096 fine channels per coarse channel)
])
def test_plain_gpu_path_matches_oracle(acclen, cut, osamp, nblock, nchunks):
    from baseline import plain_gpu as pgp
    raw = gen.raw_4bit(seed=acclen + cut, nspec=nchunks * acclen, nchan=8, nant=2)
    ch = np.arange(600, 608)
    chain = pgp.PlainGpuChain(2, ch, acclen, nchunks, nblock, osamp, cut=cut)
    vis = np.asarray(chain.run(torch.from_numpy(raw).cuda()))
    ref, _ = po.repfb_xcorr_avg(raw, ch, acclen, nchunks, nblock, 0, 8, osamp, cut=cut)
    assert vis.shape == ref.shape
    assert np.linalg.norm(vis - ref) / np.linalg.norm(ref) < 1e-4
