"""GPU parity at the full-chain streaming benchmark's own geometry: 2 antennas
x 2 pols of 4-bit packets, 64 coarse channels, chunks of 2^15 spectra, PFB
osamp 64 (4096 fine channels), 512 fine blocks per job, at the reference's
default cut (10, nslice 32788) and at cut 80 (nslice 32928), against the FP64
streaming oracle.

At this size the persistent row stage walks many tiles per CTA, every IPFB
column of the IIR time stage is cut into several segments with tails handed
between chunks, and fine blocks straddle chunks.  A third geometry (300 fine
blocks per job) puts job boundaries inside chunks.  Besides the visibilities,
each output of the chain is checked on its own against the FP64 oracle: the
IPFB timestream (``cupy_ipfb`` on the first chunk's rows, nslice 32928) and
the PFB band spectra (``cupy_pfb_band`` on one job's worth of timestream).

Bars: fine visibilities 1e-5 norm-wise relative error per job (the target of
the chain), one FFT chain (IPFB timestream, PFB band) 2e-6.  Set
AB_PARITY_REPORT to a file path to get the measured errors as JSON lines.
"""
import json
import os

import numpy as np
import pytest
import torch

from oracle import pfb_oracle as po
from tests.golden import gen
from tests.test_gpu_stream import check

pytestmark = pytest.mark.gpu

NANT, NCH, ACCLEN, OSAMP, NCHUNKS = 2, 64, 2 ** 15, 64, 3
CHANNELS = np.arange(640, 640 + NCH)
_cache = {}


def report(**kv):
    path = os.environ.get("AB_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(kv) + "\n")


@pytest.fixture(scope="module")
def raw():
    return gen.raw_4bit(seed=2026, nspec=NCHUNKS * ACCLEN, nchan=NCH, nant=NANT)


def oracle_vis(raw, cut, nblock):
    key = (cut, nblock)
    if key not in _cache:
        _cache[key] = po.repfb_xcorr_avg(raw, CHANNELS, ACCLEN, NCHUNKS, nblock, 0, NCH, OSAMP, cut=cut)
    return _cache[key]


def gpu_vis(raw, cut, nblock, mode=None):
    from albatros_axion_detection_gb300 import autotune, stream
    if mode is not None:
        autotune.set_time_filter(mode, autotune.DEFAULT_ROW_TILE)
    try:
        sc = stream.StreamCorrelator(NANT, CHANNELS, 0, NCH, ACCLEN, NCHUNKS, nblock, OSAMP, cut, nchan_raw=NCH)
    finally:
        autotune.set_time_filter(autotune.DEFAULT_MODE, autotune.DEFAULT_ROW_TILE)
    try:
        r = torch.from_numpy(raw).cuda()
        for j in range(NCHUNKS):
            sc.push(r, j, final=(j == NCHUNKS - 1))
        return sc.vis_device().permute(1, 2, 3, 0).cpu().numpy(), sc.time_filter()
    finally:
        sc.close()


def job_errors(vis, ref):
    return [float(np.linalg.norm(vis[..., k] - ref[..., k]) / np.linalg.norm(ref[..., k]))
            for k in range(ref.shape[-1])]


@pytest.mark.parametrize("cut,nblock", [(10, 512), (80, 512), (10, 300)])
def test_headline_stream_vs_oracle(raw, cut, nblock):
    ref, (q0, q1) = oracle_vis(raw, cut, nblock)
    vis, tf = gpu_vis(raw, cut, nblock)
    assert tf[0] == "iir"
    assert vis.shape == ref.shape == (4, 4, 4096, len(po.plan_chunks(NCHUNKS, ACCLEN * 4096, nblock, 4096 * OSAMP, 4)))
    check(vis, ref)
    errs = job_errors(vis, ref)
    report(test="stream_vis", cut=cut, nblock=nblock, time_stage=list(tf), per_job=errs, max=max(errs))
    assert max(errs) < 1e-5


@pytest.mark.parametrize("mode,cut", [(3, 10), (1, 80)])  # FIR form at the reference's cut; FFT form at cut 80
def test_headline_other_time_stages(raw, mode, cut):
    ref, _ = oracle_vis(raw, cut, 512)
    vis, tf = gpu_vis(raw, cut, 512, mode=mode)
    assert tf[0] == {3: "fir", 1: "fft"}[mode]
    check(vis, ref)
    errs = job_errors(vis, ref)
    report(test="stream_vis", cut=cut, nblock=512, time_stage=list(tf), per_job=errs, max=max(errs))
    assert max(errs) < 1e-5


@pytest.mark.parametrize("cut", [10, 80])
def test_headline_ipfb_timestream(raw, cut):
    """cupy_ipfb on the first chunk's rows (2*cut zero rows, then 2^15 placed
    rows) at nslice 32788 (the reference's default cut) and 32928, against the
    FP64 IPFB with the FP64 filter."""
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pg
    nslice = ACCLEN + 2 * cut
    sel = np.arange(NCH)
    spec = po.unpack_4bit_np(raw[0], 0, ACCLEN, sel)[0]
    dat = np.zeros((nslice, 2049), np.complex128)
    dat[2 * cut:] = po.make_continuous(spec, np.arange(ACCLEN), 0, CHANNELS, ACCLEN)
    filt64 = po.calculate_filter(po.get_matft(nslice), 0.45)
    exp = po.ipfb(dat, filt64)
    got = pg.cupy_ipfb(torch.from_numpy(dat.astype(np.complex64)).cuda(), pg.build_filter(nslice, 0.45))
    got = got.cpu().numpy()
    err = float(np.linalg.norm(got - exp) / np.linalg.norm(exp))
    kept = float(np.linalg.norm(got[cut:-cut] - exp[cut:-cut]) / np.linalg.norm(exp[cut:-cut]))
    report(test="ipfb_timestream", nslice=nslice, rel_err=err, rel_err_kept_rows=kept)
    assert err < 2e-6 and kept < 2e-6


def test_headline_pfb_band(raw):
    """cupy_pfb_band over one job's worth of float32 timestream (515 fine
    blocks of 262144 samples) against the FP64 PFB of the same samples."""
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pg
    cut, nblock = 10, 512
    lblock = 4096 * OSAMP
    nslice = ACCLEN + 2 * cut
    filt = po.calculate_filter(po.get_matft(nslice), 0.45)
    ts = po.stream_timestream(raw, 0, 0, np.arange(NCH), CHANNELS, ACCLEN, 2, cut, filt)
    ts32 = ts[: (nblock + 3) * lblock].astype(np.float32)
    win = po.sinc_hamming(4, lblock)
    q0, q1 = po.band_edges(CHANNELS, 0, NCH, OSAMP)
    exp = po.pfb(ts32.astype(np.float64), win, nchan=lblock // 2 + 1)[:, q0:q1]
    got = pg.cupy_pfb_band(torch.from_numpy(ts32).cuda(), win.astype(np.float32), q0, q1, nchan=lblock // 2 + 1)
    got = got.cpu().numpy()
    err = float(np.linalg.norm(got - exp) / np.linalg.norm(exp))
    report(test="pfb_band", nblock=nblock, osamp=OSAMP, rel_err=err)
    assert err < 2e-6
