"""GPU parity of the streaming unpack -> IPFB -> PFB -> xcorr chain against
the FP64 streaming oracle (fine visibilities within 1e-5 relative, norm-wise
per job)."""
import numpy as np
import pytest
import torch

from oracle import pfb_oracle as po
from tests.golden import gen

pytestmark = pytest.mark.gpu
TOL = 1e-5


def run(raw, channels, **kw):
    from albatros_axion_detection_gb300 import stream
    spec_map = kw.pop("spec_map", None)
    kw.setdefault("bits", 4)
    vis, freqs = stream.repfb_xcorr_avg(torch.from_numpy(raw).cuda(), channels,
                                        spec_map=None if spec_map is None else torch.from_numpy(spec_map).cuda(), **kw)
    return np.asarray(vis), freqs


def check(vis, ref):
    """Norm-wise relative error over all jobs, and per job against the RMS job
    norm (a job inside a data gap carries ~1e-3 of the typical power, so its
    own norm is not a meaningful scale for FP32 rounding)."""
    assert vis.shape == ref.shape, (vis.shape, ref.shape)
    assert np.linalg.norm(vis - ref) / np.linalg.norm(ref) < TOL
    scale = np.sqrt(np.mean([np.linalg.norm(ref[..., k]) ** 2 for k in range(ref.shape[-1])]))
    for k in range(ref.shape[-1]):
        e = np.linalg.norm(vis[..., k] - ref[..., k]) / scale
        assert e < TOL, f"job {k}: error {e:.3e} of the RMS job norm"


@pytest.mark.parametrize("nant,nchan_raw,chs,acclen,cut,osamp,nblock,nchunks", [
    (2, 8, (0, 8), 512, 32, 4, 16, 4),       # several jobs per chunk
    (1, 16, (3, 11), 448, 32, 1, 300, 3),    # osamp 1, job spanning chunks
    (2, 64, (0, 64), 1024, 64, 64, 8, 3),    # osamp 64 (4096 fine ch), mixed-radix nslice
    (3, 4, (0, 4), 256, 16, 16, 5, 5),       # 3 antennas
])
def test_stream_vs_oracle(nant, nchan_raw, chs, acclen, cut, osamp, nblock, nchunks):
    raw = gen.raw_4bit(seed=acclen + nant, nspec=nchunks * acclen, nchan=nchan_raw, nant=nant)
    channels = np.arange(500, 500 + nchan_raw)
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=nblock, chanstart=chs[0], chanend=chs[1], osamp=osamp, cut=cut)
    vis, freqs = run(raw, channels, **kw)
    ref, (q0, q1) = po.repfb_xcorr_avg(raw, channels, **kw)
    assert freqs[0] == q0 and len(freqs) == q1 - q0
    check(vis, ref)


def test_stream_missing_spectra():
    nant, nchan, acclen, nchunks = 2, 8, 512, 3
    raw = gen.raw_4bit(seed=77, nspec=nchunks * acclen, nchan=nchan, nant=nant)
    rng = np.random.default_rng(1)
    present = rng.random((nant, nchunks * acclen)) > 0.1
    present[:, 600:700] = False  # a long gap
    spec_map = np.where(present, np.arange(nchunks * acclen)[None, :], -1).astype(np.int32)
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=16, chanstart=0, chanend=nchan, osamp=4, cut=32)
    vis, _ = run(raw, np.arange(200, 208), spec_map=spec_map, **kw)
    ref, _ = po.repfb_xcorr_avg(raw, np.arange(200, 208), spec_present=present, **kw)
    check(vis, ref)
    # the reference's return with the missing-data percentage per antenna and job
    from albatros_axion_detection_gb300 import output, stream
    v2, mf, freqs = stream.repfb_xcorr_avg(torch.from_numpy(raw).cuda(), np.arange(200, 208),
                                           spec_map=torch.from_numpy(spec_map).cuda(), with_missing=True, **kw)
    assert np.array_equal(np.asarray(v2), vis) and len(freqs) == vis.shape[2]
    counts = present.reshape(nant, nchunks, acclen).sum(-1)
    assert mf.shape == (nant, vis.shape[-1]) and mf.max() > 0
    np.testing.assert_array_equal(mf, output.missing_fraction(counts, acclen, 16, 4))


def test_stream_channel_subset_and_gap_in_channel_numbers():
    raw = gen.raw_4bit(seed=8, nspec=2 * 512, nchan=10, nant=1)
    channels = np.array([90, 91, 92, 93, 94, 120, 121, 122, 123, 124])
    kw = dict(acclen=512, nchunks=2, nblock=20, chanstart=5, chanend=9, osamp=4, cut=32)
    vis, _ = run(raw, channels, **kw)
    ref, _ = po.repfb_xcorr_avg(raw, channels, **kw)
    check(vis, ref)


@pytest.mark.parametrize("chs,osamp", [((0, 32), 16), ((6, 13), 64)])
def test_stream_1bit_vs_oracle(chs, osamp):
    """1-bit sign packets through the chain (the 1-bit files of a mixed batch)."""
    nant, nchan_raw, acclen, cut, nchunks = 2, 32, 512, 32, 3
    raw = gen.raw_1bit(seed=osamp, nspec=nant * nchunks * acclen, nchan=nchan_raw).reshape(nant, nchunks * acclen, -1)
    channels = np.arange(300, 300 + nchan_raw)
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=6, chanstart=chs[0], chanend=chs[1], osamp=osamp, cut=cut)
    vis, freqs = run(raw, channels, bits=1, **kw)
    ref, (q0, q1) = po.repfb_xcorr_avg(raw, channels, bits=1, **kw)
    assert freqs[0] == q0 and len(freqs) == q1 - q0
    check(vis, ref)


def test_stream_rejects_bad_config():
    from albatros_axion_detection_gb300 import autotune, stream
    from albatros_axion_detection_gb300._lib import AlbatrosError
    # nslice/2 = 261 = 9*29: only the FIR time stage can run it
    sc = stream.StreamCorrelator(1, np.arange(8), 0, 8, acclen=500, nchunks=2, nblock=4, osamp=4, cut=11)
    assert sc.time_filter() == ("iir", 40)
    sc.close()
    autotune.set_time_filter(1)
    try:
        with pytest.raises((AlbatrosError, ValueError)):
            stream.StreamCorrelator(1, np.arange(8), 0, 8, acclen=500, nchunks=2, nblock=4, osamp=4, cut=11)
    finally:
        autotune.set_time_filter(autotune.DEFAULT_MODE)
    for bad in (dict(osamp=3), dict(cut=0), dict(acclen=20, cut=11), dict(osamp=128)):
        kw = dict(acclen=500, nchunks=2, nblock=4, osamp=4, cut=11)
        kw.update(bad)
        with pytest.raises((AlbatrosError, ValueError)):
            stream.StreamCorrelator(1, np.arange(8), 0, 8, **kw)


@pytest.mark.parametrize("per_cta", [2, 4, 8])
@pytest.mark.parametrize("nrows_extra", [0, 1, 3])
def test_stream_row_stage_shapes(per_cta, nrows_extra):
    """Each row-stage shape (2 or 4 pol-paired spectra, 8 time-paired spectra
    per CTA; with the scalar tail when nslice is not a multiple of the
    spectra per CTA) gives the oracle's visibilities, with and without
    missing spectra."""
    from albatros_axion_detection_gb300 import autotune
    acclen, cut = 512 + nrows_extra, 32
    raw = gen.raw_4bit(seed=77 + nrows_extra, nspec=3 * acclen, nchan=8, nant=2)
    channels = np.arange(520, 528)
    kw = dict(acclen=acclen, nchunks=3, nblock=32, chanstart=0, chanend=8, osamp=16, cut=cut)
    present = np.ones((2, 3 * acclen), bool)
    present[0, 100:131] = False
    present[1, 700:705] = False
    spec_map = np.where(present, np.arange(3 * acclen)[None, :], -1).astype(np.int32)
    ref, _ = po.repfb_xcorr_avg(raw, channels, spec_present=present, **kw)
    autotune.set_row_ffts_per_cta(per_cta)
    autotune.set_row_tc(0)  # the FFT row stage's shapes
    try:
        vis, _ = run(raw, channels, spec_map=spec_map, **kw)
    finally:
        autotune.set_row_ffts_per_cta(8)
        autotune.set_row_tc(1)
    check(vis, ref)


@pytest.mark.parametrize("bits,nrows_extra", [(4, 0), (4, 3), (1, 5)])
def test_row_prefetch_equals_one_cta_per_tile(bits, nrows_extra):
    """The persistent row stage (cp.async prefetch of map rows and packet
    words; FFT twiddles read from global or shared memory) and the
    one-CTA-per-tile form compute the same transforms: identical
    visibilities, with missing spectra and a ragged last tile."""
    from albatros_axion_detection_gb300 import autotune
    acclen, cut, nchan = 512 + nrows_extra, 32, 16
    raw = (gen.raw_4bit(seed=5 + nrows_extra, nspec=3 * acclen, nchan=nchan, nant=2) if bits == 4 else
           np.stack([gen.raw_1bit(seed=6 + a, nspec=3 * acclen, nchan=nchan) for a in range(2)]))
    channels = np.arange(700, 700 + nchan)
    kw = dict(acclen=acclen, nchunks=3, nblock=32, chanstart=2, chanend=14, osamp=16, cut=cut, bits=bits)
    present = np.ones((2, 3 * acclen), bool)
    present[0, 90:133] = False
    present[1, 600:611] = False
    spec_map = np.where(present, np.arange(3 * acclen)[None, :], -1).astype(np.int32)
    autotune.set_row_tc(0)  # the FFT row stage's forms
    try:
        a, _ = run(raw, channels, spec_map=spec_map, **kw)  # default: twiddles in shared memory
        autotune.set_row_prefetch(0)
        b, _ = run(raw, channels, spec_map=spec_map, **kw)
        autotune.set_row_prefetch(1)  # twiddles from global memory
        c, _ = run(raw, channels, spec_map=spec_map, **kw)
    finally:
        autotune.set_row_prefetch(autotune.DEFAULT_ROW_PREFETCH)
        autotune.set_row_tc(1)
    assert np.array_equal(a, b) and np.array_equal(a, c)
    ref, _ = po.repfb_xcorr_avg(raw, channels, spec_present=present, **kw)
    check(a, ref)


@pytest.mark.parametrize("channels,chs,nrows_extra", [
    (np.arange(0, 8), (0, 8), 0),                    # the DC bin (weight 1/P, no sine term)
    (np.arange(2040, 2048), (0, 8), 3),              # the top channels a band may hold, ragged last spectrum tile
    (np.arange(900, 905), (0, 5), 1),                # 5 channels: a partial channel quad
    (np.arange(1000, 1033), (0, 33), 0),             # 33 channels: two K-blocks, the second partial
    (np.arange(300, 364), (10, 50), 2),              # a 40-channel band of 64 raw channels
])
def test_row_stage_tensor_cores_vs_fft_and_oracle(channels, chs, nrows_extra):
    """The row stage as a tensor-core product (the default for 4-bit and
    1-bit packets with at most 64 channels) against the FFT row stage and the
    FP64 oracle, with missing spectra: the DC and Nyquist bins, partial
    channel quads and K-blocks, spectrum tiles cut by the window's end."""
    acclen = 512 + nrows_extra
    raw = gen.raw_4bit(seed=int(channels[0]) + nrows_extra, nspec=3 * acclen, nchan=len(channels), nant=2)
    _row_tc_vs_fft_and_oracle(raw, channels, chs, acclen, bits=4)


@pytest.mark.parametrize("nchan,chs,nrows_extra", [
    (32, (0, 32), 1),   # 32 channels: one K-block
    (64, (3, 61), 0),   # 58 of 64 channels from an odd column: two K-blocks, a partial quad
    (10, (1, 9), 2),    # 8 channels, every other one in a low nibble
])
def test_row_stage_tensor_cores_1bit_vs_fft_and_oracle(nchan, chs, nrows_extra):
    """1-bit sign packets (r0 i0 r1 i1 per channel, two channels a byte)
    through the tensor-core row stage: as the FFT row stage and the oracle."""
    acclen = 512 + nrows_extra
    raw = np.stack([gen.raw_1bit(seed=40 + nchan + a, nspec=3 * acclen, nchan=nchan) for a in range(2)])
    _row_tc_vs_fft_and_oracle(raw, np.arange(1200, 1200 + nchan), chs, acclen, bits=1)


def _row_tc_vs_fft_and_oracle(raw, channels, chs, acclen, bits):
    from albatros_axion_detection_gb300 import autotune
    kw = dict(acclen=acclen, nchunks=3, nblock=24, chanstart=chs[0], chanend=chs[1], osamp=16, cut=32, bits=bits)
    present = np.ones((2, 3 * acclen), bool)
    present[0, 200:260] = False
    present[1, 1000:1003] = False
    spec_map = np.where(present, np.arange(3 * acclen)[None, :], -1).astype(np.int32)
    a, _ = run(raw, channels, spec_map=spec_map, **kw)
    autotune.set_row_tc(0)
    try:
        b, _ = run(raw, channels, spec_map=spec_map, **kw)
    finally:
        autotune.set_row_tc(1)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-6
    ref, _ = po.repfb_xcorr_avg(raw, channels, spec_present=present, **kw)
    check(a, ref)


def test_row_stage_tensor_cores_wait_timeout_reports_fault():
    """Failure path of the tensor-core row stage's bounded waits, without a
    GPU fault: its workers withhold their first item's decoded tiles (nothing
    else signals them), the MMA thread's wait runs out after about 2 s and
    with it the other roles', the stream's fault word turns the visibilities
    NaN, and the tensor memory was freed: after a reset the same stream gives
    the visibilities of a fresh one."""
    import time
    from albatros_axion_detection_gb300 import _lib, autotune, stream
    acclen, nchunks, nchan = 512, 3, 8
    raw = torch.from_numpy(gen.raw_4bit(seed=57, nspec=nchunks * acclen, nchan=nchan, nant=2)).cuda()
    mk = lambda: stream.StreamCorrelator(2, np.arange(40, 48), 0, nchan, acclen, nchunks, 16, 16, 32, nchan_raw=nchan)
    a, b = mk(), mk()
    try:
        for j in range(nchunks):
            a.push(raw, j, final=(j == nchunks - 1))
        good = a.vis_device().clone()
        _lib.call("ab_ctx_set_option", _lib.ctx(), autotune.OPT_FAULT_TEST, 2)
        t0 = time.time()
        for j in range(nchunks):
            b.push(raw, j, final=(j == nchunks - 1))
        torch.cuda.synchronize()
        assert time.time() - t0 < 30
        assert torch.isnan(b.vis_device()).all()
        b.reset()
        for j in range(nchunks):
            b.push(raw, j, final=(j == nchunks - 1))
        torch.cuda.synchronize()
        assert torch.isfinite(good).all() and torch.equal(b.vis_device(), good)
    finally:
        _lib.call("ab_ctx_set_option", _lib.ctx(), autotune.OPT_FAULT_TEST, 0)
        a.close()
        b.close()


def test_run_from_host_overlapped_copies_equal_device_run():
    """Per-chunk host->device copies on a side stream, each push waiting on
    its own chunk's copy, give the visibilities of a run on device packets."""
    from albatros_axion_detection_gb300 import stream
    acclen, nchunks, nchan = 512, 3, 8
    raw_np = gen.raw_4bit(seed=31, nspec=nchunks * acclen, nchan=nchan, nant=2)
    mk = lambda: stream.StreamCorrelator(2, np.arange(40, 48), 0, nchan, acclen, nchunks, 16, 16, 32, nchan_raw=nchan)
    a, b = mk(), mk()
    try:
        dev = torch.from_numpy(raw_np).cuda()
        for j in range(nchunks):
            a.push(dev, j, final=(j == nchunks - 1))
        host = torch.from_numpy(raw_np).pin_memory()
        target = torch.zeros_like(dev)
        for _ in range(2):  # a second pass reuses the buffer after the first finished
            b.reset()
            b.run_from_host(host, target)
        torch.cuda.synchronize()
        assert torch.equal(a.vis_device(), b.vis_device())
        with pytest.raises(ValueError):
            b.run_from_host(torch.from_numpy(raw_np), target)  # not pinned
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("nant,osamp,acclen,nblock,nchunks", [
    (2, 64, 2048, 24, 3),   # 16 slot pairs, several jobs
    (1, 16, 1024, 40, 3),
    (2, 8, 1024, 100, 4),   # a job spanning chunks
    (1, 4, 512, 16, 4),     # one slot pair (the W_{O/2} transform in every tile)
])
def test_pfb_band_tma_bitwise_equal(nant, osamp, acclen, nblock, nchunks):
    """The band DFT with W tiles staged by TMA (1: one CTA per tile landing
    the tile in its FFT buffers; 2: persistent CTAs fetching the next tile
    while the current one is transformed) gives bitwise the same
    visibilities as one CTA per tile with plain loads (0), and all match the
    FP64 oracle."""
    from albatros_axion_detection_gb300 import autotune
    raw = gen.raw_4bit(seed=osamp * nant + acclen, nspec=nchunks * acclen, nchan=8, nant=nant)
    channels = np.arange(300, 308)
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=nblock, chanstart=0, chanend=8, osamp=osamp, cut=32)
    out = {}
    for tma in (1, 2, 0):
        autotune.set_pfb_tma(tma)
        try:
            out[tma], _ = run(raw, channels, **kw)
        finally:
            autotune.set_pfb_tma(0)
    assert np.array_equal(np.asarray(out[1]), np.asarray(out[0]))
    assert np.array_equal(np.asarray(out[2]), np.asarray(out[0]))
    ref, _ = po.repfb_xcorr_avg(raw, channels, **kw)
    check(np.asarray(out[1]), ref)
