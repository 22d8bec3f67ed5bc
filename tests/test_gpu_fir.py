"""GPU tests of the IIR and FIR forms of the IPFB time stage (csrc/fir.cu):
the IIR form is chosen for the default Wiener threshold, the FIR form when
asked for; both agree with the FFT form and the FP64 oracle, reproduce the
reference's circular wrap when cut is below the filter's reach (including the
reference's default cut = 10, whose nslice has no fast FFT), and give way to
the FFT form for thresholds whose filter decays too slowly."""
import numpy as np
import pytest
import torch

from oracle import pfb_oracle as po
from tests.golden import gen
from tests.test_gpu_stream import check

pytestmark = pytest.mark.gpu


FIR, IIR, FFT = 3, 0, 1  # time-filter modes


def stream_vis(raw_np, channels, mode=FIR, row_tile=32, thresh=0.45, bits=4, **kw):
    from albatros_axion_detection_gb300 import autotune, stream
    autotune.set_time_filter(mode, row_tile)
    try:
        sc = stream.StreamCorrelator(raw_np.shape[0], channels, kw["chanstart"], kw["chanend"], kw["acclen"],
                                     kw["nchunks"], kw["nblock"], kw["osamp"], kw["cut"], thresh, 4,
                                     nchan_raw=len(channels), bits=bits)
    finally:
        autotune.set_time_filter(autotune.DEFAULT_MODE, autotune.DEFAULT_ROW_TILE)
    try:
        raw = torch.from_numpy(raw_np).cuda()
        for j in range(kw["nchunks"]):
            sc.push(raw, j, final=(j == kw["nchunks"] - 1))
        return sc.vis_device().permute(1, 2, 3, 0).cpu().numpy(), sc.time_filter()
    finally:
        sc.close()


CFG = dict(acclen=1024, nchunks=3, nblock=64, chanstart=0, chanend=8, osamp=16, cut=64)


def test_fir_chosen_and_matches_fft_and_oracle():
    raw = gen.raw_4bit(seed=21, nspec=3 * 1024, nchan=8, nant=2)
    ch = np.arange(600, 608)
    ref, _ = po.repfb_xcorr_avg(raw, ch, **CFG)
    v_fir, tf = stream_vis(raw, ch, mode=FIR, **CFG)
    v_iir, ti = stream_vis(raw, ch, mode=IIR, **CFG)
    v_fft, t0 = stream_vis(raw, ch, mode=FFT, **CFG)
    assert tf == ("fir", 32) and ti == ("iir", 40) and t0 == ("fft", 0)
    for v in (v_fir, v_iir, v_fft):
        check(v, ref)
    assert np.linalg.norm(v_fir - v_fft) / np.linalg.norm(v_fft) < 2e-6
    assert np.linalg.norm(v_iir - v_fft) / np.linalg.norm(v_fft) < 2e-6


@pytest.mark.parametrize("mode", [FIR, IIR])
def test_row_tiles_agree(mode):
    """Row tiles 33 and 17 (FIR; tile class 64 runs 33 as well): the FIR sums
    are identical term by term (bitwise); the IIR threads' ranges (67, 41 or
    21 rows) differ, so equal to rounding."""
    raw = gen.raw_4bit(seed=22, nspec=3 * 1024, nchan=8, nant=1)
    ch = np.arange(100, 108)
    cfg = dict(CFG, osamp=64, nblock=16)
    a, _ = stream_vis(raw, ch, mode=mode, row_tile=32, **cfg)
    b, _ = stream_vis(raw, ch, mode=mode, row_tile=16, **cfg)
    c, _ = stream_vis(raw, ch, mode=mode, row_tile=64, **cfg)
    if mode == FIR:
        assert np.array_equal(a, b) and np.array_equal(a, c)
    else:
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-6
        assert np.linalg.norm(a - c) / np.linalg.norm(a) < 1e-6


@pytest.mark.parametrize("mode", [FIR, IIR])
@pytest.mark.parametrize("acclen,cut,osamp,nchunks,bits", [
    (1024, 10, 16, 3, 4),   # the reference's default cut: nslice 1044 = 4*9*29, no FFT form; wrap inside kept rows
    (512, 8, 4, 4, 4),      # cut below the filter's reach with 4*osamp = 16
    (1024, 10, 64, 3, 1),   # 1-bit packets, osamp 64
])
def test_circular_wrap_small_cut(acclen, cut, osamp, nchunks, bits, mode):
    nch = 8
    if bits == 4:
        raw = gen.raw_4bit(seed=acclen + cut, nspec=nchunks * acclen, nchan=nch, nant=2)
    else:
        rng = np.random.default_rng(acclen + cut)
        raw = rng.integers(0, 256, (2, nchunks * acclen, nch // 2), dtype=np.uint8)
    ch = np.arange(700, 700 + nch)
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=max(acclen // osamp, 1), chanstart=0, chanend=nch,
              osamp=osamp, cut=cut)
    ref, _ = po.repfb_xcorr_avg(raw, ch, bits=bits, **kw)
    v, tf = stream_vis(raw, ch, mode=mode, bits=bits, **kw)
    assert tf == (("fir", 32) if mode == FIR else ("iir", 40))
    check(v, ref)


@pytest.mark.parametrize("mode,expect", [(FIR, ("fir", 64)), (IIR, ("iir", 80))])
def test_threshold_02_uses_longer_filters(mode, expect):
    raw = gen.raw_4bit(seed=24, nspec=3 * 1024, nchan=8, nant=1)
    ch = np.arange(310, 318)
    ref, _ = po.repfb_xcorr_avg(raw, ch, filt_thresh=0.2, **CFG)
    v, tf = stream_vis(raw, ch, mode=mode, thresh=0.2, **CFG)
    assert tf == expect  # 0.2: 64 taps a side, or an 80-sample warm-up
    check(v, ref)


def test_small_threshold_uses_fft_stage():
    raw = gen.raw_4bit(seed=23, nspec=3 * 1024, nchan=8, nant=1)
    ch = np.arange(300, 308)
    ref, _ = po.repfb_xcorr_avg(raw, ch, filt_thresh=0.1, **CFG)
    for mode in (FIR, IIR):
        v, tf = stream_vis(raw, ch, mode=mode, thresh=0.1, **CFG)
        assert tf == ("fft", 0)  # the thresh 0.1 filter decays too slowly for either
        check(v, ref)


def test_time_stage_tuner(tmp_path, monkeypatch):
    from albatros_axion_detection_gb300 import autotune
    monkeypatch.setenv("ALBATROS_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    try:
        best = autotune.tune_time_stage(1024, 64, 16, limit=2)
        assert best["mode"] in (0, 1, 3) and best["ms"] > 0
        assert len(best["candidates"]) >= 2
        again = autotune.tune_time_stage(1024, 64, 16, limit=2)
        assert again["ms"] == best["ms"]
    finally:
        autotune.set_time_filter(autotune.DEFAULT_MODE, 32)
        autotune.set_plan(576, None)


@pytest.mark.parametrize("mode", [FIR, IIR])
@pytest.mark.parametrize("osamp,row_tile", [(64, 16), (64, 32), (4, 16), (64, 64)])
def test_multi_segment_columns(osamp, row_tile, mode):
    """acclen 8192 spans 2-3 segments per column (a segment holds
    row_tile*256 - 4*osamp new rows): blocks across segment edges and the
    tail state handed between chunks must match the oracle."""
    acclen, nchunks = 8192, 2
    raw = gen.raw_4bit(seed=osamp + row_tile, nspec=nchunks * acclen, nchan=4, nant=1)
    ch = np.arange(900, 904)
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=acclen // osamp // 2, chanstart=0, chanend=4, osamp=osamp,
              cut=64)
    ref, _ = po.repfb_xcorr_avg(raw, ch, **kw)
    v, tf = stream_vis(raw, ch, mode=mode, row_tile=row_tile, **kw)
    assert tf[0] == ("fir" if mode == FIR else "iir")
    check(v, ref)


@pytest.mark.parametrize("osamp,cut,thresh", [(64, 10, 0.45), (4, 64, 0.45), (64, 80, 0.2)])
def test_iir_large_tile_segments(osamp, cut, thresh):
    """The 67-row IIR tile (one CTA per SM) holds 16384 new rows per segment:
    acclen 2^15 spans two segments per column, so blocks across the segment
    edge, the tail state between chunks and (threshold 0.2, 80-row carry)
    the two-neighbour state exchange are all exercised against the oracle."""
    acclen, nchunks = 32768, 2
    raw = gen.raw_4bit(seed=osamp + cut, nspec=nchunks * acclen, nchan=2, nant=1)
    ch = np.arange(1000, 1002)
    kw = dict(acclen=acclen, nchunks=nchunks, nblock=acclen // osamp // 4, chanstart=0, chanend=2, osamp=osamp,
              cut=cut)
    ref, _ = po.repfb_xcorr_avg(raw, ch, filt_thresh=thresh, **kw)
    v, tf = stream_vis(raw, ch, mode=IIR, row_tile=64, thresh=thresh, **kw)
    assert tf == ("iir", 40 if thresh == 0.45 else 80)
    check(v, ref)

