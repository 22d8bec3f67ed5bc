"""GPU parity: correlators.  Integer paths bit-exact against the C oracle /
the reference's golden sums; float paths within 1e-5 relative of FP64."""
import os

import numpy as np
import pytest
import torch

from oracle import int_oracle as io
from oracle import pfb_oracle as po
from tests.golden import gen

pytestmark = pytest.mark.gpu


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def f_order(x):
    """numpy (M, T, F) -> torch CUDA tensor with F-ordered strides."""
    return cu(np.asfortranarray(x).T.copy()).permute(2, 1, 0)


def test_all_ant_known_answers():
    """Constant inputs 3,5,7 / 4,6,8 give exact products
    (src/correlations/tests/test_gpu_all_ant_complex_xcorr.py:35-68)."""
    from albatros_axion_detection_gb300.correlations import avg_xcorr_all_ant_gpu
    x = np.zeros((3, 10000, 2), np.complex64)
    x[:, :, 0] = np.array([3, 5, 7])[:, None]
    x[:, :, 1] = np.array([4, 6, 8])[:, None]
    out = avg_xcorr_all_ant_gpu(f_order(x), 3, 1, 10000, 2)
    o = out.cpu().numpy()
    assert o[0, 0, 0] == 9 and o[0, 1, 0] == 15 and o[0, 2, 0] == 21 and o[1, 2, 0] == 35
    assert o[0, 0, 1] == 16 and o[0, 1, 1] == 24 and o[0, 2, 1] == 32 and o[1, 2, 1] == 48
    assert np.all(o.imag == 0)
    assert out.permute(2, 1, 0).is_contiguous()


@pytest.mark.parametrize("M,T,F", [(2, 10000, 2), (4, 512, 4096), (32, 300, 7), (5, 1, 3)])
def test_all_ant_random(M, T, F):
    from albatros_axion_detection_gb300.correlations import avg_xcorr_all_ant_gpu
    rng = np.random.default_rng(M * T)
    x = (rng.standard_normal((M, T, F)) + 10j * rng.standard_normal((M, T, F))).astype(np.complex64)
    got = avg_xcorr_all_ant_gpu(f_order(x), M, 1, T, F).cpu().numpy()
    exp = po.xcorr_all_ant(x, M, 1, T, F)
    assert np.linalg.norm(got - exp) / np.linalg.norm(exp) < 1e-5


def test_all_ant_errors():
    from albatros_axion_detection_gb300.correlations import avg_xcorr_all_ant_gpu
    x = f_order(np.zeros((2, 10, 3), np.complex64))
    with pytest.raises(ValueError):
        avg_xcorr_all_ant_gpu(x, 2, 1, 10, 3, split=3)
    with pytest.raises(NotImplementedError):
        avg_xcorr_all_ant_gpu(x, 2, 1, 10, 3, split=2)
    with pytest.raises(ValueError):
        avg_xcorr_all_ant_gpu(x, 2, 1, 10, 3, out=torch.zeros((2, 2, 3), dtype=torch.complex64, device="cuda"))


@pytest.fixture(params=[16, 8], ids=["fp16-mma", "int8-mma"])
def mma_bits(request):
    """Run a coarse-correlator test with each tensor-core operand type."""
    from albatros_axion_detection_gb300 import autotune
    autotune.set_coarse_mma_bits(request.param)
    yield request.param
    autotune.set_coarse_mma_bits(16)


@pytest.mark.parametrize("nant,nspec,nchan,chunk", [(2, 2 ** 14, 64, 2 ** 12), (16, 2048, 256, None),
                                                     (1, 333, 5, 100), (3, 1000, 16, 64)])
def test_coarse_xcorr_bit_exact(nant, nspec, nchan, chunk, mma_bits):
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    raw = gen.raw_4bit_uniform(seed=nant * nchan, nspec=nspec, nchan=nchan, nant=nant)
    ch = np.arange(nchan) if nchan < 64 else np.arange(0, nchan, 3)
    re, im = xcorr_coarse_4bit(cu(raw), 0, nspec, ch, nchan, chunk=chunk, average=False)
    re, im = re.cpu().numpy(), im.cpu().numpy()
    c = nspec if chunk is None else chunk
    for k in range(re.shape[0]):
        r0, r1 = k * c, min((k + 1) * c, nspec)
        er, ei = io.xcorr_all_ant_4bit(raw, r0, r1, ch, nchan, nthreads=8)
        np.testing.assert_array_equal(re[k], er)
        np.testing.assert_array_equal(im[k], ei)


_full = {}


def test_coarse_xcorr_many_antenna_full_size(mma_bits):
    """The many-antenna coarse correlator workload at its full size: 16
    antennas x 2 pols (all 528 input pairs), 256 channels, 2^18 spectra (2 GiB
    of packets, every nibble value including 0x8), one average over all
    spectra, bit-exact against the int64 oracle."""
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    nant, nchan, nspec = 16, 256, 1 << 18
    if "raw" not in _full:
        _full["raw"] = gen.raw_4bit_uniform(seed=418, nspec=nspec, nchan=nchan, nant=nant)
        _full["ref"] = io.xcorr_all_ant_4bit(_full["raw"], 0, nspec, np.arange(nchan), nchan,
                                             nthreads=os.cpu_count() or 1)
    raw = _full["raw"]
    er, ei = _full["ref"]
    re, im = xcorr_coarse_4bit(cu(raw), 0, nspec, np.arange(nchan), nchan, average=False)
    np.testing.assert_array_equal(re.cpu().numpy()[0], er)
    np.testing.assert_array_equal(im.cpu().numpy()[0], ei)


def test_coarse_xcorr_rejects_oversized_channel_counts():
    """A channel count whose partial-sum scratch would overflow is refused on
    the host with AB_ERR_ARG before anything runs."""
    import ctypes
    from albatros_axion_detection_gb300 import _lib
    lib = _lib.load()
    raw = cu(np.zeros((2, 16, 16), np.uint8))
    ch = cu(np.zeros(4, np.int64))
    out = cu(np.zeros(16, np.int64))
    rc = lib.ab_xcorr_coarse_4bit(_lib.ctx(), raw.data_ptr(), 256, 2, 16, 8, 0, 16, None, ch.data_ptr(), 1 << 40,
                                  16, out.data_ptr(), out.data_ptr(), None)
    assert rc == -1 and b"too large" in lib.ab_last_error()


@pytest.fixture
def tc_engine():
    """Force the tcgen05 form of the coarse correlator for any antenna count."""
    from albatros_axion_detection_gb300 import autotune
    autotune.set_coarse_mma_bits(16)
    autotune.set_coarse_engine(2)
    yield
    autotune.set_coarse_engine(0)
    autotune.set_coarse_tc_slice(0)
    autotune.set_coarse_tc_tma(1)


@pytest.mark.parametrize("nant,nspec,nchan,chunk,ch", [
    (16, 4096, 256, None, "all"),       # 2 channels a tile, 32 channel groups, contiguous 16-byte loads
    (32, 1000, 12, 300, "all"),         # 1 channel a tile (128 rows), ragged chunks and slices
    (2, 2 ** 14, 64, 2 ** 12, "step3"),  # scattered channels: byte loads; most rows zero
    (13, 777, 20, None, "all"),         # ragged channel group (20 = 2 x 8 + 4), odd sample count
    (1, 333, 5, 100, "all"),
])
def test_coarse_xcorr_tcgen05_bit_exact(tc_engine, nant, nspec, nchan, chunk, ch):
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    raw = gen.raw_4bit_uniform(seed=7 * nant + nchan, nspec=nspec, nchan=nchan, nant=nant)
    chans = np.arange(nchan) if ch == "all" else np.arange(0, nchan, 3)
    re, im = xcorr_coarse_4bit(cu(raw), 0, nspec, chans, nchan, chunk=chunk, average=False)
    re, im = re.cpu().numpy(), im.cpu().numpy()
    c = nspec if chunk is None else chunk
    for k in range(re.shape[0]):
        r0, r1 = k * c, min((k + 1) * c, nspec)
        er, ei = io.xcorr_all_ant_4bit(raw, r0, r1, chans, nchan, nthreads=8)
        np.testing.assert_array_equal(re[k], er)
        np.testing.assert_array_equal(im[k], ei)


@pytest.mark.parametrize("nant,nspec,nchan,rowstart,chunk,chans", [
    (16, 5000, 64, 0, 1000, "all"),       # chunks of 15 stages + 40 samples: boxes cross chunk and slice ends
    (7, 3001, 40, 17, None, "from8"),     # 7 antennas (box rows 7-15 read as zero), rows from 17, channels
                                          # 8..34: three TMA groups and a ragged one on 16-byte loads
    (16, 2 ** 16, 256, 64, 2 ** 14, "all"),  # full boxes, 4 chunks
    (4, 2000, 32, 0, None, "step2"),      # scattered channels: no group takes TMA inside the TMA kernel
])
def test_coarse_xcorr_tcgen05_tma_exact(tc_engine, nant, nspec, nchan, rowstart, chunk, chans):
    """The TMA-staged form (packet bytes in a ring of 16 B x 64 samples x 16
    antennas boxes, samples taken in a permuted order) is bit-exact against
    the int64 oracle and equal to the register-load form."""
    from albatros_axion_detection_gb300 import autotune
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    raw = gen.raw_4bit_uniform(seed=nant * 31 + nspec, nspec=rowstart + nspec, nchan=nchan, nant=nant)
    ch = {"all": np.arange(nchan), "from8": np.arange(8, 35), "step2": np.arange(0, nchan, 2)}[chans]
    got = {}
    for tma in (1, 0):
        autotune.set_coarse_tc_tma(tma)
        re, im = xcorr_coarse_4bit(cu(raw), rowstart, rowstart + nspec, ch, nchan, chunk=chunk, average=False)
        got[tma] = (re.cpu().numpy(), im.cpu().numpy())
    np.testing.assert_array_equal(got[1][0], got[0][0])
    np.testing.assert_array_equal(got[1][1], got[0][1])
    c = nspec if chunk is None else chunk
    for k in range(got[1][0].shape[0]):
        r0, r1 = rowstart + k * c, rowstart + min((k + 1) * c, nspec)
        er, ei = io.xcorr_all_ant_4bit(raw, r0, r1, ch, nchan, nthreads=8)
        np.testing.assert_array_equal(got[1][0][k], er)
        np.testing.assert_array_equal(got[1][1][k], ei)


def test_coarse_xcorr_tcgen05_longest_slice_exact(tc_engine):
    """All nibbles 0x8 (+8) over one CTA slice of 2^17 samples, the longest the
    tcgen05 form allows: every fp32 partial sum reaches 64 * 2^17 = 2^23 and
    must stay exact in tensor memory."""
    from albatros_axion_detection_gb300 import autotune
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    autotune.set_coarse_tc_slice(1 << 17)
    nspec = 1 << 17
    raw = np.full((2, nspec, 8), 0x88, np.uint8)
    re, im = xcorr_coarse_4bit(cu(raw), 0, nspec, np.arange(4), 4, average=False)
    assert np.all(re.cpu().numpy() == nspec * 128) and np.all(im.cpu().numpy() == 0)
    # the TMA form (8 contiguous channels, 16-byte rows) stores 16 x the
    # levels: its partial sums reach 256 * 2^23 = 2^31, still exact in fp32
    raw = np.full((2, nspec, 16), 0x88, np.uint8)
    re, im = xcorr_coarse_4bit(cu(raw), 0, nspec, np.arange(8), 8, average=False)
    assert np.all(re.cpu().numpy() == nspec * 128) and np.all(im.cpu().numpy() == 0)
    raw = np.full((2, nspec, 16), 0x99, np.uint8)  # -7 everywhere: the largest negative products
    re, im = xcorr_coarse_4bit(cu(raw), 0, nspec, np.arange(8), 8, average=False)
    assert np.all(re.cpu().numpy() == nspec * 98) and np.all(im.cpu().numpy() == 0)
    # a mixed pattern at the same length: bit-exact against the int64 oracle
    raw = gen.raw_4bit_uniform(seed=17, nspec=nspec, nchan=4, nant=2)
    re, im = xcorr_coarse_4bit(cu(raw), 0, nspec, np.arange(4), 4, average=False)
    er, ei = io.xcorr_all_ant_4bit(raw, 0, nspec, np.arange(4), 4)
    np.testing.assert_array_equal(re.cpu().numpy()[0], er)
    np.testing.assert_array_equal(im.cpu().numpy()[0], ei)


def test_coarse_xcorr_tcgen05_row_lists(tc_engine):
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    raw = gen.raw_4bit(seed=3, nspec=700, nchan=32, nant=2)
    rows = np.stack([np.arange(0, 600), np.arange(100, 700)]).astype(np.int32)
    re, im = xcorr_coarse_4bit(cu(raw), 0, 0, np.arange(32), 32, rows=rows, average=False)
    shifted = np.stack([raw[0, 0:600], raw[1, 100:700]])
    er, ei = io.xcorr_all_ant_4bit(shifted, 0, 600, np.arange(32), 32)
    np.testing.assert_array_equal(re.cpu().numpy()[0], er)
    np.testing.assert_array_equal(im.cpu().numpy()[0], ei)


def test_coarse_xcorr_tcgen05_wait_timeout_reports_fault(tc_engine):
    """Failure path of the tcgen05 correlator's bounded waits, without a GPU
    fault: the producers withhold their first stage (nothing ever signals it),
    the MMA thread's wait runs out after about 2 s, and the call returns with
    every output INT64_MIN; the tensor memory was freed, so the next call is
    exact again."""
    import time
    from albatros_axion_detection_gb300 import _lib, autotune
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    raw = gen.raw_4bit_uniform(seed=99, nspec=4096, nchan=16, nant=12)
    _lib.call("ab_ctx_set_option", _lib.ctx(), autotune.OPT_FAULT_TEST, 1)
    t0 = time.time()
    re, im = xcorr_coarse_4bit(cu(raw), 0, 4096, np.arange(16), 16, average=False)
    re, im = re.cpu().numpy(), im.cpu().numpy()
    assert time.time() - t0 < 30
    assert np.all(re == np.iinfo(np.int64).min) and np.all(im == np.iinfo(np.int64).min)
    re, im = xcorr_coarse_4bit(cu(raw), 0, 4096, np.arange(16), 16, average=False)
    er, ei = io.xcorr_all_ant_4bit(raw, 0, 4096, np.arange(16), 16)
    np.testing.assert_array_equal(re.cpu().numpy()[0], er)
    np.testing.assert_array_equal(im.cpu().numpy()[0], ei)


def test_coarse_xcorr_worst_case_magnitudes(mma_bits):
    """All nibbles 0x8 (+8): the largest products, exact in the int32 / fp32
    partial sums (4096 samples x 64 per CTA slice)."""
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    raw = np.full((2, 8192, 8), 0x88, np.uint8)
    re, im = xcorr_coarse_4bit(cu(raw), 0, 8192, np.arange(4), 4, average=False)
    assert np.all(re.cpu().numpy() == 8192 * 128) and np.all(im.cpu().numpy() == 0)


def test_coarse_xcorr_row_lists(mma_bits):
    from albatros_axion_detection_gb300.correlations import xcorr_coarse_4bit
    raw = gen.raw_4bit(seed=3, nspec=700, nchan=32, nant=2)
    rows = np.stack([np.arange(0, 600), np.arange(100, 700)]).astype(np.int32)
    re, im = xcorr_coarse_4bit(cu(raw), 0, 0, np.arange(32), 32, rows=rows, average=False)
    shifted = np.stack([raw[0, 0:600], raw[1, 100:700]])
    er, ei = io.xcorr_all_ant_4bit(shifted, 0, 600, np.arange(32), 32)
    np.testing.assert_array_equal(re.cpu().numpy()[0], er)
    np.testing.assert_array_equal(im.cpu().numpy()[0], ei)


def test_pairs_4bit_golden(golden_int):
    from albatros_axion_detection_gb300 import correlations as cr
    d0, d1 = gen.sorted_4bit_pair(seed=21, nrows=2000, ncol=33)
    got = cr.avg_xcorr_4bit(cu(d0), cu(d1), np.arange(2000))
    np.testing.assert_array_equal(got, golden_int["x4_sum"] / 2000)
    s0, s1 = gen.specnum_pair(seed=22, n=2000, span=2600)
    got = cr.avg_xcorr_4bit_2ant(cu(d0), cu(d1), s0, s1, 0, 0)
    np.testing.assert_array_equal(got, golden_int["x4_2ant_sum"] / int(golden_int["x4_2ant_rows"]))
    assert np.isnan(cr.avg_xcorr_4bit(d0, d1, []))


def test_pairs_1bit_golden(golden_int):
    from albatros_axion_detection_gb300 import correlations as cr
    for nch in (32, 29):
        nb = int(np.ceil(nch / 4))
        e0, e1 = gen.sorted_1bit_pair(seed=23 + nch, nrows=1500, nbytes=nb)
        got = cr.avg_xcorr_1bit(cu(e0), cu(e1), np.arange(1500), nch)
        np.testing.assert_array_equal(got, golden_int[f"x1_{nch}_sum"] / 1500)
    e0, e1 = gen.sorted_1bit_pair(seed=31, nrows=2000, nbytes=8)
    s0, s1 = gen.specnum_pair(seed=22, n=2000, span=2600)
    vv, n = cr.avg_xcorr_1bit_vanvleck_2ant(cu(e0), cu(e1), 32, s0, s1, 0, 0)
    assert n == int(golden_int["vv_2ant_rows"])
    np.testing.assert_array_equal(np.stack(vv), golden_int["vv_2ant"])
    vv1 = cr.avg_xcorr_1bit_vanvleck(cu(e0), cu(e1), np.arange(2000), 32)
    exp = io.vanvleck_sums(e0, e1, 32, 2000)
    for a, b in zip(vv1, exp):
        np.testing.assert_array_equal(a, b.astype(np.float32) / 2000)


def test_float_gpu_single_baseline():
    from albatros_axion_detection_gb300 import correlations as cr
    rng = np.random.default_rng(4)
    d0 = (rng.standard_normal((1000, 16)) + 1j * rng.standard_normal((1000, 16))).astype(np.complex64)
    d1 = (rng.standard_normal((1000, 16)) + 1j * rng.standard_normal((1000, 16))).astype(np.complex64)
    sn = np.arange(900)
    got, n = cr.avg_xcorr_4bit_float_gpu(cu(d0), cu(d1), sn, sn)
    exp = (d0[:900].astype(np.complex128) * np.conj(d1[:900])).mean(0)
    assert n == 900 and np.linalg.norm(got.cpu().numpy() - exp) / np.linalg.norm(exp) < 1e-5
