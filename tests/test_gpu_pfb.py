"""GPU parity: matft / filter / IPFB / PFB vs the FP64 oracle and the
reference's golden outputs.  Tolerances are norm-wise relative errors:
FP32 arithmetic with FP64-derived twiddles."""
import numpy as np
import pytest
import torch

from oracle import pfb_oracle as po
from tests.golden import gen

pytestmark = pytest.mark.gpu
TOL_FILTER = 1e-6   # FP64 compute, rounded to complex64
TOL_FFT = 2e-6      # FP32 FFT chains


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b)


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("nslice", [12, 64, 4096, 32928])
def test_matft_and_filter(nslice):
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    m = pu.get_matft(nslice).cpu().numpy()
    mo = po.get_matft(nslice)
    assert rel(m, mo) < TOL_FILTER
    f = pu.calculate_filter(pu.get_matft(nslice), 0.45).cpu().numpy()
    fo = po.calculate_filter(mo, 0.45)
    assert rel(f, fo) < TOL_FILTER
    fb = pu.build_filter(nslice, 0.45).cpu().numpy()
    assert rel(fb, fo) < TOL_FILTER


def test_ipfb_golden(golden_pfb):
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    dat = gen.ipfb_input(seed=41, nslice=12)
    filt = pu.calculate_filter(cu(golden_pfb["matft_12"]), 0.45)
    res = pu.cupy_ipfb(cu(dat), filt)
    assert res.shape == (12, 4096) and res.stride() == (1, 12)
    got = res.cpu().numpy()[2:-2].ravel()
    assert rel(got, golden_pfb["ipfb_12_cut2"]) < TOL_FFT


@pytest.mark.parametrize("nslice", [2, 12, 64, 98, 1000, 4096, 32928])
def test_ipfb_vs_oracle(nslice):
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    dat = gen.ipfb_input(seed=nslice, nslice=nslice)
    filt = pu.build_filter(nslice, 0.45)
    got = pu.cupy_ipfb(cu(dat), filt).cpu().numpy()
    exp = po.ipfb(dat.astype(np.complex128), filt.cpu().numpy().astype(np.complex128))
    assert rel(got, exp) < TOL_FFT


@pytest.mark.parametrize("nslice", [22, 1044, 2018, 8212, 32788])
def test_ipfb_any_length_vs_oracle(nslice):
    """Lengths whose nslice/2 has a prime factor above 7 (11; 29; 1009; 2053;
    1171, the reference's default cut on 2^15 spectra) run their time-axis
    transforms with direct DFT passes for those factors, like cuFFT runs any
    length for the reference."""
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    dat = gen.ipfb_input(seed=nslice, nslice=nslice)
    filt = pu.build_filter(nslice, 0.45)
    got = pu.cupy_ipfb(cu(dat), filt).cpu().numpy()
    exp = po.ipfb(dat.astype(np.complex128), filt.cpu().numpy().astype(np.complex128))
    assert rel(got, exp) < TOL_FFT


def test_ipfb_rejects_odd_length():
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    from albatros_axion_detection_gb300._lib import AlbatrosError
    dat = gen.ipfb_input(seed=1, nslice=21)
    with pytest.raises((ValueError, AlbatrosError)):
        pu.cupy_ipfb(cu(dat), torch.zeros((4096, 11), dtype=torch.complex64, device="cuda"))


def test_pfb_golden(golden_pfb):
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    ts = gen.timestream(seed=42, n=4096 * 2 * 7)
    win = po.sinc_hamming(4, 8192).astype(np.float32)
    got = pu.cupy_pfb(cu(ts), win, nchan=4097).cpu().numpy()
    assert got.shape == golden_pfb["pfb_os2"].shape
    assert rel(got, golden_pfb["pfb_os2"]) < TOL_FFT


@pytest.mark.parametrize("lblock,nblock", [(64, 5), (1024, 3), (4096, 7), (8192, 4), (4096 * 16, 3), (4096 * 64, 2)])
def test_pfb_vs_oracle(lblock, nblock):
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    ts = gen.timestream(seed=lblock, n=lblock * (nblock + 3) + 17)
    win = po.sinc_hamming(4, lblock).astype(np.float32)
    got = pu.cupy_pfb(cu(ts), win, nchan=lblock // 2 + 1).cpu().numpy()
    exp = po.pfb(ts, win.astype(np.float64), nchan=lblock // 2 + 1)
    assert got.shape == exp.shape
    assert rel(got, exp) < TOL_FFT


@pytest.mark.parametrize("osamp,c0,c1", [(64, 100, 164), (16, 0, 7), (1, 5, 2049), (4, 2047, 2048)])
def test_pfb_band_matches_full(osamp, c0, c1):
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pu
    lblock = 4096 * osamp
    ts = gen.timestream(seed=osamp, n=lblock * 6)
    win = po.sinc_hamming(4, lblock).astype(np.float32)
    full = po.pfb(ts, win.astype(np.float64), nchan=lblock // 2 + 1)
    q1 = min(c1 * osamp, lblock // 2 + 1)
    band = pu.cupy_pfb_band(cu(ts), win, c0 * osamp, q1, nchan=lblock // 2 + 1).cpu().numpy()
    assert rel(band, full[:, c0 * osamp:q1]) < TOL_FFT
