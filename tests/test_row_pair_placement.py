"""CPU check of the row stage's time-pair placement (csrc/ipfb.cu, put_pair_t)
against the reference's row transform, irfft(dat, axis=1) over 2*(2049-1)
points (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91 via
pycufft.irfft, which divides by n).

Two spectra A, B (consecutive rows of one input, or the two pols) share one
complex inverse FFT: bin k gets A_k + i B_k, bin P-k gets conj(A_k) + i conj(B_k),
and the DC and Nyquist bins take only the real parts (irfft ignores their
imaginary parts).  The real and imaginary parts of the result are then the
two real transforms.
"""
import numpy as np
import pytest

P = 4096


def put_pair(A, B, chans):
    """Full P-bin buffer as put_pair_t fills it for the selected channels."""
    buf = np.zeros(P, complex)
    for k in chans:
        a, b = A[k], B[k]
        if k == 0 or 2 * k == P:
            buf[k] = complex(a.real, b.real)
        else:
            buf[k] = a + 1j * b
            buf[P - k] = np.conj(a) + 1j * np.conj(b)
    return buf


@pytest.mark.parametrize("chans", [np.arange(0, 2049), np.arange(100, 164), np.array([0, 1, 2047, 2048]),
                                   np.array([5, 900, 2048])])
def test_time_pair_equals_two_irffts(chans):
    rng = np.random.default_rng(len(chans))
    A = np.zeros(P // 2 + 1, complex)
    B = np.zeros(P // 2 + 1, complex)
    A[chans] = rng.standard_normal(len(chans)) + 1j * rng.standard_normal(len(chans))  # imag at DC/Nyquist too
    B[chans] = rng.standard_normal(len(chans)) + 1j * rng.standard_normal(len(chans))
    z = np.fft.ifft(put_pair(A, B, chans))  # the kernel: unnormalised inverse, then * 1/P
    np.testing.assert_allclose(z.real, np.fft.irfft(A, n=P), atol=1e-12)
    np.testing.assert_allclose(z.imag, np.fft.irfft(B, n=P), atol=1e-12)
