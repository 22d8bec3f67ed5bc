"""CPU model of the library's FFT passes (csrc/fft.cuh dif_pass / dit_pass,
csrc/fft_static.cuh), which replace the reference's cuFFT calls
(albatros_analysis/src/utils/pycufft.py:27-161).

A forward transform runs decimation-in-frequency passes of radices
R_1 .. R_m in order: pass p (span S_p = n / (R_1 .. R_p)) takes each group of
R_p elements S_p apart, applies the radix-R_p DFT, and multiplies output k of
the butterfly at offset j by exp(-2 pi i j k / (R_p S_p)).  Frequency f,
written in mixed radix f = f_1 + R_1 f_2 + R_1 R_2 f_3 + ..., ends at
position pos(f) = sum_p f_p S_p.  The inverse runs the adjoint passes in
reverse order (conjugate twiddle, then the inverse butterfly), taking
digit-reversed input to natural order, so forward -> pointwise -> inverse
needs no permutation.  Checked here for the compile-time plans (4096 =
16*16*16, 16464 = 7*7*7*3*16, 16384) and radix orders the autotuner tries.
"""
import numpy as np
import pytest


def _dft_matrix(R, sign):
    k = np.arange(R)
    return np.exp(sign * 2j * np.pi * np.outer(k, k) / R)


def dif_forward(x, radices):
    x = np.asarray(x, complex).copy()
    n, S = x.size, x.size
    for R in radices:
        S //= R
        v = x.reshape(n // (R * S), R, S)                      # [block][r][j], element base + r*S
        v = np.einsum("kr,brj->bkj", _dft_matrix(R, -1), v)    # butterfly
        v *= np.exp(-2j * np.pi * np.outer(np.arange(R), np.arange(S)) / (R * S))[None]  # twiddle j*k
        x = v.reshape(n)
    return x


def dit_inverse(X, radices):
    X = np.asarray(X, complex).copy()
    n = X.size
    spans = []
    S = n
    for R in radices:
        S //= R
        spans.append((R, S))
    for R, S in reversed(spans):
        v = X.reshape(n // (R * S), R, S)
        v = v * np.exp(2j * np.pi * np.outer(np.arange(R), np.arange(S)) / (R * S))[None]  # conjugate twiddle
        v = np.einsum("kr,brj->bkj", _dft_matrix(R, 1), v)     # inverse butterfly
        X = v.reshape(n)
    return X  # unnormalised: n * ifft


def positions(n, radices):
    pos = np.zeros(n, np.int64)
    f = np.arange(n)
    S, place = n, 1
    for R in radices:
        S //= R
        pos += ((f // place) % R) * S
        place *= R
    return pos


ORDERS = [(16, 16, 16), (7, 7, 7, 3, 16), (16, 16, 16, 4), (8, 8, 8, 8), (2, 3, 4, 5, 7), (3, 7, 8, 7, 7, 2),
          (8, 4, 7, 7, 3)]


@pytest.mark.parametrize("radices", ORDERS)
def test_forward_lands_in_digit_reversed_positions(radices):
    n = int(np.prod(radices))
    x = np.random.default_rng(n).standard_normal(n) + 1j * np.random.default_rng(n + 1).standard_normal(n)
    X = dif_forward(x, radices)
    pos = positions(n, radices)
    assert np.array_equal(np.sort(pos), np.arange(n))
    np.testing.assert_allclose(X[pos], np.fft.fft(x), atol=1e-9 * np.sqrt(n))


@pytest.mark.parametrize("radices", ORDERS)
def test_forward_pointwise_inverse_needs_no_permutation(radices):
    """The time stage's filter: multiply the digit-reversed spectrum by the
    filter at the same positions and invert; equals circular filtering."""
    n = int(np.prod(radices))
    rng = np.random.default_rng(3 * n)
    x = rng.standard_normal(n)
    H = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    pos = positions(n, radices)
    Hpos = np.empty(n, complex)
    Hpos[pos] = H
    y = dit_inverse(dif_forward(x, radices) * Hpos, radices) / n
    np.testing.assert_allclose(y, np.fft.ifft(np.fft.fft(x) * H), atol=1e-9)


def test_autotuner_orders_are_valid_plans():
    """Every radix order the autotuner proposes for the bench's nslice/2
    multiplies to the length and uses the radices the passes carry."""
    from albatros_axion_detection_gb300 import autotune
    assert autotune.factorise(16394) is None  # cut 10: nslice/2 = 2 * 7 * 1171 has no FFT plan
    for n in (16464, 16384, 4096 * 3):
        for order in autotune.candidate_orders(n, limit=24):
            assert int(np.prod(order)) == n and set(order) <= {2, 3, 4, 5, 7, 8}
