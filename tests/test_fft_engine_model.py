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


def plan_any(n):
    """make_plan_any (csrc/api.cu): radices 8, 4, 2, 7, 5, 3 as far as they
    divide n, then each remaining prime factor as one direct DFT pass."""
    radices, m = [], n
    for r in (8, 4, 2, 7, 5, 3):
        while m % r == 0:
            radices.append(r)
            m //= r
    f = 11
    while f * f <= m:
        while m % f == 0:
            radices.append(f)
            m //= f
        f += 2
    if m > 1:
        radices.append(m)
    return radices


@pytest.mark.parametrize("n", [16394, 2 * 13 * 11, 4 * 1009, 3 * 11 * 11, 1009])
def test_any_length_plans_with_direct_dft_passes(n):
    """nslice/2 of the reference's default cut (16394 = 2 * 7 * 1171) and
    other lengths with prime factors above 7: the plan multiplies to n, its
    direct DFT passes land frequencies in the same digit-reversed positions,
    and forward -> pointwise -> inverse is circular filtering."""
    radices = plan_any(n)
    assert int(np.prod(radices)) == n and len(radices) <= 12
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    X = dif_forward(x, radices)
    pos = positions(n, radices)
    assert np.array_equal(np.sort(pos), np.arange(n))
    np.testing.assert_allclose(X[pos], np.fft.fft(x), atol=1e-8 * np.sqrt(n))
    H = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    Hpos = np.empty(n, complex)
    Hpos[pos] = H
    y = dit_inverse(X * Hpos, radices) / n
    np.testing.assert_allclose(y, np.fft.ifft(np.fft.fft(x) * H), atol=1e-9)


@pytest.mark.parametrize("R,S,T", [(1171, 1, 32788), (1171, 2, 32788), (13, 22, 572)])
def test_direct_pass_twiddle_indices(R, S, T):
    """generic_pass (csrc/fft.cuh): stepping e += k (mod R) gives (r k) mod R,
    and every table index j k (T / (R S)), e (T / R) stays below T."""
    assert T % (R * S) == 0
    tstep, rstep = T // (R * S), T // R
    for k in (0, 1, R // 2, R - 1):
        e = 0
        for r in range(R):
            assert e == (r * k) % R and e * rstep < T
            e += k
            if e >= R:
                e -= R
    assert (S - 1) * (R - 1) * tstep < T


def smooth_at_least(n):
    """The smallest length >= n whose prime factors are 2, 3, 5, 7."""
    while True:
        m = n
        for r in (2, 3, 5, 7):
            while m % r == 0:
                m //= r
        if m == 1:
            return n
        n += 1


@pytest.mark.parametrize("R", [1171, 1009, 2053, 37])
def test_bluestein_pass_restatement(R):
    """bluestein_pass (csrc/fft.cuh) with the tables of get_bluestein
    (csrc/api.cu): a = x c (c_m = exp(-i pi (m^2 mod 2R) / R)), circular
    convolution of length L (7-smooth, >= 2R - 1) with conj(c) wrapped around,
    times c again, is the length-R DFT; the inverse as conj(DFT(conj x))."""
    L = smooth_at_least(2 * R - 1)
    m = np.arange(R)
    c = np.exp(-1j * np.pi * ((m * m) % (2 * R)) / R)
    b = np.zeros(L, complex)
    b[:R] = np.conj(c)
    b[L - R + 1:] = np.conj(c[1:][::-1])
    filt = np.fft.fft(b) / L
    rng = np.random.default_rng(R)
    x = rng.standard_normal(R) + 1j * rng.standard_normal(R)
    a = np.zeros(L, complex)
    a[:R] = x * c
    conv = np.fft.ifft(np.fft.fft(a) * filt) * L  # the engine's unnormalised inverse, filter carries 1/L
    np.testing.assert_allclose(conv[:R] * c, np.fft.fft(x), atol=1e-9 * np.sqrt(R))
    a[:R] = np.conj(x) * c
    conv = np.fft.ifft(np.fft.fft(a) * filt) * L
    np.testing.assert_allclose(np.conj(conv[:R] * c), R * np.fft.ifft(x), atol=1e-9 * np.sqrt(R))
