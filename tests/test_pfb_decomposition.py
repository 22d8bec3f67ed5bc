"""CPU check of the forward-PFB decomposition the GPU stages use (csrc/pfb.cuh,
csrc/pfb.cu) against a direct real FFT of the folded block, as in the
reference's cupy_pfb (albatros_analysis/src/utils/pfb_gpu_utils.py:105-121).

For lblock L = P*O (P = 4096) and a tap-folded block y[k], k = n + P t':
  stage A  W_s[n] = sum_t' y[n + P t'] w_O^(s t')            s = 0 .. O/2 (real input)
  stage B  Y[O u + s] = sum_n w_P^(u n) w_L^(s n) W_s[n]       one P-point DFT per slot s
and, the block being real, the slot-s transform Z_s also gives the mirror
offset: Y[O u + O - s] = conj Z_s[P - 1 - u].  Slots 0 .. O/2 - 1 with their
mirrors, plus W_{O/2} (carried with W_0 in the packed record), cover every
fine offset.  The band kernels take w_L^e from three 64-entry tables indexed
by the 6-bit digits of e (e < 2^18), and split w_L^(s n) for n = tid + 256 q
into a per-thread and a per-q factor.
"""
import numpy as np
import pytest

P = 4096


def w(N, e):
    return np.exp(-2j * np.pi * np.asarray(e, dtype=np.float64) / N)


def tw3(e, L):
    """w_L^e from the digit tables of pfb_stage_band2_kernel: [w^(4096 i)], [w^(64 i)], [w^i], i < 64."""
    e = np.asarray(e)
    assert (e < 1 << 18).all()
    t_hi = np.where(np.arange(64) * 4096 < L, w(L, np.arange(64) * 4096), 1.0)
    t_mid = np.where(np.arange(64) * 64 < L, w(L, np.arange(64) * 64), 1.0)
    t_lo = w(L, np.arange(64))
    return t_hi[e >> 12] * t_mid[(e >> 6) & 63] * t_lo[e & 63]


@pytest.mark.parametrize("O", [4, 16, 64])
def test_stage_a_b_with_mirrors_equals_rfft(O):
    L = P * O
    y = np.random.default_rng(O).standard_normal(L)
    ref = np.fft.rfft(y)                                   # (L/2 + 1,) bins, q = O u + s
    Wa = np.fft.fft(y.reshape(O, P), axis=0)[: O // 2 + 1]  # stage A: W_s[n], s <= O/2
    Y = np.zeros(L // 2 + 1, complex)
    n = np.arange(P)
    for s in range(O // 2):
        Z = np.fft.fft(Wa[s] * w(L, s * n))               # stage B for slot s
        Y[O * np.arange(P // 2) + s] = Z[: P // 2]
        if s:
            u = np.arange(P // 2)                          # mirror offset O - s
            Y[O * u + O - s] = np.conj(Z[P - 1 - u])
    Z = np.fft.fft(Wa[O // 2] * w(L, (O // 2) * n))        # W_{O/2}, the second round of slot 0
    Y[O * np.arange(P // 2) + O // 2] = Z[: P // 2]
    Y[L // 2] = np.fft.fft(Wa[0] * w(L, 0 * n))[P // 2]   # Nyquist bin: u = P/2, s = 0
    np.testing.assert_allclose(Y, ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())


@pytest.mark.parametrize("O", [1, 2, 4, 16, 64])
def test_twiddle_digit_tables(O):
    L = P * O
    e = np.arange(L)
    np.testing.assert_allclose(tw3(e, L), w(L, e), atol=1e-12)


@pytest.mark.parametrize("O", [4, 64])
def test_twiddle_split_per_thread_and_pass(O):
    """w_L^(s n) = w_L^(s tid) * w_L^(256 s q) for n = tid + 256 q (256 threads, 16 passes)."""
    L = P * O
    tid = np.arange(256)[:, None]
    q = np.arange(16)[None, :]
    for s in (1, O // 2 - 1, O - 1):
        n = tid + 256 * q
        lhs = w(L, (s * n) % L)
        rhs = tw3((s * tid) % L, L) * w(L, (256 * s * q) % L)
        np.testing.assert_allclose(lhs, rhs, atol=1e-12)
