"""CPU model of the IIR time stage's per-item schedule (csrc/fir.cu,
iir_fold_kernel) against the exact circular Wiener filter of the reference's
cupy_ipfb (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91, filter of
calculate_filter :29-36 on get_matft :123-137).

Per column n the reference multiplies the time-axis spectrum by
filt = m (1+t^2) / (t^2 + |m|^2), m = W(z) = sum_k w[k P + n] z^-k on the unit
circle.  The kernel applies the same filter as g W(z) / (A(z) A(1/z)) (4-tap
FIR, causal and anti-causal 3-pole recursions) with each of 256 threads
owning U rows: zero-state passes, then start states built from the D
neighbours' end states, zf(k-1) + Phi zf(k-2) + ..., where Phi (U rows of the
homogeneous recursion) acts through five samples of 1/A's impulse response.
This model runs that schedule in float32, vectorised over threads, and checks
it against the exact filter in float64.
"""
import numpy as np
import pytest

P, THRESH, NTHREADS = 4096, 0.45, 256


def sinc_hamming(ntap, L):
    N = ntap * L
    n = np.arange(N)
    return np.hamming(N) * np.sinc((n - N / 2) / L)


def factor(w, t):
    """Monic minimum-phase A (degree 3) and b0^2 with t^2 + W(z)W(1/z) = b0^2 A(z)A(1/z)."""
    d = np.array([sum(w[i] * w[i + k] for i in range(4 - k)) for k in range(4)])
    d[0] += t * t
    m = max([k for k in range(4) if abs(d[k]) > 1e-12 * abs(d[0])] + [0])  # degree of D (column 0: m = 0)
    a = np.zeros(4)
    a[0] = 1.0
    if m == 0:
        return a, d[0]
    r = np.roots(np.concatenate([d[m:0:-1], d[:m + 1]]))  # z^m D(z), palindromic of degree 2m
    a[:m + 1] = np.real(np.poly(r[np.abs(r) < 1]))
    return a, d[m] / a[m]


def impulse(a, n):
    h = np.zeros(n)
    h[0] = 1.0
    for k in range(1, n):
        h[k] = -sum(a[j] * h[k - j] for j in (1, 2, 3) if k >= j)
    return h


def carry_rows(h):
    """Rows after which 1/A's impulse response stays below 1e-10 of its peak, rounded up to 40 or 80."""
    last = np.max(np.nonzero(np.abs(h) > 1e-10 * np.abs(h).max())[0]) + 1
    return 40 if last <= 40 else 80 if last <= 80 else None


def recursion(vals, s, A):
    """v[m] = vals[m] - a1 v[m-1] - a2 v[m-2] - a3 v[m-3], per thread (axis 0); s = (v[-1], v[-2], v[-3])."""
    f = np.float32
    out = np.empty_like(vals)
    p1, p2, p3 = s[:, 0].copy(), s[:, 1].copy(), s[:, 2].copy()
    for m in range(vals.shape[1]):
        v = (vals[:, m] - A[0] * p1 - A[1] * p2 - A[2] * p3).astype(f)
        p3, p2, p1 = p2, p1, v
        out[:, m] = v
    return out, np.stack([p1, p2, p3], axis=1)


def incoming(z, D, direction, A, hh):
    """sum over d = 1..D of Phi^(d-1) z[k + direction*d], terms outside the threads omitted."""
    f = np.float32
    n = z.shape[0]
    s = np.zeros_like(z)
    for d in range(D, 0, -1):
        if d < D:  # s <- Phi s through the impulse response hh = h[U-5:U]
            u0 = -(A[0] * s[:, 0] + A[1] * s[:, 1] + A[2] * s[:, 2])
            u1 = -(A[1] * s[:, 0] + A[2] * s[:, 1])
            u2 = -A[2] * s[:, 0]
            s = np.stack([hh[4] * u0 + hh[3] * u1 + hh[2] * u2, hh[3] * u0 + hh[2] * u1 + hh[1] * u2,
                          hh[2] * u0 + hh[1] * u1 + hh[0] * u2], axis=1).astype(f)
        j = np.arange(n) + direction * d
        ok = (j >= 0) & (j < n)
        s[ok] += z[j[ok]]
    return s


def schedule_error(U, D, n):
    """Norm-wise error of one item of the kernel's schedule for column n."""
    f = np.float32
    nslice = 4 * P + 160
    w = sinc_hamming(4, P)[np.arange(4) * P + n]
    a, b0sq = factor(w, THRESH)
    g = (1 + THRESH ** 2) / b0sq
    h = impulse(a, 200)
    assert carry_rows(h) == 40  # the default threshold carries states over 40 rows

    # the factored filter is the reference's Wiener filter on the unit circle
    z = np.exp(2j * np.pi * np.fft.fftfreq(nslice))
    Wz = sum(w[k] * z ** (-k) for k in range(4))
    Az = sum(a[k] * z ** (-k) for k in range(4))
    Azi = sum(a[k] * z ** k for k in range(4))
    H = g * Wz / (Az * Azi)
    filt = Wz * (1 + THRESH ** 2) / (THRESH ** 2 + np.abs(Wz) ** 2)
    np.testing.assert_allclose(H, filt, rtol=1e-10, atol=1e-12)

    x = np.random.default_rng(n + 7 * U).standard_normal(nslice)
    y_exact = np.real(np.fft.ifft(np.fft.fft(x) * H))

    # one item: computed rows [ylo, ylo + nrows), threads own U rows from ylo - D*U
    ylo, nrows = 1000, (NTHREADS - 2 * D) * U
    nthr = min(NTHREADS, (D * U + nrows - 1) // U + D + 1)
    xw = x[(ylo - D * U - 3 + np.arange(nthr * U + 3)) % nslice].astype(f)
    cw = (g * w).astype(f)
    A = a[1:].astype(f)
    hh = h[U - 5:U].astype(f)
    rows = np.arange(nthr)[:, None] * U + np.arange(U)[None, :]
    u = (cw[0] * xw[rows + 3] + cw[1] * xw[rows + 2] + cw[2] * xw[rows + 1] + cw[3] * xw[rows]).astype(f)
    zero = np.zeros((nthr, 3), f)
    _, zf = recursion(u, zero, A)                             # pass 1: causal, zero state
    v, _ = recursion(u, incoming(zf, D, -1, A, hh), A)        # pass 2: from the true start state
    _, zb = recursion(v[:, ::-1].copy(), zero, A)             # pass 3: anti-causal, zero state
    yk, _ = recursion(v[:, ::-1].copy(), incoming(zb, D, 1, A, hh), A)  # pass 4
    y = yk[:, ::-1][D:].reshape(-1)[:nrows]
    ye = y_exact[(ylo + np.arange(nrows)) % nslice]
    return np.linalg.norm(y - ye) / np.linalg.norm(ye)


@pytest.mark.parametrize("U,D", [(21, 2), (41, 1), (21, 4), (41, 2), (67, 1), (67, 2)])  # D*U >= 40: the tiles the library runs
@pytest.mark.parametrize("n", [0, 1, 1000, 2048, 2112, 4095])  # 2112: 1/A decays slowest (37 rows)
def test_iir_schedule_matches_exact_filter(U, D, n):
    assert schedule_error(U, D, n) < 1e-6


def test_iir_schedule_needs_the_full_carry():
    """With short thread ranges the carried states are what links the threads:
    over 9 or 18 rows the slowest column misses the bound, over 45 it meets it."""
    assert schedule_error(9, 1, 2112) > 1e-4
    assert schedule_error(9, 2, 2112) > 1e-6
    assert schedule_error(9, 5, 2112) < 1e-6
