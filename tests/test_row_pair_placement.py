"""CPU check of the row stage's time-pair placement (csrc/ipfb.cu, put_pair_t)
against the reference's row transform, irfft(dat, axis=1) over 2*(2049-1)
points (albatros_analysis/src/utils/pfb_gpu_utils.py:56-91 via
pycufft.irfft, which divides by n).

Two spectra A, B (consecutive rows of one input, or the two pols) share one
complex inverse FFT: bin k gets A_k + i B_k, bin P-k gets conj(A_k) + i conj(B_k),
and the DC and Nyquist bins take only the real parts (irfft ignores their
imaginary parts).  The real and imaginary parts of the result are then the
two real transforms.  Also checks the prefetching row stage's byte decode
(32-bit word loads, byte shifts, 4-bit nibbles and 1-bit bit pairs) against
the oracle's unpack.
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


def row_stage_decode(raw2d, cols, bits, pol):
    """The prefetching row stage's decode (csrc/ipfb.cu, row_stage_tpair_pf_kernel):
    each thread loads the little-endian 32-bit word holding its byte (byte
    offset 2*col + pol for 4-bit, col >> 1 for 1-bit, word at offset & ~3),
    shifts the byte out, and decodes it.  Returns (rows, len(cols)) complex."""
    nrow, rb = raw2d.shape
    words = raw2d.reshape(nrow, rb // 4, 4).astype(np.uint32)
    words = words[..., 0] | (words[..., 1] << 8) | (words[..., 2] << 16) | (words[..., 3] << 24)
    out = np.zeros((nrow, len(cols)), complex)
    for j, col in enumerate(cols):
        boff = 2 * col + pol if bits == 4 else col >> 1
        b = (words[:, boff >> 2] >> (8 * (boff & 3))) & 0xFF
        if bits == 4:
            out[:, j] = (((b >> 4) + 7) & 15) - 7 + 1j * (((b & 15) + 7) & 15) - 7j
        else:
            q = (b >> (0 if col & 1 else 4)) & 15
            s2 = 0 if pol else 2
            out[:, j] = (((q >> (s2 + 1)) & 1) * 2 - 1) + 1j * (((q >> s2) & 1) * 2 - 1)
    return out


@pytest.mark.parametrize("bits,nchan", [(4, 64), (4, 2048), (1, 64), (1, 2048)])
def test_row_stage_decode_matches_oracle_unpack(bits, nchan):
    """Word loads + byte shifts + nibble / bit decode equal the reference's
    unpack (the oracle's C restatement of unpacking.c:155-246, pinned to the
    reference's fixtures)."""
    from oracle import int_oracle as io
    from tests.golden import gen
    raw = gen.raw_4bit(seed=nchan, nspec=40, nchan=nchan) if bits == 4 else gen.raw_1bit(seed=nchan, nspec=40,
                                                                                          nchan=nchan)
    if bits == 4:
        cols = np.array([0, 1, 2, 3, 5, nchan // 2, nchan - 1])
        e0, e1 = io.unpack_4bit(raw, 0, 40, cols, nchan)
    else:
        c0, c1 = 2, nchan - 2
        cols = np.arange(c0, c1)
        e0, e1 = io.unpack_1bit(raw, 0, 40, c0, c1, nchan)
    np.testing.assert_array_equal(row_stage_decode(raw, cols, bits, 0), e0)
    np.testing.assert_array_equal(row_stage_decode(raw, cols, bits, 1), e1)
