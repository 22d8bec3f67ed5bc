"""CPU model of the tensor-core IPFB row stage (csrc/row_tc.cu): the inverse
real FFT of a spectrum with nsel selected channels as the product of a
cos/sin basis with the decoded 4-bit levels.

Checked here: the basis (scaled by 2^11, split into fp16 hi and lo parts) and
the levels give the reference's irfft (albatros_analysis/src/utils/
pfb_gpu_utils.py:56-91 starts with cupy's irfft of each 2049-bin spectrum)
to about 1e-7 with fp32 accumulation; the split error is at most 2^-23 per
basis entry; the pre-swizzled image (128-row K-major tiles, 128-byte
swizzle) holds every (phase, K) entry exactly once at the place the MMA reads
it; and the B tile a decoder thread writes (row, chunk) covers every entry
once."""
import numpy as np
import pytest

from oracle import pfb_oracle as po

P, SCALE = 4096, 2048.0


def basis(kabs):
    n = np.arange(P)[:, None]
    k = np.asarray(kabs)[None, :]
    ak = np.where((k == 0) | (2 * k == P), 1.0 / P, 2.0 / P)
    th = 2 * np.pi * ((k * n) % P) / P
    A = np.empty((P, 2 * len(kabs)))
    A[:, 0::2] = SCALE * ak * np.cos(th)
    A[:, 1::2] = -SCALE * ak * np.sin(th)
    return A


def split(A):
    hi = A.astype(np.float16)
    lo = (A - hi.astype(np.float64)).astype(np.float16)
    return hi, lo


def sw128(row, c):
    return row * 128 + (((c ^ row) & 7) << 4)


@pytest.mark.parametrize("kabs", [list(range(1000, 1064)), [0, 5, 2048, 7, 2047], list(range(0, 128, 2))[:33]])
def test_basis_product_matches_irfft(kabs):
    rng = np.random.default_rng(len(kabs))
    nsel = len(kabs)
    A = basis(kabs)
    hi, lo = split(A)
    assert np.max(np.abs(A - hi.astype(np.float64) - lo.astype(np.float64))) <= 2.0 ** -23
    raw = rng.integers(0, 256, (64, nsel), dtype=np.uint8)  # 64 spectra, one pol
    re, im = po.decode_4bit(raw)
    B = np.empty((64, 2 * nsel), np.float32)
    B[:, 0::2], B[:, 1::2] = re, im
    # fp32 accumulation of the exact fp16 x small-integer products, as the MMA
    D = (hi.astype(np.float32) @ B.T + lo.astype(np.float32) @ B.T) / np.float32(SCALE)
    spec = np.zeros((64, P // 2 + 1), np.complex128)
    spec[:, kabs] = re + 1j * im
    ref = np.fft.irfft(spec, n=P, axis=1).T  # (P, 64): phase-major, as the stage writes
    err = np.linalg.norm(D - ref) / np.linalg.norm(ref)
    assert err < 3e-7, err


def test_basis_image_layout_is_a_bijection():
    """Byte offsets of (phase row rr, K index j) in a tile's image: K-block
    j // 64, chunk (j % 64) // 8 swizzled with rr, element j % 8."""
    KB = 2
    seen = set()
    for rr in range(128):
        for j in range(64 * KB):
            kb, c, el = j // 64, (j % 64) // 8, j % 8
            off = kb * 16384 + sw128(rr, c) + 2 * el
            assert off not in seen
            seen.add(off)
    assert seen == set(range(0, 2 * 128 * 64 * KB, 2))


def test_b_tile_decoder_writes_cover_the_tile():
    """256 threads: channel quad c4 = tid % 16, rows tid // 16 + 16 i; each
    writes the 16-byte chunk (K-block c4 // 8, chunk c4 % 8) of its row."""
    offs = []
    for tid in range(256):
        c4 = tid % 16
        for r in range(tid // 16, 128, 16):
            offs.append((c4 // 8) * 16384 + sw128(r, c4 % 8))
    assert len(offs) == len(set(offs)) == 128 * 16
    assert set(offs) == set(range(0, 2 * 16384, 16))
