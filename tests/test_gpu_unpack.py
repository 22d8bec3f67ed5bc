"""GPU parity: unpack / sortpols / make_continuous vs the reference's golden
outputs and the C oracle, bit-exact."""
import numpy as np
import pytest
import torch

from oracle import int_oracle as io
from oracle import pfb_oracle as po
from tests.golden import gen

pytestmark = pytest.mark.gpu


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", ["all", "one", "two"])
def test_unpack4_golden_fixture(golden_int, name):
    from albatros_axion_detection_gb300.unpacking import unpack_4bit
    p0, p1 = unpack_4bit(cu(gen.fixture_4bit_packed()), 0, 2, golden_int[f"u4_fix_{name}_ch"], 10)
    np.testing.assert_array_equal(p0.cpu().numpy(), golden_int[f"u4_fix_{name}_p0"])
    np.testing.assert_array_equal(p1.cpu().numpy(), golden_int[f"u4_fix_{name}_p1"])


def test_unpack4_golden_random(golden_int):
    from albatros_axion_detection_gb300.unpacking import unpack_4bit
    raw = gen.raw_4bit(seed=11, nspec=300, nchan=64)
    p0, p1 = unpack_4bit(cu(raw), 7, 291, golden_int["u4_rand_ch"], 64)
    np.testing.assert_array_equal(p0.cpu().numpy(), golden_int["u4_rand_p0"])
    np.testing.assert_array_equal(p1.cpu().numpy(), golden_int["u4_rand_p1"])


@pytest.mark.parametrize("channels", [np.arange(0, 64), np.arange(8, 40), np.array([63, 0, 7, 7, 31]), np.arange(3, 4)])
def test_unpack4_all_nibbles(channels):
    """Uniform bytes cover every nibble, 0x8 included; contiguous (vector) and
    gathered channel paths."""
    from albatros_axion_detection_gb300.unpacking import unpack_4bit
    raw = gen.raw_4bit_uniform(seed=5, nspec=1000, nchan=64)
    p0, p1 = unpack_4bit(cu(raw), 3, 997, channels, 64)
    e0, e1 = io.unpack_4bit(raw, 3, 997, channels, 64)
    np.testing.assert_array_equal(p0.cpu().numpy(), e0)
    np.testing.assert_array_equal(p1.cpu().numpy(), e1)


def test_unpack4_edge_cases():
    from albatros_axion_detection_gb300.unpacking import unpack_4bit
    raw = cu(gen.raw_4bit_uniform(seed=6, nspec=10, nchan=8))
    p0, p1 = unpack_4bit(raw, 4, 4, np.arange(8), 8)
    assert p0.shape == (0, 8)
    p0, _ = unpack_4bit(raw, 0, 10, np.array([], np.int64), 8)
    assert p0.shape == (10, 0)
    with pytest.raises(ValueError):
        unpack_4bit(raw, 0, 11, np.arange(8), 8)
    with pytest.raises(ValueError):
        unpack_4bit(raw, 0, 10, np.array([8]), 8)
    with pytest.raises(TypeError):
        unpack_4bit(raw.cpu().numpy(), 0, 10, np.arange(8), 8)


def test_unpack1_golden(golden_int):
    from albatros_axion_detection_gb300.unpacking import unpack_1bit
    p0, p1 = unpack_1bit(cu(gen.fixture_1bit_packed()), 0, 2, np.arange(2, 6), 8)
    np.testing.assert_array_equal(p0.cpu().numpy(), golden_int["u1_fix_p0"])
    np.testing.assert_array_equal(p1.cpu().numpy(), golden_int["u1_fix_p1"])
    # the reference GPU test's single-row case (test_1bit_unpack_gpu.py:86-99)
    q0, q1 = unpack_1bit(cu(gen.fixture_1bit_packed()), 1, 2, np.arange(2, 4), 8)
    assert q0[0, 1].item() == 1 + 1j and q1[0, 1].item() == -1 - 1j
    raw1 = gen.raw_1bit(seed=12, nspec=300, nchan=64)
    p0, p1 = unpack_1bit(cu(raw1), 3, 299, np.arange(6, 40), 64)
    np.testing.assert_array_equal(p0.cpu().numpy(), golden_int["u1_rand_p0"])
    np.testing.assert_array_equal(p1.cpu().numpy(), golden_int["u1_rand_p1"])


def test_sortpols_golden(golden_int):
    from albatros_axion_detection_gb300.unpacking import sortpols
    for c0, c1 in ((2, 7), (0, 8)):
        a, b = sortpols(cu(gen.fixture_1bit_packed()), 8, 1, 0, 2, c0, c1)
        np.testing.assert_array_equal(a.cpu().numpy(), golden_int[f"sp1_fix_{c0}_{c1}_p0"])
        np.testing.assert_array_equal(b.cpu().numpy(), golden_int[f"sp1_fix_{c0}_{c1}_p1"])
    raw1 = cu(gen.raw_1bit(seed=12, nspec=300, nchan=64))
    for c0, c1 in ((0, 64), (6, 31), (10, 12)):
        a, b = sortpols(raw1, 64, 1, 3, 299, c0, c1)
        np.testing.assert_array_equal(a.cpu().numpy(), golden_int[f"sp1_rand_{c0}_{c1}_p0"])
        np.testing.assert_array_equal(b.cpu().numpy(), golden_int[f"sp1_rand_{c0}_{c1}_p1"])
    a, b = sortpols(cu(gen.raw_4bit(seed=11, nspec=300, nchan=64)), 64, 4, 7, 291, 5, 45)
    np.testing.assert_array_equal(a.cpu().numpy(), golden_int["sp4_rand_p0"])
    np.testing.assert_array_equal(b.cpu().numpy(), golden_int["sp4_rand_p1"])


def test_make_continuous():
    from albatros_axion_detection_gb300.baseband_data_classes import make_continuous_gpu
    rng = np.random.default_rng(2)
    spec = (rng.standard_normal((50, 6)) + 1j * rng.standard_normal((50, 6))).astype(np.complex64)
    # distinct rows modulo nspec: colliding rows are a write race in the reference too
    specnum = np.sort(rng.choice(np.arange(1000, 1064), 50, replace=False)) + 64 * 3
    channels = np.array([3, 10, 11, 12, 400, 2048])
    out = make_continuous_gpu(cu(spec), specnum, 1000, channels, 64, nchans=2049)
    exp = po.make_continuous(spec, specnum, 1000, channels, 64, 2049)
    np.testing.assert_array_equal(out.cpu().numpy(), exp.astype(np.complex64))
    full = cu(spec[:, :1])
    same = make_continuous_gpu(full, np.arange(50), 0, [0], 50, nchans=1)
    assert same.data_ptr() == full.data_ptr()


@pytest.mark.parametrize("mode", [0, 1, -1])
@pytest.mark.parametrize("name,bits,nchan,rows", [("h4_fix", 4, 10, (0, 2)), ("h4_rand", 4, 64, (7, 291)),
                                                  ("h1_fix", 1, 8, (0, 2)), ("h1_rand", 1, 64, (3, 299))])
def test_hist_golden(golden_int, name, bits, nchan, rows, mode):
    from albatros_axion_detection_gb300.unpacking import hist
    from tests.test_oracle_golden import hist_input
    h = hist(cu(hist_input(name)), rows[0], rows[1], nchan, bits, mode)
    assert h.dtype == torch.uint64 and h.shape == (2 ** bits, nchan)
    np.testing.assert_array_equal(h.cpu().numpy(), golden_int[f"{name}_{'b' if mode == -1 else mode}"])


@pytest.mark.parametrize("bits,nchan,nspec,r0,r1", [(4, 300, 70001, 13, 69990), (4, 2048, 4096, 0, 4096),
                                                    (4, 3, 5000, 1, 4999), (1, 130, 90001, 5, 90000),
                                                    (1, 2048, 3000, 0, 3000), (1, 2, 700, 0, 1)])
def test_hist_vs_oracle(bits, nchan, nspec, r0, r1):
    """Many CTAs over rows and channel tiles, ragged tile and row edges."""
    from albatros_axion_detection_gb300.unpacking import hist
    raw = gen.raw_4bit_uniform(seed=nchan, nspec=nspec, nchan=nchan) if bits == 4 else \
        gen.raw_1bit(seed=nchan, nspec=nspec, nchan=nchan)
    d = cu(raw)
    for mode in (0, 1, -1):
        np.testing.assert_array_equal(hist(d, r0, r1, nchan, bits, mode).cpu().numpy(),
                                      io.hist(raw, r0, r1, nchan, bits, mode))


def test_hist_edge_cases():
    from albatros_axion_detection_gb300.unpacking import hist
    d = cu(gen.raw_4bit_uniform(seed=3, nspec=10, nchan=8))
    assert not hist(d, 4, 4, 8, 4, -1).cpu().numpy().any()  # empty row range: zeros
    for bad in (dict(bit_depth=2, mode=0), dict(bit_depth=4, mode=2)):
        with pytest.raises(ValueError):
            hist(d, 0, 10, 8, **bad)
    with pytest.raises(ValueError):
        hist(d, 0, 11, 8, 4, 0)  # past the end of the data
    with pytest.raises(ValueError):
        hist(cu(gen.raw_1bit(seed=1, nspec=4, nchan=8)), 0, 4, 7, 1, 0)  # odd 1-bit channel count


@pytest.mark.parametrize("bits", [4, 1])
def test_unpack_int8_complex_equals_float(bits):
    """The int8-complex outputs hold exactly the complex64 decodes' levels."""
    from albatros_axion_detection_gb300.unpacking import unpack_1bit, unpack_4bit
    if bits == 4:
        raw = cu(gen.raw_4bit_uniform(seed=8, nspec=777, nchan=40))
        ch, fn = np.array([0, 3, 4, 17, 39, 21]), unpack_4bit
    else:
        raw = cu(gen.raw_1bit(seed=8, nspec=777, nchan=40))
        ch, fn = np.arange(6, 30), unpack_1bit
    f0, f1 = fn(raw, 5, 770, ch, 40)
    i0, i1 = fn(raw, 5, 770, ch, 40, dtype=torch.int8)
    assert i0.dtype == torch.int8 and i0.shape == (765, len(ch), 2)
    for f, i in ((f0, i0), (f1, i1)):
        assert torch.equal(torch.view_as_real(f), i.float())
    e0, _ = fn(raw, 3, 3, ch, 40, dtype=torch.int8)
    assert e0.shape == (0, len(ch), 2)
    with pytest.raises(ValueError):
        fn(raw, 0, 4, ch, 40, dtype=torch.float16)
