"""The oracle pinned against the reference: golden outputs of the reference's
own C (unpacking.c, correlations_cpu.c) and CPU PFB code (pfb_cpu_utils.py),
generated by tests/golden/make_golden.py.  CPU only."""
import numpy as np
import pytest

from oracle import int_oracle as io
from oracle import pfb_oracle as po
from tests.golden import gen


def test_fixture_4bit_matches_reference_test_description(golden_int):
    e0, e1 = gen.fixture_4bit_expected()
    np.testing.assert_array_equal(golden_int["u4_fix_all_p0"], e0)
    np.testing.assert_array_equal(golden_int["u4_fix_all_p1"], e1)
    np.testing.assert_array_equal(golden_int["u4_fix_one_p0"], e0[:, 3:4])
    np.testing.assert_array_equal(golden_int["u4_fix_two_p1"], e1[:, [2, 5]])


@pytest.mark.parametrize("name", ["all", "one", "two"])
def test_oracle_unpack4_fixture(golden_int, name):
    raw = gen.fixture_4bit_packed().reshape(-1, 20)
    p0, p1 = io.unpack_4bit(raw, 0, 2, golden_int[f"u4_fix_{name}_ch"], 10)
    np.testing.assert_array_equal(p0, golden_int[f"u4_fix_{name}_p0"])
    np.testing.assert_array_equal(p1, golden_int[f"u4_fix_{name}_p1"])


def test_oracle_unpack4_random(golden_int):
    raw = gen.raw_4bit(seed=11, nspec=300, nchan=64)
    assert gen.checksum(raw) == str(golden_int["u4_rand_sum"])
    p0, p1 = io.unpack_4bit(raw, 7, 291, golden_int["u4_rand_ch"], 64)
    np.testing.assert_array_equal(p0, golden_int["u4_rand_p0"])
    np.testing.assert_array_equal(p1, golden_int["u4_rand_p1"])
    # independent NumPy decoder (the reference's test_against_jon idea)
    q0, q1 = po.unpack_4bit_np(raw, 7, 291, golden_int["u4_rand_ch"])
    np.testing.assert_array_equal(p0, q0)
    np.testing.assert_array_equal(p1, q1)


def test_nibble_8_decodes_plus_8():
    raw = np.array([[0x88, 0x8F]], np.uint8)
    p0, p1 = io.unpack_4bit(raw, 0, 1, [0], 1)
    assert p0[0, 0] == 8 + 8j and p1[0, 0] == 8 - 1j


def test_oracle_unpack1(golden_int):
    p0, p1 = io.unpack_1bit(gen.fixture_1bit_packed().reshape(-1, 4), 0, 2, 2, 6, 8)
    np.testing.assert_array_equal(p0, golden_int["u1_fix_p0"])
    np.testing.assert_array_equal(p1, golden_int["u1_fix_p1"])
    r0, i0, r1, i1 = gen.fixture_1bit_values()
    np.testing.assert_array_equal(p0, (r0 + 1j * i0)[:, 2:6])
    np.testing.assert_array_equal(p1, (r1 + 1j * i1)[:, 2:6])
    raw1 = gen.raw_1bit(seed=12, nspec=300, nchan=64)
    assert gen.checksum(raw1) == str(golden_int["u1_rand_sum"])
    p0, p1 = io.unpack_1bit(raw1, 3, 299, 6, 40, 64)
    np.testing.assert_array_equal(p0, golden_int["u1_rand_p0"])
    np.testing.assert_array_equal(p1, golden_int["u1_rand_p1"])


def test_oracle_sortpols(golden_int):
    p1raw = gen.fixture_1bit_packed().reshape(-1, 4)
    for c0, c1 in ((2, 7), (0, 8)):
        a, b = io.sortpols(p1raw, 8, 1, 0, 2, c0, c1)
        np.testing.assert_array_equal(a, golden_int[f"sp1_fix_{c0}_{c1}_p0"])
        np.testing.assert_array_equal(b, golden_int[f"sp1_fix_{c0}_{c1}_p1"])
    # bit patterns asserted by src/correlations/tests/test_1bit_unpack.py:81-94
    a, b = io.sortpols(p1raw, 8, 1, 0, 2, 2, 7)
    assert a[1, 0] == 0b01110101 and a[0, 0] == 0b10101010 and a[1, 1] == 0b01000000
    assert b[1, 0] == 0b10001010 and b[0, 0] == 0b01010101 and b[1, 1] == 0b10000000
    raw1 = gen.raw_1bit(seed=12, nspec=300, nchan=64)
    for c0, c1 in ((0, 64), (6, 31), (10, 12)):
        a, b = io.sortpols(raw1, 64, 1, 3, 299, c0, c1)
        np.testing.assert_array_equal(a, golden_int[f"sp1_rand_{c0}_{c1}_p0"])
        np.testing.assert_array_equal(b, golden_int[f"sp1_rand_{c0}_{c1}_p1"])
    raw = gen.raw_4bit(seed=11, nspec=300, nchan=64)
    a, b = io.sortpols(raw, 64, 4, 7, 291, 5, 45)
    np.testing.assert_array_equal(a, golden_int["sp4_rand_p0"])
    np.testing.assert_array_equal(b, golden_int["sp4_rand_p1"])


def test_oracle_xcorr_4bit(golden_int):
    d0, d1 = gen.sorted_4bit_pair(seed=21, nrows=2000, ncol=33)
    re, im = io.avg_xcorr_4bit_sums(d0, d1, 2000)
    np.testing.assert_array_equal(re, golden_int["x4_sum"].real.astype(np.int64))
    np.testing.assert_array_equal(im, golden_int["x4_sum"].imag.astype(np.int64))
    s0, s1 = gen.specnum_pair(seed=22, n=2000, span=2600)
    re, im, n = io.avg_xcorr_4bit_2ant_sums(d0, d1, s0, s1, 0, 0)
    assert n == int(golden_int["x4_2ant_rows"])
    np.testing.assert_array_equal(re, golden_int["x4_2ant_sum"].real.astype(np.int64))
    np.testing.assert_array_equal(im, golden_int["x4_2ant_sum"].imag.astype(np.int64))


def test_oracle_xcorr_1bit(golden_int):
    for nch in (32, 29):
        nb = int(np.ceil(nch / 4))
        e0, e1 = gen.sorted_1bit_pair(seed=23 + nch, nrows=1500, nbytes=nb)
        re, im = io.avg_xcorr_1bit_sums(e0, e1, nch, 1500)
        np.testing.assert_array_equal(re, golden_int[f"x1_{nch}_sum"].real.astype(np.int64))
        np.testing.assert_array_equal(im, golden_int[f"x1_{nch}_sum"].imag.astype(np.int64))
    e0, e1 = gen.sorted_1bit_pair(seed=31, nrows=2000, nbytes=8)
    s0, s1 = gen.specnum_pair(seed=22, n=2000, span=2600)
    out, n = io.vanvleck_2ant_sums(e0, e1, 32, s0, s1, 0, 0)
    assert n == int(golden_int["vv_2ant_rows"])
    np.testing.assert_array_equal(np.stack(out), golden_int["vv_2ant"].astype(np.int64))


def test_oracle_all_ant_matches_pairwise():
    """The all-baseline int64 oracle agrees with the pairwise one (same decode)."""
    raw = gen.raw_4bit_uniform(seed=3, nspec=200, nchan=16, nant=2)
    ch = np.array([1, 4, 9, 15])
    re, im = io.xcorr_all_ant_4bit(raw, 10, 190, ch, 16)
    for i in range(4):
        for j in range(4):
            a, p = divmod(i, 2)
            b, q = divmod(j, 2)
            d0 = raw[a, 10:190].reshape(180, 16, 2)[:, ch, p]
            d1 = raw[b, 10:190].reshape(180, 16, 2)[:, ch, q]
            r2, i2 = io.avg_xcorr_4bit_sums(d0, d1, 180)
            np.testing.assert_array_equal(re[i, j], r2)
            np.testing.assert_array_equal(im[i, j], i2)


def test_fp64_oracle_vs_reference_pfb_code(golden_pfb):
    """FP64 restatement vs the reference's own float32 CPU PFB module."""
    m = po.get_matft(12)
    rel = np.abs(golden_pfb["matft_12"] - m).max() / np.abs(m).max()
    assert rel < 1e-6
    f = po.calculate_filter(m, 0.45)
    dat = gen.ipfb_input(seed=41, nslice=12)
    assert gen.checksum(dat) == str(golden_pfb["ipfb_in_sum"])
    ref = golden_pfb["ipfb_12_cut2"]
    mine = po.ipfb(dat.astype(np.complex128), f)[2:-2].ravel()
    assert np.linalg.norm(ref - mine) / np.linalg.norm(mine) < 1e-6
    ts = gen.timestream(seed=42, n=4096 * 2 * 7)
    assert gen.checksum(ts) == str(golden_pfb["pfb_in_sum"])
    win = po.sinc_hamming(4, 8192).astype(np.float32).astype(np.float64)
    p = po.pfb(ts, win, nchan=4097)
    assert np.linalg.norm(golden_pfb["pfb_os2"] - p) / np.linalg.norm(p) < 1e-6


def test_fp64_ipfb_inverts_circular_pfb():
    """Property of the restated IPFB: with threshold 0 it exactly inverts a PFB
    whose input is periodic over nslice blocks (the IPFB's circular model)."""
    rng = np.random.default_rng(0)
    nslice = 64
    x = rng.standard_normal(nslice * 4096)
    xx = np.concatenate([x, x[:3 * 4096]])
    spec = po.pfb(xx, po.sinc_hamming(4, 4096), nchan=2049)  # (nslice, 2049)
    filt = po.calculate_filter(po.get_matft(nslice), 0.0)
    back = po.ipfb(spec, filt).ravel()
    assert np.linalg.norm(back - x) / np.linalg.norm(x) < 1e-8


HIST_CASES = [("h4_fix", 4, 10, (0, 2)), ("h4_rand", 4, 64, (7, 291)), ("h1_fix", 1, 8, (0, 2)),
              ("h1_rand", 1, 64, (3, 299))]


def hist_input(name):
    """Raw rows of the histogram fixtures (tests/golden/make_golden.py:hist_cases)."""
    return {"h4_fix": lambda: gen.fixture_4bit_packed().reshape(-1, 20),
            "h4_rand": lambda: gen.raw_4bit(seed=11, nspec=300, nchan=64),
            "h1_fix": lambda: gen.fixture_1bit_packed().reshape(-1, 4),
            "h1_rand": lambda: gen.raw_1bit(seed=12, nspec=300, nchan=64)}[name]()


@pytest.mark.parametrize("mode", [0, 1, -1])
@pytest.mark.parametrize("name,bits,nchan,rows", HIST_CASES)
def test_oracle_hist_golden(golden_int, name, bits, nchan, rows, mode):
    h = io.hist(hist_input(name), rows[0], rows[1], nchan, bits, mode)
    np.testing.assert_array_equal(h, golden_int[f"{name}_{'b' if mode == -1 else mode}"])
    # every selected level lands in exactly one bin
    assert int(h.sum()) == (rows[1] - rows[0]) * nchan * (4 if mode == -1 else 2)


def test_hist_reference_known_answers(golden_int):
    """The reference's own assertions (test_1bit_unpack.py:110-133,
    test_4bit_float_unpack.py:131-170) on the fixtures."""
    h = {m: golden_int[f"h1_fix_{m}"] for m in ("0", "1", "b")}
    assert (h["0"][0, 3], h["0"][1, 3], h["0"][0, 4]) == (1, 3, 2)
    assert (h["1"][0, 3], h["1"][1, 3], h["1"][0, 4]) == (3, 1, 2)
    assert (h["b"][0, 3], h["b"][1, 3], h["b"][0, 4]) == (4, 4, 4)
    h4 = {m: golden_int[f"h4_fix_{m}"] for m in ("0", "1", "b")}
    e0, e1 = gen.fixture_4bit_expected()
    r0, i0, r1, i1 = e0.real, e0.imag, e1.real, e1.imag
    assert h4["0"][0, 3] == 1 and h4["0"][4, 3] == 1
    assert h4["0"][0, :].sum() == np.sum(r0 == 0) + np.sum(i0 == 0)
    assert h4["1"][0, 3] == 1 and h4["1"][12, 3] == 1
    assert h4["1"][7, :].sum() == np.sum(r1 == 7) + np.sum(i1 == 7)
    assert h4["b"][12, 3] == 1 and h4["b"][4, 3] == 1
    assert h4["b"][0, :].sum() == sum(np.sum(a == 0) for a in (r0, i0, r1, i1))


@pytest.mark.parametrize("name", ["wrap", "gaps4", "gaps1"])
def test_oracle_file_iterator(golden_int, name, tmp_path):
    """Chunk spectrum numbers and the file rows serving them vs the
    reference's BasebandFileIterator on the same files; header fields and
    wrap-fixed spectrum numbers vs its Baseband."""
    from oracle import ingest_oracle as ig
    sc = gen.baseband_scenarios()[name]
    paths = gen.write_scenario(sc, str(tmp_path), name)
    for k, p in enumerate(paths):
        hdr, chans, sn, over, _ = ig.read_file(p)
        np.testing.assert_array_equal(hdr, golden_int[f"bb_{name}_{k}_hdr"])
        np.testing.assert_array_equal(chans, golden_int[f"bb_{name}_{k}_chans"])
        np.testing.assert_array_equal(sn, golden_int[f"bb_{name}_{k}_specnum"])
        assert over == bool(golden_int[f"bb_{name}_{k}_overflowed"])
    chunks = ig.iterate(paths, 0, sc["idxstart"], sc["acclen"], sc["nchunks"])
    np.testing.assert_array_equal([len(c[0]) for c in chunks], golden_int[f"bfi_{name}_counts"])
    for i, key in enumerate(("specnums", "files", "rows")):
        np.testing.assert_array_equal(np.concatenate([c[i] for c in chunks]), golden_int[f"bfi_{name}_{key}"])
