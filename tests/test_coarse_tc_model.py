"""CPU model of the tensor-core (tcgen05) coarse correlator's producer side
(csrc/xcorr_tc.cu): the nibble decode by integer tricks, the 16-byte rows it
writes into the 128-byte swizzled K-major tiles, and the time-slice plan.

A producer thread loads 8 consecutive samples of one antenna (16 bytes each:
8 channels x 2 pols), adds 7 to every nibble modulo 16 without carries,
gathers byte b of samples t and t+1 into one word (byte permute), turns the
nibbles into fp16 pairs (0x6400 | n is 1024 + n; minus 1031) and writes row
(channel half, antenna, pol, re|im) as 8 fp16 samples at chunk kc of the
row.  Checked here: the decoded levels equal the oracle's unpack (0x8 -> +8),
every (row, chunk) of a tile is written once, the 8 lanes of each 16-byte
store phase hit 8 distinct bank quads, and the slices cover every sample of
every chunk once with at most 2^17 samples a CTA (fp32 sums exact)."""
import numpy as np

from oracle import pfb_oracle as po


def nib_plus7(w):
    w = np.asarray(w, dtype=np.uint64)
    return (((w & 0x77777777) + 0x77777777) ^ (w & 0x88888888)) & 0xFFFFFFFF


def byte_perm(x, y, s):
    """__byte_perm: byte k of the result is byte (s >> 4k) & 7 of the 8 bytes y:x."""
    src = [(int(x) >> (8 * i)) & 255 for i in range(4)] + [(int(y) >> (8 * i)) & 255 for i in range(4)]
    return sum(src[(s >> (4 * k)) & 7] << (8 * k) for k in range(4))


def nib_to_h2(n2):
    """Two fp16 values (low half, high half): (0x6400 | n) - 1031 for the 4-bit n of each half."""
    x = (int(n2) & 0x000F000F) | 0x64006400
    lo = np.frombuffer(np.uint16(x & 0xFFFF).tobytes(), np.float16)[0]
    hi = np.frombuffer(np.uint16(x >> 16).tobytes(), np.float16)[0]
    return float(np.float16(lo - np.float16(1031))), float(np.float16(hi - np.float16(1031)))


def producer_rows(bytes8x16, cpt=2, ant=3):
    """(row -> 8 decoded samples) written by one thread for one antenna, as
    the kernel computes them from its 8 x 16 loaded bytes."""
    bpt = bytes8x16.shape[1]
    rows_per_ch = 128 // cpt
    w = [[nib_plus7(int.from_bytes(bytes8x16[i, 4 * q:4 * q + 4].tobytes(), "little")) for q in range(bpt // 4)]
         for i in range(8)]
    out = {}
    for b in range(bpt):
        j, pol = b >> 1, b & 1
        tile, h = j // cpt, j % cpt
        row_re = h * rows_per_ch + 4 * ant + 2 * pol
        sel = (b & 3) * 0x1111 + 0x4400
        re, im = [], []
        for m in range(4):
            p = byte_perm(int(w[2 * m][b >> 2]), int(w[2 * m + 1][b >> 2]), sel)
            im += nib_to_h2(p)
            re += nib_to_h2(p >> 4)
        out[(tile, row_re)] = re
        out[(tile, row_re + 1)] = im
    return out


def test_nibble_plus7_has_no_carries():
    rng = np.random.default_rng(0)
    for w in rng.integers(0, 2 ** 32, 2000, dtype=np.uint64):
        r = int(nib_plus7(w))
        for k in range(8):
            assert (r >> (4 * k)) & 15 == (((int(w) >> (4 * k)) & 15) + 7) & 15


def test_producer_decode_matches_oracle_unpack():
    rng = np.random.default_rng(1)
    for cpt in (2, 1):
        bpt = 8 * cpt * 2  # 4*cpt channels x 2 pols
        b = rng.integers(0, 256, (8, bpt), dtype=np.uint8)
        b[0, :] = 0x88  # +8 + 8j everywhere in one sample
        b[1, :] = 0x00
        rows = producer_rows(b, cpt=cpt, ant=3)
        nch = bpt // 2
        for j in range(nch):
            for pol in range(2):
                re, im = po.decode_4bit(b[:, 2 * j + pol])
                tile, h = j // cpt, j % cpt
                r = h * (128 // cpt) + 4 * 3 + 2 * pol
                assert rows[(tile, r)] == list(re.astype(float)), (cpt, j, pol)
                assert rows[(tile, r + 1)] == list(im.astype(float)), (cpt, j, pol)


def sw128_offset(row, c):
    return row * 128 + (((c ^ row) & 7) << 4)


def test_swizzled_tile_writes_are_a_bijection():
    offs = {sw128_offset(r, c) for r in range(128) for c in range(8)}
    assert offs == set(range(0, 128 * 128, 16))


def test_store_phases_are_bank_conflict_free():
    """A warp holds threads pt = 32w' + lane, lane -> (antenna pt >> 3, chunk
    kc = pt & 7); each 16-byte store instruction (fixed byte b and re|im) runs
    in 4 phases of 8 lanes, which must cover 8 distinct 16-byte bank quads."""
    for cpt in (2, 1):
        na = 128 // cpt // 4
        for wp in range(4):
            for b in range(8 * cpt * 2):
                j, pol = b >> 1, b & 1
                h = j % cpt
                for ri in range(2):
                    for phase in range(4):
                        quads = set()
                        for lane in range(8 * phase, 8 * phase + 8):
                            pt = 32 * wp + lane
                            ant, kc = (pt >> 3) % na, pt & 7
                            row = h * (128 // cpt) + 4 * ant + 2 * pol + ri
                            quads.add((sw128_offset(row, kc) // 16) % 8)
                        assert len(quads) == 8


def slice_plan(nrows, chunk_rows, ncols, nant, num_sms=152, kt=64, max_slice=1 << 17):
    """The launcher's slice choice (launch_coarse_tc in csrc/xcorr_tc.cu)."""
    cpc = 4 * (2 if nant <= 16 else 1)
    groups = -(-ncols // cpc)
    nchunks = -(-nrows // chunk_rows)
    per = max(1, -(-(4 * num_sms) // (groups * nchunks)))
    sl = -(-chunk_rows // per)
    sl = min(max(-(-sl // kt) * kt, kt), max_slice)
    spc = -(-chunk_rows // sl)
    return sl, spc, groups, nchunks


def test_slices_cover_each_chunk_once():
    for nrows, chunk, ncols, nant in [(1 << 18, 1 << 18, 256, 16), (1 << 17, 1 << 14, 64, 2), (3000, 1024, 6, 4),
                                      (333, 100, 5, 1), (1 << 20, 1 << 20, 8, 32), (2048, 2048, 256, 16)]:
        sl, spc, groups, nchunks = slice_plan(nrows, chunk, ncols, nant)
        assert sl % 64 == 0 and sl <= 1 << 17 and nchunks * spc <= 65535
        for c in range(nchunks):
            end = min((c + 1) * chunk, nrows)
            cover = np.zeros(end - c * chunk, np.int64)
            for s in range(spc):
                lo = c * chunk + s * sl
                hi = min(lo + sl, end)
                if hi > lo:
                    cover[lo - c * chunk:hi - c * chunk] += 1
            assert np.all(cover == 1)


# ---------------------------------------------------------------------------
# The TMA form (coarse_xcorr_tc_tma_kernel): scaled decode and barrier protocol.

def scaled_pair(p, hi):
    """16 (n - 7) for the nibbles of bytes 0 and 2 of p: low nibbles under
    0x7400 (16384 + 16 n), high nibbles in place under 0x6400 (1024 + 16 n)."""
    if hi:
        x, c = (int(p) & 0x00F000F0) | 0x64006400, 0x6470
    else:
        x, c = (int(p) & 0x000F000F) | 0x74007400, 0x7407
    cf = np.frombuffer(np.uint16(c).tobytes(), np.float16)[0]
    out = []
    for half in (x & 0xFFFF, x >> 16):
        v = np.frombuffer(np.uint16(half).tobytes(), np.float16)[0]
        out.append(float(np.float16(v - cf)))
    return out


def test_scaled_decode_is_16_times_the_level():
    """Every byte value: both scaled fp16 conversions give exactly 16 x the
    oracle's level (0x8 -> +8), and the largest product sums of a CTA slice
    (2^17 samples of 128 x 128) stay multiples of 256 below 2^32 (exact in
    fp32, whose 24-bit significand then spans 2^8 .. 2^32)."""
    lv_re, lv_im = po.decode_4bit(np.arange(256, dtype=np.uint8))
    for v in range(256):
        w = nib_plus7(v | (v << 16))
        assert scaled_pair(w, True) == [16.0 * float(lv_re[v])] * 2
        assert scaled_pair(w, False) == [16.0 * float(lv_im[v])] * 2
    assert (1 << 17) * 128 * 128 <= 2 ** 31 < 2 ** 32


class _Bar:
    """mbarrier: arrival count, phase counter, parity wait."""

    def __init__(self, count):
        self.count, self.pending, self.phase = count, count, 0

    def arrive(self):
        self.pending -= 1
        if self.pending == 0:
            self.phase, self.pending = self.phase + 1, self.count

    def passed(self, parity):  # the phase with this parity has completed
        return (self.phase & 1) != parity


def _run_protocol(nop, nrg, nst, seed, per_slot=False, fence=True):
    """One CTA of the TMA form under a random interleaving: two decoder groups
    (stages g, g + 2, ...), the MMA thread, the TMA thread; MMAs complete in
    order, their completion arrivals reach the barriers after independent
    random delays, and a box may land before its slot's reads unless the
    readers fence.  Returns the first violation, or None."""
    rnd = np.random.default_rng(seed)
    nv = nop if (nop % 2 == 0 or per_slot) else 2 * nop
    G = 3  # threads a group (model)
    full, empty = [_Bar(G) for _ in range(nv)], [_Bar(1) for _ in range(nv)]
    rfull, rempty = [_Bar(1) for _ in range(nrg)], [_Bar(G) for _ in range(nrg)]
    held = [None] * nop          # stage whose operands a physical slot holds
    ring = [None] * nrg          # stage whose box a packet slot holds
    unread = {}                  # packet slot -> readers that released it without a fence
    done, arrivals, queue = set(), [], []
    dec = {(g, t): [g, 0] for g in range(2) for t in range(G)}
    mma_s = tma_s = 0
    for _ in range(100000):
        acts = [("dec", k) for k, (s, _) in dec.items() if s < nst]
        acts += [("mma",)] * (mma_s < nst) + [("tma",)] * (tma_s < nst)
        acts += [("complete",)] * bool(queue) + [("deliver",)] * bool(arrivals)
        if not acts:
            return None
        a = acts[rnd.integers(len(acts))]
        if a[0] == "deliver":
            arrivals.pop(rnd.integers(len(arrivals))).arrive()
        elif a[0] == "complete":
            s = queue.pop(0)
            done.add(s)
            arrivals.append(empty[s % nv])
        elif a[0] == "tma":
            s, r = tma_s, tma_s % nrg
            if s >= nrg and not rempty[r].passed(((s // nrg) - 1) & 1):
                continue
            if unread.get(r):
                return "box landed before a read"
            ring[r] = s
            rfull[r].arrive()
            tma_s += 1
        elif a[0] == "mma":
            s = mma_s
            if not full[s % nv].passed((s // nv) & 1):
                continue
            if held[s % nop] != s:
                return "MMA read another stage's operands"
            queue.append(s)
            mma_s += 1
        else:
            k = a[1]
            s, st = dec[k]
            r = s % nrg
            if st == 0:  # read the box, release the slot
                if not rfull[r].passed((s // nrg) & 1):
                    continue
                if ring[r] != s:
                    return "read another stage's box"
                if not fence:
                    unread[r] = unread.get(r, 0) + 1  # the read may still be in flight
                rempty[r].arrive()
                dec[k][1] = 1
            else:  # write the operand slot
                if not fence:
                    unread[r] -= 1
                sp = s - nop
                v, ph = (s % nop, s // nop - 1) if per_slot else (sp % nv, sp // nv)
                if sp >= 0 and not empty[v].passed(ph & 1):
                    continue
                if sp >= 0 and sp not in done:
                    return "operands overwritten before their MMA completed"
                held[s % nop] = s
                full[s % nv].arrive()
                dec[k] = [s + 2, 0]
    return "stalled"


def test_tma_form_barrier_protocol():
    """The kernel's protocol (operand barriers per stage mod lcm(2, stages),
    one packet slot per box, fence before releasing a slot) is correct in
    every interleaving tried, for the shipped two operand stages with four
    packet slots and for three stages with two; per-physical-slot operand
    barriers with three stages, or releasing packet slots without the fence,
    are not."""
    for nop, nrg in ((2, 4), (3, 2), (2, 2)):
        for seed in range(60):
            assert _run_protocol(nop, nrg, 24, seed) is None, (nop, nrg, seed)
    assert any(_run_protocol(3, 2, 24, seed, per_slot=True) for seed in range(60))
    assert any(_run_protocol(2, 4, 24, seed, fence=False) for seed in range(60))
