"""Baseband files -> device spectrum rows + spectrum map, and the file-driven
streaming run.

Reference: Baseband / get_header (albatros_analysis/src/correlations/
baseband_data_classes.py:100-217, :338-359), the spectrum-number wrap fixes
(:208-217 within a file, :594-603 across files), BasebandFileIterator
(:522-715) and the driver's repfb_xcorr_avg(idxs, files, ...)
(scripts/xcorr/helper_gpu_stream.py, helper_gpu_stream_clean.py:295-402).

The header and the per-packet spectrum numbers are read on the host (as the
reference keeps them there); each file's packet block goes to the device in
one copy from pinned memory, where ``ab_packets_to_rows`` splits it into
spectrum rows and ``ab_spec_map_add`` records, for every spectrum number of
the run, the row holding it.  The chain then reads gaps as zeros through that
map (no per-chunk host loop, no zero-filled full-band arrays).
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib, output
from .stream import StreamCorrelator

WRAP = 1 << 32


@dataclass
class BasebandHeader:
    """Header fields with the reference's names and bit-mode adjustment
    (1-bit: channel pairs (c, c+1), length doubled; 4-bit: every other entry,
    length halved; baseband_data_classes.py:179-185)."""
    header_bytes: int
    bytes_per_packet: int
    length_channels: int
    spectra_per_packet: int
    bit_mode: int
    have_trimble: int
    channels: np.ndarray
    gps_week: int
    gps_timestamp: int
    gps_latitude: float
    gps_longitude: float
    gps_elevation: float
    num_packets: int

    @property
    def row_bytes(self) -> int:
        return (self.bytes_per_packet - 4) // self.spectra_per_packet


def read_header(path: str) -> BasebandHeader:
    """Reference: src/correlations/baseband_data_classes.py:100-185 (Baseband header fields)."""
    with open(path, "rb") as f:
        head = f.read(48)
        if len(head) < 48:
            raise ValueError(f"{path}: truncated header")
        hb, bpp, lch, spp, bits, trimble = struct.unpack(">6Q", head)
        if hb < 80 or (hb - 80) % 8:
            raise ValueError(f"{path}: bad header size field {hb}")
        nch = (hb - 80) // 8
        chans = np.frombuffer(f.read(8 * nch), dtype=">u8").astype(np.int64)
        tail = f.read(40)
        if len(chans) != nch or len(tail) < 40:
            raise ValueError(f"{path}: truncated header")
        week, stamp = struct.unpack(">2Q", tail[:16])
        lat, lon, elev = struct.unpack(">3d", tail[16:])
        size = os.fstat(f.fileno()).st_size
    header_bytes = 8 + hb
    if bits == 1:
        chans = np.ravel(np.column_stack((chans, chans + 1)))
        lch = int(lch * 2)
    elif bits == 4:
        chans = chans[::2]
        lch = int(lch // 2)
    else:
        raise ValueError(f"{path}: bit_mode {bits} not supported (1 or 4)")
    if bpp <= 4 or spp <= 0 or (bpp - 4) % spp:
        raise ValueError(f"{path}: {bpp} bytes per packet do not hold {spp} spectra")
    return BasebandHeader(header_bytes, int(bpp), int(lch), int(spp), int(bits), int(trimble), chans, int(week),
                          int(stamp), lat, lon, elev, int((size - header_bytes) // bpp))


def get_header(path: str, verbose: bool = False) -> Dict:
    """The reference's get_header dictionary (header fields only).

    Reference: src/correlations/baseband_data_classes.py:344-365."""
    h = read_header(path)
    if verbose:
        print(h)
    d = {k: getattr(h, k) for k in h.__dataclass_fields__}
    return d


def fix_wraps(spec_num: np.ndarray) -> Tuple[np.ndarray, bool]:
    """Undo one uint32 wrap inside a file (baseband_data_classes.py:208-217):
    2^32 is added after the single negative step; more than one is an error."""
    s = np.asarray(spec_num, dtype=np.int64).copy()
    w = np.flatnonzero(np.diff(s) < 0)
    if len(w) > 1:
        raise ValueError("Why are there two -ve diffs in specnum? Investigate this file")
    if len(w) == 1:
        s[w[0] + 1:] += WRAP
    return s, len(w) == 1


def read_packets(path: str, readlen=-1, header: Optional[BasebandHeader] = None):
    """(header, pinned uint8 (npkt, bytes_per_packet) packets, wrap-fixed
    int64 spectrum numbers, overflowed).  readlen as the reference: >= 1
    packets, (0, 1) a fraction, 0 none, -1 all.

    Reference: src/correlations/baseband_data_classes.py:156-228 (packets, spectrum numbers, wrap fix)."""
    h = header or read_header(path)
    if readlen >= 1:
        npk = min(int(readlen), h.num_packets)
    elif 0 < readlen < 1:
        npk = int(h.num_packets * readlen)
    elif readlen == 0:
        npk = 0
    else:
        npk = h.num_packets
    buf = torch.empty((npk, h.bytes_per_packet), dtype=torch.uint8, pin_memory=torch.cuda.is_available())
    arr = buf.numpy()
    with open(path, "rb") as f:
        f.seek(h.header_bytes)
        got = f.readinto(memoryview(arr).cast("B")) if npk else 0
    if got != arr.nbytes:
        raise ValueError(f"{path}: short read ({got} of {arr.nbytes} bytes)")
    sn = np.ascontiguousarray(arr[:, :4]).view(">u4").reshape(-1).astype(np.int64)
    sn, over = fix_wraps(sn)
    return h, buf, sn, over


def first_specnum(path: str, header: Optional[BasebandHeader] = None) -> Optional[int]:
    """Spectrum number of a file's first packet (None when it has none), read
    without loading the file; an inside-file wrap never changes it."""
    h = header or read_header(path)
    if h.num_packets == 0:
        return None
    with open(path, "rb") as f:
        f.seek(h.header_bytes)
        return int(struct.unpack(">I", f.read(4))[0])


@dataclass
class AntennaFiles:
    """The files of one antenna that a run reads, with each file's rows in
    the antenna's row block and its spectrum numbers after both wrap fixes."""
    header: BasebandHeader
    start: int                                   # spectrum number of run row 0
    paths: List[str] = field(default_factory=list)
    row0: List[int] = field(default_factory=list)
    specnums: List[np.ndarray] = field(default_factory=list)
    packets: List[torch.Tensor] = field(default_factory=list)  # pinned host packets, released after upload
    npkt: List[int] = field(default_factory=list)

    @property
    def rows(self) -> int:
        return sum(self.npkt) * self.header.spectra_per_packet


def plan_antenna(paths: Sequence[str], fileidx: int, idxstart: int, nspec: int) -> AntennaFiles:
    """Read the files of one antenna from paths[fileidx] until nspec spectra
    from the start (idxstart + the first file's first spectrum number) are
    covered.  A file's spectrum numbers get 2^32 per earlier file that wrapped
    inside (the BasebandFileIterator's overflow counter, :594-603)."""
    ctr, af = 0, None
    for path in paths[fileidx:]:
        if af is not None:  # a file starting past the run is not read at all
            s0 = first_specnum(path)
            if s0 is not None and s0 + ctr * WRAP >= af.start + nspec:
                break
        h, pk, sn, over = read_packets(path)
        sn = sn + ctr * WRAP
        if over:
            ctr += 1
        if af is None:
            if len(sn) == 0:
                raise ValueError(f"{path}: no packets")
            af = AntennaFiles(h, int(idxstart + sn[0]))
        else:
            for k in ("bytes_per_packet", "spectra_per_packet", "bit_mode", "length_channels"):
                if getattr(h, k) != getattr(af.header, k):
                    raise ValueError(f"{path}: {k} differs from the first file of the antenna")
            if len(sn) and sn[0] >= af.start + nspec:
                break
        af.paths.append(path)
        af.row0.append(af.rows)
        af.specnums.append(sn)
        af.packets.append(pk)
        af.npkt.append(int(pk.shape[0]))
        if len(sn) and sn[-1] + h.spectra_per_packet >= af.start + nspec:
            break
    if af is None:
        raise ValueError("no files")
    return af


def ingest(files: Sequence[Sequence[str]], idxs: Sequence[int], nspec: int, device=None, fileidx: int = 0):
    """Device (raw, spec_map, antennas): raw (nant, rows, row_bytes) uint8 with
    each antenna's files' spectra back to back, spec_map (nant, nspec) int32
    (row of spectrum start_a + g, -1 when missing) for the streaming chain.

    Reference: the per-chunk host walk of BasebandFileIterator.__next__
    (src/correlations/baseband_data_classes.py:614-715)."""
    if len(files) != len(idxs) or not files:
        raise ValueError("one file list and one start index per antenna")
    dev = torch.device(device if device is not None else "cuda")
    ants = [plan_antenna(f, fileidx, int(i), int(nspec)) for f, i in zip(files, idxs)]
    h0 = ants[0].header
    for a in ants[1:]:
        if a.header.row_bytes != h0.row_bytes or a.header.bit_mode != h0.bit_mode:
            raise ValueError("antennas differ in packet format")
    nrows = max(a.rows for a in ants)
    raw = torch.zeros((len(ants), max(nrows, 1), h0.row_bytes), dtype=torch.uint8, device=dev)
    spec_map = torch.empty((len(ants), int(nspec)), dtype=torch.int32, device=dev)
    s = _lib.stream_ptr(raw)
    for k, a in enumerate(ants):
        m = spec_map[k]
        _lib.call("ab_spec_map_init", m.data_ptr(), m.numel(), s)
        for r0, sn, pk in zip(a.row0, a.specnums, a.packets):
            if pk.shape[0] == 0:
                continue
            body = pk.to(dev, non_blocking=True)  # the pinned buffer is held until this copy is done
            dst = raw[k, r0: r0 + pk.shape[0] * a.header.spectra_per_packet]
            _lib.call("ab_packets_to_rows", body.data_ptr(), pk.shape[0], pk.shape[1], dst.data_ptr(), s)
            dsn = torch.from_numpy(sn).to(dev, non_blocking=True)
            _lib.call("ab_spec_map_add", dsn.data_ptr(), len(sn), a.header.spectra_per_packet, r0, a.start,
                      m.data_ptr(), m.numel(), s)
        _lib.call("ab_spec_map_finish", m.data_ptr(), m.numel(), s)
        a.packets = []  # the uploads hold their pinned buffers until done; nothing else needs them
    return raw, spec_map, ants


def repfb_xcorr_avg(idxs: Sequence[int], files: Sequence[Sequence[str]], acclen: int, nchunks: int, nblock: int,
                    chanstart: int, chanend: int, osamp: int, cut: int = 10, filt_thresh: float = 0.45,
                    device=None):
    """The reference driver's file-level call (helper_gpu_stream.py /
    helper_gpu_stream_clean.py:295): antenna a reads files[a] from its first
    file, starting idxs[a] spectra after that file's first spectrum.  Returns
    (vis, missing_fraction, freqs): vis (M, M, nchan, njobs) complex64
    F-ordered and NaN-masked, missing_fraction (nant, njobs) in percent, freqs
    the fine channel numbers.  Channels are the first antenna's header
    channels with [chanstart, chanend) selected as column indices."""
    raw, spec_map, ants = ingest(files, idxs, int(acclen) * int(nchunks), device)
    h = ants[0].header
    sc = StreamCorrelator(len(ants), h.channels, chanstart, chanend, acclen, nchunks, nblock, osamp, cut, filt_thresh,
                          nchan_raw=h.length_channels, bits=h.bit_mode)
    try:
        for j in range(int(nchunks)):
            sc.push(raw, j, spec_map, final=(j == int(nchunks) - 1))
        v = sc.vis_device().permute(1, 2, 3, 0).cpu().numpy()
        freqs = np.arange(sc.q0, sc.q1)
    finally:
        sc.close()
    present = output.chunk_presence(spec_map, len(ants), int(nchunks), int(acclen))
    return output.mask_invalid(np.asfortranarray(v)), output.missing_fraction(present, acclen, nblock, osamp), freqs


class BasebandFileIterator:
    """Chunks of acclen spectra of one antenna's files, as the reference's
    iterator yields them (baseband_data_classes.py:522-715): {"pol0", "pol1",
    "specnums"} with the present spectra's rows first and zeros after, pols
    unpacked to complex64 (type "float") or separated bytes (type "packed",
    sortpols layout).  The rows come from the device ingest; each chunk is a
    gather of its present rows and one unpack launch."""

    def __init__(self, file_paths, fileidx, idxstart, acclen, nchunks=None, channels=None, chanstart=0, chanend=None,
                 type="packed", device=None):
        from .unpacking import sortpols, unpack_1bit, unpack_4bit  # noqa: F401
        self.acclen, self.nchunks, self.type = int(acclen), nchunks, type
        h0 = read_header(file_paths[fileidx])
        n = int(nchunks) * self.acclen if nchunks else sum(read_header(p).num_packets for p in file_paths[fileidx:]) * \
            h0.spectra_per_packet
        self.raw, self.spec_map, ants = ingest([file_paths], [idxstart], n, device, fileidx)
        self.header = ants[0].header
        self.spec_num_start = ants[0].start
        if channels is not None:
            self.channel_idxs = np.sort(np.asarray(channels, dtype=np.int64))
        else:
            end = self.header.length_channels if chanend is None else int(chanend)
            self.channel_idxs = np.arange(int(chanstart), end, dtype=np.int64)
        self.chanstart, self.chanend = int(self.channel_idxs[0]), int(self.channel_idxs[-1]) + 1
        if self.header.bit_mode == 1 and (self.chanstart % 2 or self.chanend % 2):
            raise ValueError("Start and end channel indices must be divisible by 2 in 1-bit mode.")
        self.chunksread = 0
        self.nspec = n

    def __iter__(self):
        return self

    def __next__(self):
        from .unpacking import sortpols, unpack_1bit, unpack_4bit
        k = self.chunksread
        if (self.nchunks and k == self.nchunks) or (k + 1) * self.acclen > self.nspec:
            raise StopIteration
        m = self.spec_map[0, k * self.acclen: (k + 1) * self.acclen]
        pres = torch.nonzero(m >= 0).flatten()
        rows = self.raw[0].index_select(0, m.index_select(0, pres).long()).contiguous()
        nr = rows.shape[0]
        specnums = self.spec_num_start + k * self.acclen + pres.cpu().numpy().astype(np.int64)
        h = self.header
        if self.type == "float":
            if h.bit_mode == 4:
                p0, p1 = unpack_4bit(rows, 0, nr, self.channel_idxs, h.length_channels)
            else:
                p0, p1 = unpack_1bit(rows, 0, nr, self.channel_idxs, h.length_channels)
            dtype, ncols = torch.complex64, len(self.channel_idxs)
        else:
            p0, p1 = sortpols(rows, h.length_channels, h.bit_mode, 0, nr, self.chanstart, self.chanend)
            dtype, ncols = torch.uint8, p0.shape[1]
        pol0 = torch.zeros((self.acclen, ncols), dtype=dtype, device=rows.device)
        pol1 = torch.zeros_like(pol0)
        pol0[:nr], pol1[:nr] = p0, p1
        self.chunksread += 1
        return {"pol0": pol0, "pol1": pol1, "specnums": specnums}
