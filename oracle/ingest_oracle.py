"""CPU restatement of the reference's baseband file reading -- test
infrastructure only (used by tests/ as the checker, never by the product).

Follows albatros_analysis/src/correlations/baseband_data_classes.py:
  * Baseband.__init__ (:156-217): header fields, per-packet spectrum numbers
    read as big-endian uint32, one wrap inside a file undone by adding 2^32
    after the negative step;
  * BasebandFileIterator (:522-715): the file loader adds 2^32 per earlier
    file that wrapped (:594-603); the start is idxstart + the first file's
    first spectrum (:567); __next__ walks the acclen spectra of a chunk
    through gaps between files, files' spectrum ranges (rows by searchsorted,
    get_rows_from_specnum :493-519) and on to the next file when the chunk
    reaches past the current one's last spectrum.
Pinned against the reference's own classes run on the same files
(tests/golden/make_golden.py: ingest_cases).
"""
from __future__ import annotations

import struct
from typing import List, Sequence, Tuple

import numpy as np


def read_file(path: str):
    """(header tuple (header_bytes, bytes_per_packet, length_channels,
    spectra_per_packet, bit_mode, num_packets), channels, spec_num (int64,
    internal wrap undone), overflowed, payload (npkt, bytes_per_packet-4)), as
    Baseband reads a file (src/correlations/baseband_data_classes.py:156-228)."""
    with open(path, "rb") as f:
        blob = f.read()
    hb, bpp, lch, spp, bits, _ = struct.unpack(">6Q", blob[:48])
    nch = (hb - 80) // 8
    chans = np.frombuffer(blob[48:48 + 8 * nch], dtype=">u8").astype(np.int64)
    header_bytes = 8 + hb
    if bits == 1:
        chans, lch = np.ravel(np.column_stack((chans, chans + 1))), lch * 2
    elif bits == 4:
        chans, lch = chans[::2], lch // 2
    npkt = (len(blob) - header_bytes) // bpp
    body = np.frombuffer(blob[header_bytes:header_bytes + npkt * bpp], dtype=np.uint8).reshape(npkt, bpp)
    sn = body[:, :4].copy().view(">u4").reshape(-1).astype(np.int64)
    neg = np.flatnonzero(np.diff(sn) < 0)
    if len(neg) > 1:
        raise ValueError("two negative steps in the spectrum numbers")
    if len(neg) == 1:
        sn[neg[0] + 1:] += 1 << 32
    return (header_bytes, bpp, lch, spp, bits, npkt), chans, sn, len(neg) == 1, body[:, 4:]


def iterate(paths: Sequence[str], fileidx: int, idxstart: int, acclen: int, nchunks: int):
    """Per chunk (spectrum numbers present, file index, row in that file),
    rows counted in spectra (packet * spp + j), following
    BasebandFileIterator (src/correlations/baseband_data_classes.py:522-715).
    Like the reference, a chunk that reaches the last file's last spectrum
    ends the iteration undelivered."""
    files = []
    ctr = 0
    for p in paths:
        hdr, _, sn, over, _ = read_file(p)
        files.append((hdr[3], sn + ctr * (1 << 32)))
        ctr += int(over)
    fi = fileidx
    spp, sn = files[fi]
    idx = (sn[:, None] + np.arange(spp)[None, :]).ravel()
    pos = int(idxstart + idx[0])
    out: List[Tuple[np.ndarray, np.ndarray, np.ndarray]] = []
    for _ in range(nchunks):
        got_s, got_f, got_r = [], [], []
        rem = acclen
        while rem:
            if pos < idx[0]:  # gap before the current file
                step = min(int(idx[0]) - pos, rem)
                rem -= step
                pos += step
                continue
            span = int(idx[-1]) - pos + 1
            take = span if rem >= span else rem
            lo = np.searchsorted(idx, pos, side="left")
            hi = np.searchsorted(idx, pos + take, side="left")
            got_s.append(idx[lo:hi])
            got_f.append(np.full(hi - lo, fi))
            got_r.append(np.arange(lo, hi))
            rem -= take
            pos += take
            if take == span:  # reached the current file's last spectrum: open the next one
                fi += 1
                if fi == len(files):  # out of files: this chunk is not delivered (:677-678)
                    return out
                spp, sn = files[fi]
                idx = (sn[:, None] + np.arange(spp)[None, :]).ravel()
        out.append(tuple(np.concatenate(x) if x else np.zeros(0, np.int64) for x in (got_s, got_f, got_r)))
    return out
