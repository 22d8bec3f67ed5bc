"""Autotuner for the chain's time stage: IIR / FIR row tile, or FFT radix order.

The IPFB time-axis deconvolution has three forms in the library.  The IIR and
FIR forms (the default wherever the reference's Wiener filter decays fast
enough; IIR first) have one tunable tile: the kept rows per thread (16, 32 or,
for the IIR form, 64), which sets the rows a CTA filters and how many CTAs
share an SM.  The FFT form runs one real FFT of
nslice = acclen + 2*cut points per coarse sample phase (a complex FFT of
n = nslice/2 points) and its inverse; two lengths have compile-time plans
(n = 16464 for acclen 2^15, cut 80, and n = 16384), every other length runs
the runtime mixed-radix plan whose radix order decides how many shared-memory
passes and twiddle loads it makes.  The reference delegates all of this to
cuFFT's planner (albatros_analysis/src/utils/pycufft.cu:201-303).  Here each
candidate (FIR tiles, the FFT's built-in plan, and the orderings of n's
factorisation over the radices the kernels carry: 8, 4, 2, 7, 5, 3) is timed
on the streaming chain's own time stage, and the fastest is installed in the
library context (``ab_ctx_set_time_filter``, ``ab_ctx_set_fft_plan``).

Results are cached per device name and configuration in a JSON file
(``$ALBATROS_GB300_TUNE_CACHE``, default ``~/.cache/albatros_gb300/autotune.json``).
"""
from __future__ import annotations

import ctypes
import itertools
import json
import os
import threading
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib

BUILTIN = "builtin"          # the library's own plan (compile-time where one exists)
STATIC_LENGTHS = (16464, 16384)
_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("ALBATROS_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "albatros_gb300", "autotune.json"))


def _load_cache() -> Dict[str, object]:
    try:
        with open(cache_path()) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _save_cache(d: Dict[str, object]) -> None:
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home only loses the cache


def factorise(n: int) -> Optional[Dict[int, int]]:
    """Exponents of 2, 3, 5, 7 in n (None if n has another prime factor)."""
    e = {}
    for p in (2, 3, 5, 7):
        k = 0
        while n % p == 0:
            n //= p
            k += 1
        e[p] = k
    return e if n == 1 else None


def _pow2_splits(k: int) -> List[Tuple[int, ...]]:
    """Ways to write 2^k as radices 8/4/2, with at most one 4 and one 2
    beyond the 8s (more small radices only add passes)."""
    out = []
    for n8 in range(k // 3, -1, -1):
        r = k - 3 * n8
        for n4 in range(r // 2, -1, -1):
            n2 = r - 2 * n4
            if n4 + n2 <= 2:
                out.append((8,) * n8 + (4,) * n4 + (2,) * n2)
    return out


def candidate_orders(n: int, limit: int = 40) -> List[Tuple[int, ...]]:
    """Distinct radix orders of n, fewest passes first; at most `limit`."""
    e = factorise(n)
    if e is None or n < 2:
        return []
    odd = (3,) * e[3] + (5,) * e[5] + (7,) * e[7]
    seen, cands = set(), []
    for p2 in _pow2_splits(e[2]):
        ms = tuple(sorted(p2 + odd, reverse=True))
        if len(ms) > 12:
            continue
        for perm in itertools.permutations(ms):
            if perm not in seen:
                seen.add(perm)
                cands.append(perm)
    cands.sort(key=lambda r: (len(r), [-x for x in r]))
    # keep every order with the fewest passes first, then the rest
    return cands[:limit]


def set_plan(n: int, radices: Optional[Sequence[int]], device: Optional[int] = None) -> None:
    """Install (or clear, with None) the radix order for length n."""
    c = _lib.ctx(device)
    if radices is None:
        _lib.call("ab_ctx_set_fft_plan", c, int(n), None, 0)
        return
    arr = (ctypes.c_int32 * len(radices))(*[int(r) for r in radices])
    _lib.call("ab_ctx_set_fft_plan", c, int(n), ctypes.cast(arr, ctypes.c_void_p), len(radices))


DEFAULT_MODE = 0
DEFAULT_ROW_TILE = 16  # rows-per-thread class of the IIR / FIR time stage (21 / 17 rows)
_filter_setting = {"mode": DEFAULT_MODE, "row_tile": DEFAULT_ROW_TILE}


def set_time_filter(mode: int = DEFAULT_MODE, row_tile: int = 0, device: Optional[int] = None) -> None:
    """Time stage of streams created from now on: mode 0 = IIR where the
    filter factors and decays fast enough, else FIR where it is accurate,
    else FFT (the default); 1 = FFT only; 2 = FFT where its length factors,
    else IIR or FIR; 3 = FIR, else FFT.  row_tile 16/32/64 (0 keeps it)."""
    _lib.call("ab_ctx_set_time_filter", _lib.ctx(device), int(mode), int(row_tile))
    _filter_setting["mode"] = int(mode)
    if row_tile:
        _filter_setting["row_tile"] = int(row_tile)


# ab_ctx_set_option keys (AB_OPT_* in include/albatros_gb300.h)
OPT_ROW_FFTS_PER_CTA = 1
OPT_COARSE_MMA_BITS = 3
OPT_ROW_PREFETCH = 5
OPT_COARSE_ENGINE = 6
OPT_COARSE_TC_SLICE = 7
OPT_PFB_TMA = 9
OPT_FAULT_TEST = 10
OPT_COARSE_TC_TMA = 11
OPT_ROW_TC = 12
DEFAULT_ROW_PREFETCH = 2


def set_coarse_mma_bits(bits: int, device: Optional[int] = None) -> None:
    """Operand type of the coarse correlator's tensor-core MMA: 16 (fp16,
    exact, the default) or 8 (int8)."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_COARSE_MMA_BITS, int(bits))


def set_coarse_engine(engine: int, device: Optional[int] = None) -> None:
    """Tensor-core path of the fp16 coarse correlator: 0 (default) tcgen05
    from 9 antennas up and warp-level mma.sync below, 1 always mma.sync, 2
    tcgen05 for any antenna count up to 32."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_COARSE_ENGINE, int(engine))


def set_coarse_tc_slice(samples: int, device: Optional[int] = None) -> None:
    """Time samples one CTA of the tcgen05 coarse correlator sums (0: chosen
    per call; else a multiple of 64 up to 131072)."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_COARSE_TC_SLICE, int(samples))


def set_coarse_tc_tma(on: int, device: Optional[int] = None) -> None:
    """tcgen05 coarse correlator: packet bytes staged by TMA into a ring in
    shared memory (1, default) or loaded into registers (0); both exact."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_COARSE_TC_TMA, int(on))


def set_row_tc(on: int, device: Optional[int] = None) -> None:
    """Streaming row stage (inverse real FFT of every spectrum) of streams
    created from now on: a matrix product on the tcgen05 tensor cores (1,
    default; 4-bit or 1-bit packets, at most 64 channels) or the FFT (0)."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_ROW_TC, int(on))


def set_pfb_tma(on: int, device: Optional[int] = None) -> None:
    """Streaming PFB band DFT: plain loads (0, default), W tiles staged by
    TMA into each CTA's FFT buffers (1), or persistent CTAs fetching the next
    tile with TMA (2); the same arithmetic."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_PFB_TMA, int(on))


def set_row_prefetch(mode, device: Optional[int] = None) -> None:
    """Time-paired row stage: 2 (default) persistent CTAs with cp.async
    prefetch and the FFT twiddles in shared memory, 1 the same with the
    twiddles read from global memory, 0 one CTA per tile."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_ROW_PREFETCH, int(mode))


def set_row_ffts_per_cta(n: int, device: Optional[int] = None) -> None:
    """Spectra per CTA of the streaming row stage: 8 (time-paired, the
    default), 4 or 2 (pol-paired)."""
    _lib.call("ab_ctx_set_option", _lib.ctx(device), OPT_ROW_FFTS_PER_CTA, int(n))


def _time_chain(acclen: int, cut: int, osamp: int, nchunks: int = 2, reps: int = 2, mode: int = 0,
                row_tile: int = DEFAULT_ROW_TILE) -> Tuple[float, Tuple[str, int]]:
    """(ms per launch of the chain's time stage for one antenna, the form that
    ran) with the given time-filter setting; the previous setting is restored."""
    from .stream import StreamCorrelator
    prev = dict(_filter_setting)
    set_time_filter(mode, row_tile)
    try:
        return _time_chain_now(acclen, cut, osamp, nchunks, reps)
    finally:
        set_time_filter(prev["mode"], prev["row_tile"])


def _time_chain_now(acclen: int, cut: int, osamp: int, nchunks: int, reps: int) -> Tuple[float, Tuple[str, int]]:
    from .stream import StreamCorrelator
    dev = torch.device("cuda", torch.cuda.current_device())
    nch = 8
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    raw = torch.randint(0, 256, (1, nchunks * acclen, 2 * nch), generator=g, device=dev, dtype=torch.uint8)
    channels = np.arange(100, 100 + nch)
    nblock = max(acclen // osamp, 1)
    sc = StreamCorrelator(1, channels, 0, nch, acclen, nchunks, nblock, osamp, cut, 0.45, 4, nchan_raw=nch)
    try:
        for j in range(nchunks):  # warm-up (tables, attributes)
            sc.push(raw, j, final=(j == nchunks - 1))
        best = float("inf")
        for _ in range(reps):
            sc.reset()
            sc.profile(True)
            for j in range(nchunks):
                sc.push(raw, j, final=(j == nchunks - 1))
            ms, nl = sc.stage_times()["time_deconv"]
            sc.profile(False)
            best = min(best, ms / max(nl, 1))
        return best, sc.time_filter()
    finally:
        sc.close()


def tune_time_fft(acclen: int, cut: int, osamp: int = 64, *, use_cache: bool = True, limit: int = 24,
                  verbose: bool = False) -> Tuple[object, float]:
    """Choose the radix order for the time-axis FFT of nslice = acclen + 2*cut
    (n = nslice/2 points) and install it.  Returns (choice, ms per launch),
    choice = BUILTIN or the radix tuple."""
    _lib.require_cuda()
    n = (acclen + 2 * cut) // 2
    key = f"{torch.cuda.get_device_name()}|time_fft|{n}"
    with _lock:
        cache = _load_cache() if use_cache else {}
        hit = cache.get(key)
    if hit is not None:
        choice = BUILTIN if hit["radices"] == BUILTIN else tuple(hit["radices"])
        set_plan(n, None if choice == BUILTIN else choice)
        return choice, float(hit["ms"])
    results = []
    set_plan(n, None)
    try:
        results.append((BUILTIN, _time_chain(acclen, cut, osamp, mode=1)[0]))
    except (ValueError, _lib.AlbatrosError):
        pass  # no default plan for this length in the FFT kernels' limits
    for r in candidate_orders(n, limit):
        set_plan(n, r)
        try:
            results.append((r, _time_chain(acclen, cut, osamp, mode=1)[0]))
        except (ValueError, _lib.AlbatrosError):
            continue
        if verbose:
            print(f"n={n} radices={r}: {results[-1][1]:.3f} ms", flush=True)
    if not results:
        set_plan(n, None)
        raise ValueError(f"no FFT plan of length {n} runs in the time stage")
    choice, ms = min(results, key=lambda x: x[1])
    set_plan(n, None if choice == BUILTIN else choice)
    with _lock:
        cache = _load_cache()
        cache[key] = {"radices": BUILTIN if choice == BUILTIN else list(choice), "ms": ms,
                      "candidates": len(results), "builtin_ms": results[0][1]}
        if use_cache:
            _save_cache(cache)
    return choice, ms


def tune_time_stage(acclen: int, cut: int, osamp: int = 64, *, use_cache: bool = True, limit: int = 24,
                    verbose: bool = False) -> Dict[str, object]:
    """Choose the time stage for (acclen, cut, osamp): the IIR or FIR form with
    each of its row tiles, or the FFT form with its tuned radix order, whichever is
    fastest on this device.  Returns {"mode", "row_tile", "radices", "ms",
    "form"}; ``apply`` installs it."""
    _lib.require_cuda()
    key = f"{torch.cuda.get_device_name()}|time_stage|{acclen}|{cut}|{osamp}"
    with _lock:
        hit = (_load_cache() if use_cache else {}).get(key)
    if hit is not None:
        apply(hit)
        return hit
    cands = []
    for mode, kind in ((0, "iir"), (3, "fir")):
        for tile in ((64, 32, 16) if kind == "iir" else (32, 16)):  # FIR runs tile 64 as 32
            ms, form = _time_chain(acclen, cut, osamp, mode=mode, row_tile=tile)
            if form[0] != kind:
                break  # this form does not apply to the filter
            cands.append({"mode": mode, "row_tile": tile, "radices": None, "ms": ms, "form": list(form)})
            if verbose:
                print(f"acclen={acclen} cut={cut} osamp={osamp} {form} tile={tile}: {ms:.3f} ms", flush=True)
    try:
        radices, ms = tune_time_fft(acclen, cut, osamp, use_cache=use_cache, limit=limit if not cands else 0,
                                    verbose=verbose)
        cands.append({"mode": 1, "row_tile": _filter_setting["row_tile"],
                      "radices": radices if radices == BUILTIN else list(radices), "ms": ms, "form": ["fft", 0]})
    except (ValueError, _lib.AlbatrosError):
        pass
    if not cands:
        raise ValueError(f"no time stage runs for acclen={acclen}, cut={cut}, osamp={osamp}")
    best = min(cands, key=lambda c: c["ms"])
    best = dict(best, candidates=[(c["mode"], c["row_tile"], c["ms"]) for c in cands])
    with _lock:
        cache = _load_cache()
        cache[key] = best
        if use_cache:
            _save_cache(cache)
    apply(best)
    return best


def apply(choice: Dict[str, object]) -> None:
    """Install a ``tune_time_stage`` result for the streams created next."""
    set_time_filter(int(choice["mode"]), int(choice["row_tile"]))
    if int(choice["mode"]) == 1 and choice.get("radices") not in (None, BUILTIN):
        r = tuple(choice["radices"])
        set_plan(int(np.prod(r)), r)


def tune_configs(configs: Iterable[Tuple[int, int, int]], **kw) -> Dict[Tuple[int, int, int], Dict[str, object]]:
    """tune_time_stage once per distinct (acclen, cut, osamp)."""
    out = {}
    for cfg in configs:
        cfg = tuple(int(x) for x in cfg)
        if cfg not in out:
            out[cfg] = tune_time_stage(*cfg, **kw)
    return out
