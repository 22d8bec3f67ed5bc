"""ctypes binding of ``lib/libalbatros_gb300.so`` (C-ABI in include/albatros_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded,
every op raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libalbatros_gb300.so")

P, I64, I32, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "ab_version": (I32, []),
    "ab_strerror": (ctypes.c_char_p, [I32]),
    "ab_last_error": (ctypes.c_char_p, []),
    "ab_ctx_create": (I32, [I32, ctypes.POINTER(P)]),
    "ab_ctx_destroy": (I32, [P]),
    "ab_ctx_set_fft_plan": (I32, [P, I64, P, I64]),
    "ab_ctx_set_time_filter": (I32, [P, I32, I32]),
    "ab_ctx_set_option": (I32, [P, I32, I32]),
    "ab_unpack_4bit": (I32, [P, P, P, I64, I64, P, I64, I64, P]),
    "ab_unpack_4bit_range": (I32, [P, P, P, I64, I64, I64, I64, I64, P]),
    "ab_unpack_1bit": (I32, [P, P, P, I64, I64, P, I64, I64, P]),
    "ab_sortpols": (I32, [P, P, P, I64, I64, I64, I64, I32, I64, I64, P]),
    "ab_make_continuous": (I32, [P, I64, I64, P, I64, P, I64, I64, P, P]),
    "ab_hist": (I32, [P, P, I64, I64, I64, I32, I32, P]),
    "ab_unpack_4bit_i8": (I32, [P, P, P, I64, I64, P, I64, I64, P]),
    "ab_unpack_1bit_i8": (I32, [P, P, P, I64, I64, P, I64, I64, P]),
    "ab_packets_to_rows": (I32, [P, I64, I64, P, P]),
    "ab_spec_map_init": (I32, [P, I64, P]),
    "ab_spec_map_add": (I32, [P, I64, I32, I64, I64, P, I64, P]),
    "ab_spec_map_finish": (I32, [P, I64, P]),
    "ab_get_matft": (I32, [P, P, I64, I64, I64, P]),
    "ab_calculate_filter": (I32, [P, P, I64, D, P]),
    "ab_build_filter": (I32, [P, P, I64, I64, I64, D, P]),
    "ab_ipfb": (I32, [P, P, P, P, I64, I64, P]),
    "ab_pfb": (I32, [P, P, I64, P, I64, I64, P, P]),
    "ab_pfb_band": (I32, [P, P, I64, P, I64, I64, I64, I64, P, P]),
    "ab_avg_xcorr_all_ant": (I32, [P, I64, I64, I64, I64, P, P]),
    "ab_xcorr_coarse_4bit": (I32, [P, P, I64, I64, I64, I64, I64, I64, P, P, I64, I64, P, P, P]),
    "ab_xcorr_coarse_4bit_noalloc": (I32, [P, I64, I64, I64, I64, I64, I64, P, P, I64, I64, P, P, P]),
    "ab_avg_xcorr_4bit_pairs": (I32, [P, P, P, P, I64, I64, P, P, P]),
    "ab_avg_xcorr_1bit_pairs": (I32, [P, P, P, P, I64, I64, I64, P, P]),
    "ab_stream_create": (I32, [P, I64, I64, I64, P, P, I64, I64, I64, I64, I64, D, I64, I64, I64, I64,
                               ctypes.POINTER(P)]),
    "ab_stream_destroy": (I32, [P]),
    "ab_stream_reset": (I32, [P, P]),
    "ab_stream_push": (I32, [P, P, I64, P, I64, I64, P]),
    "ab_stream_push_final": (I32, [P, P, I64, P, I64, I64, P]),
    "ab_stream_vis": (P, [P]),
    "ab_stream_profile": (I32, [P, I32]),
    "ab_stream_stage_times": (I32, [P, P, P]),
    "ab_stream_kernel_launches": (I64, [P]),
    "ab_stream_workspace_bytes": (I64, [P]),
    "ab_stream_fir_taps": (I64, [P]),
    "ab_stream_time_filter": (I32, [P, P, P]),
    "ab_stream_set_workspace": (I32, [P, P, I64]),
}

_lib = None
_lock = threading.Lock()
_ctx: dict[int, int] = {}


class AlbatrosError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, fn: str, code: int, detail: str):
        super().__init__(f"{fn} failed with status {code}: {detail}")
        self.code = code


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the library (building it first if this checkout has no build)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            from . import build as _build
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def call(name: str, *args) -> int:
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        detail = lib.ab_last_error().decode(errors="replace")
        if rc == -1:
            raise ValueError(f"{name}: {detail}")
        raise AlbatrosError(name, rc, detail)
    return rc


def require_cuda() -> None:
    if not torch.cuda.is_available():
        raise RuntimeError("albatros_axion_detection_gb300 needs a CUDA device (no CPU path)")


def ctx(device: int | None = None) -> int:
    """Per-device library context (twiddle tables, plans, scratch)."""
    require_cuda()
    dev = torch.cuda.current_device() if device is None else int(device)
    with _lock:
        c = _ctx.get(dev)
    if c is not None:
        return c
    out = ctypes.c_void_p()
    with torch.cuda.device(dev):
        call("ab_ctx_create", dev, ctypes.byref(out))
    with _lock:
        _ctx[dev] = out.value
    return out.value


def stream_ptr(tensor_or_device=None) -> int:
    """Raw cudaStream_t of torch's current stream on the tensor's device."""
    if isinstance(tensor_or_device, torch.Tensor):
        return torch.cuda.current_stream(tensor_or_device.device).cuda_stream
    return torch.cuda.current_stream(tensor_or_device).cuda_stream


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()
