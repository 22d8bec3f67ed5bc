"""Device-array helpers: accept torch CUDA tensors or any object exposing
``__cuda_array_interface__`` / DLPack (the reference passes CuPy arrays), and
validate shapes on the host before a pointer reaches a kernel."""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def device_array(a, dtype: torch.dtype | None = None, name: str = "array") -> torch.Tensor:
    """Zero-copy view of a device array as a torch CUDA tensor.

    Host arrays are rejected, as the reference's GPU path asserts
    ``isinstance(data, xp.ndarray)`` (albatros_analysis/src/correlations/unpacking.py:240,297)."""
    _lib.require_cuda()
    if isinstance(a, torch.Tensor):
        t = a
    elif isinstance(a, np.ndarray):
        raise TypeError(f"{name} must be a device array, got a host numpy array")
    elif hasattr(a, "__cuda_array_interface__"):
        t = torch.as_tensor(a, device="cuda")
    elif hasattr(a, "__dlpack__") and hasattr(a, "__dlpack_device__") and a.__dlpack_device__()[0] == 2:
        t = torch.from_dlpack(a)  # kDLCUDA
    else:
        raise TypeError(f"{name} must be a device array (torch CUDA tensor or __cuda_array_interface__), "
                        f"got {type(a).__name__}")
    if not t.is_cuda:
        raise TypeError(f"{name} must live on a CUDA device")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must have dtype {dtype}, got {t.dtype}")
    return t


def to_device(a, dtype: torch.dtype, device=None) -> torch.Tensor:
    """Host or device array -> contiguous torch CUDA tensor of `dtype` (copies host data)."""
    _lib.require_cuda()
    if isinstance(a, torch.Tensor):
        t = a
    elif hasattr(a, "__cuda_array_interface__"):
        t = torch.as_tensor(a, device="cuda")
    else:
        t = torch.from_numpy(np.ascontiguousarray(a))
    dev = device if device is not None else (t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device()))
    return t.to(device=dev, dtype=dtype).contiguous()


def host_int64(a, name: str = "array") -> np.ndarray:
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64).ravel())
