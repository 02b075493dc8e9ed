"""Host/device array plumbing shared by the drop-in modules.

Arrays may be numpy arrays (host memory: the library stages them through the
device) or torch CUDA tensors (device memory: zero copy).  torch is only
imported when a tensor is passed in.
"""
from __future__ import annotations

import ctypes

import numpy as np


def is_cuda_tensor(x) -> bool:
    return type(x).__module__.startswith("torch") and bool(getattr(x, "is_cuda", False))


def is_tensor(x) -> bool:
    return type(x).__module__.startswith("torch")


def dtype_name(x) -> str:
    if is_tensor(x):
        return str(x.dtype).replace("torch.", "")
    return np.asarray(x).dtype.name


def require_dtype(x, want: str, what: str):
    """The reference's typed memoryviews reject other dtypes with ValueError
    ("Buffer dtype mismatch"); keep that behaviour."""
    got = dtype_name(x)
    if got != want:
        raise ValueError("Buffer dtype mismatch, expected '%s' for %s but got '%s'"
                         % (want, what, got))


def host_ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def dev_ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def torch_sync(t):
    """Make work queued by torch on the tensor's device visible to the library
    (the library issues on its own stream)."""
    import torch
    torch.cuda.current_stream(t.device).synchronize()
