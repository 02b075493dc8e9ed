"""Redshift-space displacement of particle positions on the GPU.

``pos_redshift_space(pos, vel, BoxSize, Hubble, redshift, axis)`` as
Pylians3's library/redshift_space_library/redshift_space_library.pyx:29-50:
in place, pos[:, axis] += vel[:, axis] * (1 + redshift) / Hubble, wrapped
into [0, BoxSize].  ``pos``/``vel`` are (n, 3) float32 numpy arrays or CUDA
tensors (zero copy).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._arrays import dev_ptr, host_ptr, is_cuda_tensor, require_dtype, torch_sync


def pos_redshift_space(pos, vel, BoxSize, Hubble, redshift, axis):
    require_dtype(pos, "float32", "pos")
    require_dtype(vel, "float32", "vel")
    if pos.ndim != 2 or int(pos.shape[1]) != 3 or tuple(vel.shape) != tuple(pos.shape):
        raise ValueError("pos and vel must both be (n, 3)")
    n = int(pos.shape[0])
    args = (ctypes.c_float(BoxSize), ctypes.c_float(Hubble), ctypes.c_float(redshift), int(axis))
    if is_cuda_tensor(pos) and is_cuda_tensor(vel):
        if not pos.is_contiguous():
            raise ValueError("pos must be contiguous (it is updated in place)")
        ctx = _native.context(pos.device.index or 0)
        v = vel.contiguous()
        torch_sync(pos)
        ctx.check(ctx.lib.pyl_rsd(ctx.ptr, dev_ptr(pos), dev_ptr(v), n, *args,
                                  _native.PYL_DEVICE_PTRS))
        ctx.synchronize()
        return
    if not (isinstance(pos, np.ndarray) and pos.flags.c_contiguous):
        raise ValueError("pos must be a C-contiguous numpy array (it is updated in place)")
    ctx = _native.context(0)
    v = np.ascontiguousarray(vel)
    ctx.check(ctx.lib.pyl_rsd(ctx.ptr, host_ptr(pos), host_ptr(v), n, *args, 0))
