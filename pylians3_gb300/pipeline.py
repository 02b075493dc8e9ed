"""Particles to power spectrum in one call on the GPU.

``power_spectrum(pos, dims, BoxSize, MAS, axis)`` does what the reference's
canonical caller does (library/Pk_library/Pk_snapshot.py:81-89):

    delta = zeros((dims,)*3); MA(pos, delta, BoxSize, MAS, W)
    delta /= mean(delta); delta -= 1
    Pk(delta, BoxSize, axis, MAS)

but keeps the grid resident on the device and folds the overdensity step into
the spectrum (pyl_pk_particles).  Only the positions go to the device and only
the spectra come back.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._arrays import dev_ptr, host_ptr, is_cuda_tensor, require_dtype, torch_sync
from .Pk_library import MAS_function, _Outputs, _raise_or_exit


class Spectrum:
    """Result holder with the attributes of class Pk that were requested."""


DEPOSIT_FLAGS = {
    "auto": 0,                                   # fixed-point tiles for unit weights
    "float": _native.PYL_DEPOSIT_FLOAT,          # float32 shared atomics
    "compensated": _native.PYL_COMPENSATED,      # float32 + TwoSum error grid
}


def power_spectrum(pos, dims, BoxSize, MAS="CIC", axis=2, W=None, window=None,
                   what=0, ctx=None, deposit="auto"):
    """Spectrum of the particles' overdensity field on a dims^3 grid.

    pos: (n, 3) float32 numpy array (pinned memory copies fastest, see
    ``pinned_empty``) or torch CUDA tensor.  MAS is the deposit scheme;
    ``window`` the window to deconvolve (default: the same as MAS).
    ``what``: extra outputs (Pk_library.PK_1D | PK_2D | PK_PHASE).
    ``deposit``: accumulation of the grid, one of DEPOSIT_FLAGS.
    """
    require_dtype(pos, "float32", "pos")
    if pos.ndim != 2 or int(pos.shape[1]) != 3:
        raise ValueError("pos must be (n, 3)")
    if MAS not in _native.MAS_CODE:
        raise ValueError("option not valid!!! (MAS must be NGP, CIC, TSC or PCS)")
    n = int(pos.shape[0])
    if W is not None and int(W.shape[0]) < n:
        raise ValueError("W has %d entries for %d particles" % (int(W.shape[0]), n))
    win = MAS_function(MAS if window is None else window)
    if deposit not in DEPOSIT_FLAGS:
        raise ValueError("deposit must be one of %s" % sorted(DEPOSIT_FLAGS))
    dflags = DEPOSIT_FLAGS[deposit]
    out = _Outputs(int(dims), what)
    if is_cuda_tensor(pos):
        ctx = ctx or _native.context(pos.device.index or 0)
        p = pos.contiguous()
        w = None if W is None else W.contiguous()
        torch_sync(p)
        rc = ctx.lib.pyl_pk_particles(
            ctx.ptr, dev_ptr(p), n, dev_ptr(w) if w is not None else None, int(dims),
            ctypes.c_float(BoxSize), _native.MAS_CODE[MAS], int(axis), win, int(what),
            ctypes.byref(out.struct), _native.PYL_DEVICE_PTRS | dflags)
    else:
        ctx = ctx or _native.context(0)
        p = np.ascontiguousarray(pos)
        w = None if W is None else np.ascontiguousarray(W, np.float32)
        rc = ctx.lib.pyl_pk_particles(
            ctx.ptr, host_ptr(p), n, host_ptr(w) if w is not None else None, int(dims),
            ctypes.c_float(BoxSize), _native.MAS_CODE[MAS], int(axis), win, int(what),
            ctypes.byref(out.struct), dflags)
    _raise_or_exit(ctx, rc)
    res = Spectrum()
    out.assign(res)
    return res
