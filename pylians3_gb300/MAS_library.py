"""Drop-in ``MAS_library`` on the GB300: particle mass assignment.

Same functions, argument meaning and observable behaviour as Pylians3's
library/MAS_library/MAS_library.pyx:
  * ``MA(pos, number, BoxSize, MAS='CIC', W=None, verbose=False,
    renormalize_2D=True)``  (:57-112): accumulates into ``number``.
  * ``NGP/CIC/TSC/PCS(pos, number, BoxSize)`` and
    ``NGPW/CICW/TSCW/PCSW(pos, number, BoxSize, W)`` (:123-545).
  * ``NGPW_d/CICW_d`` with a float64 grid (:229-266, :338-358).
  * ``NGPc3D..PCSWc3D(pos, number, BoxSize, threads)`` (:1305-1389): the
    reference's OpenMP entry points; ``threads`` is accepted and ignored.
  * ``CIC_interp(density, BoxSize, pos, den)`` (:558-599): trilinear
    interpolation of a grid at the positions, written into ``den``.
The deposit runs on the GPU (libpylgpu.so, pyl_ma); there is no CPU path.
``pos``/``number``/``W`` may be numpy arrays or torch CUDA tensors.
"""
from __future__ import annotations

import ctypes
import sys
import time

import numpy as np

from . import _native
from ._arrays import (dev_ptr, host_ptr, is_cuda_tensor, is_tensor, require_dtype,
                      torch_sync)

__all__ = ["MA", "NGP", "CIC", "TSC", "PCS", "NGPW", "CICW", "TSCW", "PCSW",
           "NGPW_d", "CICW_d", "NGPc3D", "CICc3D", "TSCc3D", "PCSc3D",
           "NGPWc3D", "CICWc3D", "TSCWc3D", "PCSWc3D", "FLOAT_type", "CIC_interp"]

_RENORM = {"NGP": 1.0, "CIC": 2.0, "TSC": 3.0, "PCS": 4.0}


def FLOAT_type():
    """The grid type of the deposit (MAS_library.pyx:11-13)."""
    return np.float32


def _deposit(pos, number, BoxSize, MAS, W, coord, renormalize_2D, grid_dtype="float32"):
    """pos (n, coord) float32; number (dims,)*coord (or (dims, dims, 1))."""
    require_dtype(pos, "float32", "pos")
    require_dtype(number, grid_dtype, "number")
    if W is not None:
        require_dtype(W, "float32", "W")
    n = int(pos.shape[0])
    dims = int(number.shape[0])
    shape = tuple(int(s) for s in number.shape)
    if coord == 3 and shape != (dims, dims, dims):
        raise ValueError("number must be a (dims, dims, dims) cube, got %s" % (shape,))
    if coord == 2 and shape not in ((dims, dims), (dims, dims, 1)):
        raise ValueError("number must be (dims, dims) for 2D positions, got %s" % (shape,))
    if W is not None and int(W.shape[0]) < n:
        raise ValueError("W has %d entries for %d particles" % (int(W.shape[0]), n))
    ctx = _native.context(number.device.index if is_cuda_tensor(number) else 0)
    lib = ctx.lib
    mas = _native.MAS_CODE[MAS]
    fn = lib.pyl_ma if grid_dtype == "float32" else lib.pyl_ma_f64
    if is_cuda_tensor(number):
        import torch
        dev = number.device
        p = pos if is_cuda_tensor(pos) else torch.as_tensor(np.asarray(pos), device=dev)
        p = p.contiguous()
        w = None
        if W is not None:
            w = (W if is_cuda_tensor(W) else torch.as_tensor(np.asarray(W), device=dev)).contiguous()
        g = number if number.is_contiguous() else number.contiguous()
        torch_sync(g)
        ctx.check(fn(ctx.ptr, dev_ptr(p), n, coord, dev_ptr(w) if w is not None else None,
                     dev_ptr(g), dims, ctypes.c_float(BoxSize), mas,
                     1 if renormalize_2D else 0, _native.PYL_DEVICE_PTRS))
        ctx.synchronize()
        if g is not number:
            number.copy_(g)
        return
    if is_tensor(pos) or is_tensor(number) or (W is not None and is_tensor(W)):
        pos = pos.cpu().numpy() if is_tensor(pos) else pos
        W = W.cpu().numpy() if (W is not None and is_tensor(W)) else W
    p = np.ascontiguousarray(pos)
    w = None if W is None else np.ascontiguousarray(W)
    g = number if number.flags.c_contiguous else np.ascontiguousarray(number)
    ctx.check(fn(ctx.ptr, host_ptr(p), n, coord, host_ptr(w) if w is not None else None,
                 host_ptr(g), dims, ctypes.c_float(BoxSize), mas,
                 1 if renormalize_2D else 0, 0))
    if g is not number:
        number[...] = g


def MA(pos, number, BoxSize, MAS="CIC", W=None, verbose=False, renormalize_2D=True):
    """Mass assignment (MAS_library.pyx:57-112); accumulates into ``number``."""
    coord, coord_aux = pos.shape[1], number.ndim
    if coord != coord_aux:
        print("pos have %d dimensions and the density %d!!!" % (coord, coord_aux))
        sys.exit()
    if verbose:
        if W is None:
            print("\nUsing %s mass assignment scheme" % MAS)
        else:
            print("\nUsing %s mass assignment scheme with weights" % MAS)
    start = time.time()
    if coord not in (2, 3) or MAS not in _native.MAS_CODE:
        print("option not valid!!!")
        sys.exit()
    _deposit(pos, number, BoxSize, MAS, W, coord, renormalize_2D)
    if verbose:
        print("Time taken = %.3f seconds\n" % (time.time() - start))


def _single(MAS, pos, number, BoxSize, W=None, grid_dtype="float32"):
    # The per-scheme functions take the 3D grid; MA's 2D path hands them
    # expand_dims(number, 2), i.e. (dims, dims, 1), with no renormalisation.
    coord = int(pos.shape[1])
    if coord == 2 and number.ndim == 3 and int(number.shape[2]) == 1:
        _deposit(pos, number, BoxSize, MAS, W, 2, False, grid_dtype)
    else:
        _deposit(pos, number, BoxSize, MAS, W, 3, False, grid_dtype)


def NGP(pos, number, BoxSize):
    """MAS_library.pyx:273-292"""
    _single("NGP", pos, number, BoxSize)


def CIC(pos, number, BoxSize):
    """MAS_library.pyx:123-166"""
    _single("CIC", pos, number, BoxSize)


def TSC(pos, number, BoxSize):
    """MAS_library.pyx:369-404"""
    _single("TSC", pos, number, BoxSize)


def PCS(pos, number, BoxSize):
    """MAS_library.pyx:463-497"""
    _single("PCS", pos, number, BoxSize)


def NGPW(pos, number, BoxSize, W):
    """MAS_library.pyx:305-325"""
    _single("NGP", pos, number, BoxSize, W)


def CICW(pos, number, BoxSize, W):
    """MAS_library.pyx:179-216"""
    _single("CIC", pos, number, BoxSize, W)


def TSCW(pos, number, BoxSize, W):
    """MAS_library.pyx:417-452"""
    _single("TSC", pos, number, BoxSize, W)


def PCSW(pos, number, BoxSize, W):
    """MAS_library.pyx:510-545"""
    _single("PCS", pos, number, BoxSize, W)


def NGPW_d(pos, number, BoxSize, W):
    """float64 grid, MAS_library.pyx:338-358"""
    _single("NGP", pos, number, BoxSize, W, "float64")


def CICW_d(pos, number, BoxSize, W):
    """float64 grid, MAS_library.pyx:229-266"""
    _single("CIC", pos, number, BoxSize, W, "float64")


def _c3d(MAS, pos, number, BoxSize, W=None):
    _deposit(pos, number, BoxSize, MAS, W, int(pos.shape[1]), False)


def NGPc3D(pos, number, BoxSize, threads=1):
    """MAS_library.pyx:1306 (threads ignored: the deposit runs on the GPU)"""
    _c3d("NGP", pos, number, BoxSize)


def NGPWc3D(pos, number, W, BoxSize, threads=1):
    """MAS_library.pyx:1311"""
    _c3d("NGP", pos, number, BoxSize, W)


def CICc3D(pos, number, BoxSize, threads=1):
    """MAS_library.pyx:1328"""
    _c3d("CIC", pos, number, BoxSize)


def CICWc3D(pos, number, W, BoxSize, threads=1):
    """MAS_library.pyx:1333"""
    _c3d("CIC", pos, number, BoxSize, W)


def TSCc3D(pos, number, BoxSize, threads=1):
    """MAS_library.pyx:1350"""
    _c3d("TSC", pos, number, BoxSize)


def TSCWc3D(pos, number, W, BoxSize, threads=1):
    """MAS_library.pyx:1355"""
    _c3d("TSC", pos, number, BoxSize, W)


def PCSc3D(pos, number, BoxSize, threads=1):
    """MAS_library.pyx:1372"""
    _c3d("PCS", pos, number, BoxSize)


def PCSWc3D(pos, number, W, BoxSize, threads=1):
    """MAS_library.pyx:1377"""
    _c3d("PCS", pos, number, BoxSize, W)


def CIC_interp(density, BoxSize, pos, den):
    """Trilinear (CIC) interpolation of ``density`` (dims^3 float32) at
    ``pos`` ((n, 3) float32) into ``den`` ((n,) float32), in place
    (MAS_library.pyx:558-599)."""
    require_dtype(density, "float32", "density")
    require_dtype(pos, "float32", "pos")
    require_dtype(den, "float32", "den")
    if density.ndim != 3 or pos.ndim != 2 or den.ndim != 1:
        raise ValueError("density must be 3D, pos 2D and den 1D")
    n = int(pos.shape[0])
    dims = int(density.shape[0])
    if int(den.shape[0]) < n:
        raise ValueError("den has %d entries for %d positions" % (int(den.shape[0]), n))
    cuda = [is_cuda_tensor(x) for x in (density, pos, den)]
    if all(cuda):
        ctx = _native.context(den.device.index or 0)
        g, p = density.contiguous(), pos.contiguous()
        out = den if den.is_contiguous() else den.contiguous()
        torch_sync(out)
        ctx.check(ctx.lib.pyl_cic_interp(ctx.ptr, dev_ptr(g), dims, ctypes.c_float(BoxSize),
                                         dev_ptr(p), n, dev_ptr(out), _native.PYL_DEVICE_PTRS))
        ctx.synchronize()
        if out is not den:
            den.copy_(out)
        return
    if any(cuda):
        raise ValueError("density, pos and den must be all host arrays or all CUDA tensors")
    ctx = _native.context(0)
    g = np.ascontiguousarray(density.cpu().numpy() if is_tensor(density) else density)
    p = np.ascontiguousarray(pos.cpu().numpy() if is_tensor(pos) else pos)
    out = den if (isinstance(den, np.ndarray) and den.flags.c_contiguous) else np.empty(n, np.float32)
    ctx.check(ctx.lib.pyl_cic_interp(ctx.ptr, host_ptr(g), dims, ctypes.c_float(BoxSize),
                                     host_ptr(p), n, host_ptr(out), 0))
    if out is not den:
        den[:n] = out
