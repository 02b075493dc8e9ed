"""Drop-in ``Pk_library`` on the GB300: FFTs and the power spectrum.

Same names, argument meaning and observable behaviour as Pylians3's
library/Pk_library/Pk_library.pyx:
  * ``Pk(delta, BoxSize, axis=2, MAS='CIC', threads=1, verbose=True)``
    (:263-418) with attributes k3D, Pk[:,0:3], Nmodes3D, k1D, Pk1D, Nmodes1D,
    kpar, kper, Pk2D, Nmodes2D, Pkphase.
  * ``FFT3Dr_f(a, threads)`` (:117-130) and ``IFFT3Dr_f(a, threads)``
    (:149-162), float32/complex64, inverse normalised by 1/N^3.
  * helpers ``frequencies``, ``MAS_function``, ``MAS_correction``,
    ``check_number_modes`` (:56-99).
All the arithmetic over the grid runs on the GPU (libpylgpu.so); ``threads``
is accepted for compatibility and ignored.  ``delta`` may be a numpy array or
a torch CUDA tensor (zero copy).
"""
from __future__ import annotations

import ctypes
import math
import sys
import time

import numpy as np

from . import _native
from ._arrays import dev_ptr, host_ptr, is_cuda_tensor, is_tensor, require_dtype, torch_sync

__all__ = ["Pk", "FFT3Dr_f", "IFFT3Dr_f", "frequencies", "MAS_function",
           "MAS_correction", "check_number_modes"]


def frequencies(BoxSize, dims):
    """kF, kN, kmax_par, kmax_per, kmax (Pk_library.pyx:56-61)."""
    kF = 2.0 * np.pi / BoxSize
    middle = dims // 2
    kN = middle * kF
    kmax_par = middle
    kmax_per = int(np.sqrt(middle ** 2 + middle ** 2))
    kmax = int(np.sqrt(middle ** 2 + middle ** 2 + middle ** 2))
    return kF, kN, kmax_par, kmax_per, kmax


def MAS_function(MAS):
    """MAS_index (Pk_library.pyx:72-78)."""
    return {"NGP": 1, "CIC": 2, "TSC": 3, "PCS": 4}.get(MAS, 0)


def MAS_correction(x, MAS_index):
    """(x / sin x)^p, 1 at x = 0 (Pk_library.pyx:83-84)."""
    return 1.0 if x == 0.0 else math.pow(x / math.sin(x), MAS_index)


def check_number_modes(Nmodes, dims):
    """Pk_library.pyx:87-99: exits when not every independent mode is counted."""
    own_modes = 1 if dims % 2 == 1 else 8
    repeated_modes = (dims ** 3 - own_modes) // 2
    indep_modes = repeated_modes + own_modes
    if int(np.sum(Nmodes)) != indep_modes:
        print("WARNING: Not all modes counted")
        print("Counted  %d independent modes" % (int(np.sum(Nmodes))))
        print("Expected %d independent modes" % indep_modes)
        sys.exit()


def _check_cube(a, what):
    if a.ndim != 3 or not (a.shape[0] == a.shape[1] == a.shape[2]):
        raise ValueError("%s must be a (dims, dims, dims) array, got %s" % (what, tuple(a.shape)))


def FFT3Dr_f(a, threads=1):
    """r2c 3D FFT, unnormalised, complex64 (dims, dims, dims//2+1)."""
    require_dtype(a, "float32", "a")
    _check_cube(a, "a")
    dims = int(a.shape[0])
    h = dims // 2 + 1
    if is_cuda_tensor(a):
        import torch
        ctx = _native.context(a.device.index or 0)
        src = a.contiguous()
        out = torch.empty((dims, dims, h), dtype=torch.complex64, device=a.device)
        torch_sync(src)
        ctx.check(ctx.lib.pyl_fft_r2c(ctx.ptr, dev_ptr(src), dev_ptr(out), dims,
                                      _native.PYL_DEVICE_PTRS))
        ctx.synchronize()
        return out
    ctx = _native.context(0)
    src = np.ascontiguousarray(a)
    out = np.empty((dims, dims, h), np.complex64)
    ctx.check(ctx.lib.pyl_fft_r2c(ctx.ptr, host_ptr(src), host_ptr(out), dims, 0))
    return out


def IFFT3Dr_f(a, threads=1):
    """c2r 3D FFT normalised by 1/dims^3, float32 (dims, dims, dims)."""
    require_dtype(a, "complex64", "a")
    dims = int(a.shape[0])
    h = dims // 2 + 1
    if a.ndim != 3 or tuple(int(s) for s in a.shape) != (dims, dims, h):
        raise ValueError("a must be (dims, dims, dims//2+1), got %s" % (tuple(a.shape),))
    if is_cuda_tensor(a):
        import torch
        ctx = _native.context(a.device.index or 0)
        src = a.contiguous()
        out = torch.empty((dims, dims, dims), dtype=torch.float32, device=a.device)
        torch_sync(src)
        ctx.check(ctx.lib.pyl_fft_c2r(ctx.ptr, dev_ptr(src), dev_ptr(out), dims,
                                      _native.PYL_DEVICE_PTRS))
        ctx.synchronize()
        return out
    ctx = _native.context(0)
    src = np.ascontiguousarray(a)
    out = np.empty((dims, dims, dims), np.float32)
    ctx.check(ctx.lib.pyl_fft_c2r(ctx.ptr, host_ptr(src), host_ptr(out), dims, 0))
    return out


class _Outputs:
    """Host float64 output arrays of pyl_pk / pyl_pk_particles."""

    def __init__(self, dims, what):
        kmax, kmax_par, kmax_per = _native.pk_sizes(dims)
        self.what = what
        self.k3D = np.zeros(kmax)
        self.Pk = np.zeros((kmax, 3))
        self.Nmodes3D = np.zeros(kmax)
        n2 = (kmax_par + 1) * (kmax_per + 1)
        self.k1D = np.zeros(kmax_par)
        self.Pk1D = np.zeros(kmax_par)
        self.Nmodes1D = np.zeros(kmax_par)
        self.kpar = np.zeros(n2)
        self.kper = np.zeros(n2)
        self.Pk2D = np.zeros(n2)
        self.Nmodes2D = np.zeros(n2)
        self.Pkphase = np.zeros(kmax)
        self.struct = _native.PkOut(*[a.ctypes.data for a in (
            self.k3D, self.Pk, self.Nmodes3D, self.k1D, self.Pk1D, self.Nmodes1D,
            self.kpar, self.kper, self.Pk2D, self.Nmodes2D, self.Pkphase)])

    def assign(self, obj):
        obj.k3D, obj.Pk, obj.Nmodes3D = self.k3D, self.Pk, self.Nmodes3D
        if self.what & _native.PYL_PK_1D:
            obj.k1D, obj.Pk1D, obj.Nmodes1D = self.k1D, self.Pk1D, self.Nmodes1D
        if self.what & _native.PYL_PK_2D:
            obj.kpar, obj.kper = self.kpar, self.kper
            obj.Pk2D, obj.Nmodes2D = self.Pk2D, self.Nmodes2D
        if self.what & _native.PYL_PK_PHASE:
            obj.Pkphase = self.Pkphase


def _raise_or_exit(ctx, rc):
    if rc == _native.PYL_ERR_MODES:
        # the reference prints and exits (check_number_modes, :87-99)
        msg = ctx.lib.pyl_last_error(ctx.ptr)
        print(msg.decode() if msg else "WARNING: Not all modes counted")
        sys.exit()
    ctx.check(rc)


class Pk:
    """1D, 2D and 3D power spectra of a density field (Pk_library.pyx:263-418).

    ``what`` (an extension; default all outputs, as the reference) selects the
    outputs: a bit mask of PK_1D, PK_2D, PK_PHASE; k3D/Pk/Nmodes3D always.
    """

    def __init__(self, delta, BoxSize, axis=2, MAS="CIC", threads=1, verbose=True,
                 what=_native.PYL_PK_ALL):
        start = time.time()
        require_dtype(delta, "float32", "delta")
        _check_cube(delta, "delta")
        if verbose:
            print("\nComputing power spectrum of the field...")
        dims = int(delta.shape[0])
        axis = int(axis)
        MAS_index = MAS_function(MAS)
        out = _Outputs(dims, what)
        if is_cuda_tensor(delta):
            ctx = _native.context(delta.device.index or 0)
            src = delta.contiguous()
            torch_sync(src)
            rc = ctx.lib.pyl_pk(ctx.ptr, dev_ptr(src), dims, float(BoxSize), axis,
                                MAS_index, int(what), ctypes.byref(out.struct),
                                _native.PYL_DEVICE_PTRS)
        else:
            ctx = _native.context(0)
            src = np.ascontiguousarray(delta.cpu().numpy() if is_tensor(delta) else delta)
            rc = ctx.lib.pyl_pk(ctx.ptr, host_ptr(src), dims, float(BoxSize), axis,
                                MAS_index, int(what), ctypes.byref(out.struct), 0)
        _raise_or_exit(ctx, rc)
        out.assign(self)
        if verbose:
            print("Time taken = %.2f seconds" % (time.time() - start))


PK_3D, PK_1D, PK_2D, PK_PHASE, PK_ALL = (0, _native.PYL_PK_1D, _native.PYL_PK_2D,
                                         _native.PYL_PK_PHASE, _native.PYL_PK_ALL)
