"""Drop-in ``Pk_library`` on the GB300: FFTs and the power spectrum.

Same names, argument meaning and observable behaviour as Pylians3's
library/Pk_library/Pk_library.pyx:
  * ``Pk(delta, BoxSize, axis=2, MAS='CIC', threads=1, verbose=True)``
    (:263-418) with attributes k3D, Pk[:,0:3], Nmodes3D, k1D, Pk1D, Nmodes1D,
    kpar, kper, Pk2D, Nmodes2D, Pkphase.
  * ``FFT3Dr_f(a, threads)`` (:117-130) and ``IFFT3Dr_f(a, threads)``
    (:149-162), float32/complex64, inverse normalised by 1/N^3.
  * helpers ``frequencies``, ``MAS_function``, ``MAS_correction``,
    ``check_number_modes`` (:56-99), ``frequencies_2D``,
    ``check_number_modes_2D`` (:64-69, :102-115).
  * ``XPk(delta, BoxSize, axis=2, MAS=None, threads=1)`` (:529-735),
    ``Pk_plane(delta, BoxSize, MAS='CIC', threads=1, verbose=True)``
    (:435-511), ``correct_MAS(delta, BoxSize, MAS='CIC', threads=1)``
    (:1882-1939), ``FFT2Dr_f`` / ``IFFT2Dr_f`` (:181-196, :213-228).
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

__all__ = ["Pk", "XPk", "Pk_plane", "correct_MAS", "FFT3Dr_f", "IFFT3Dr_f", "FFT2Dr_f",
           "IFFT2Dr_f", "frequencies", "frequencies_2D", "MAS_function", "MAS_correction",
           "check_number_modes", "check_number_modes_2D"]


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


# ----------------------------------------------------------------------------
# Rows around the spectrum: correct_MAS, the 2D FFTs and Pk_plane, XPk
# ----------------------------------------------------------------------------
def _call_grid(fn_name, a, out_shape, out_dtype, *args):
    """Runs pyl_<fn>(ctx, in, out, *args, flags) on numpy or CUDA tensors."""
    if is_cuda_tensor(a):
        import torch
        ctx = _native.context(a.device.index or 0)
        src = a.contiguous()
        out = torch.empty(out_shape, dtype=getattr(torch, out_dtype), device=a.device)
        torch_sync(src)
        ctx.check(getattr(ctx.lib, fn_name)(ctx.ptr, dev_ptr(src), dev_ptr(out), *args,
                                            _native.PYL_DEVICE_PTRS))
        ctx.synchronize()
        return out
    ctx = _native.context(0)
    src = np.ascontiguousarray(a.cpu().numpy() if is_tensor(a) else a)
    out = np.empty(out_shape, out_dtype)
    ctx.check(getattr(ctx.lib, fn_name)(ctx.ptr, host_ptr(src), host_ptr(out), *args, 0))
    return out


def correct_MAS(delta, BoxSize, MAS="CIC", threads=1):
    """The field with its independent Fourier modes divided by the MAS window
    (Pk_library.pyx:1882-1939); returns a new float32 field."""
    start = time.time()
    require_dtype(delta, "float32", "delta")
    _check_cube(delta, "delta")
    print("\nComputing power spectrum of the field...")
    dims = int(delta.shape[0])
    start2 = time.time()
    out = _call_grid("pyl_correct_mas", delta, (dims, dims, dims), "float32", dims,
                     MAS_function(MAS))
    print("Time to complete loop = %.2f" % (time.time() - start2))
    print("Time taken = %.2f seconds" % (time.time() - start))
    return out


def frequencies_2D(BoxSize, dims):
    """kF, kN, kmax_par, kmax_per, kmax of a 2D grid (Pk_library.pyx:64-69)."""
    kF = 2.0 * np.pi / BoxSize
    middle = dims // 2
    kN = middle * kF
    return kF, kN, middle, middle, int(np.sqrt(middle ** 2 + middle ** 2))


def check_number_modes_2D(Nmodes, dims):
    """Pk_library.pyx:102-115: exits when not every independent mode is counted."""
    own_modes = 1 if dims % 2 == 1 else 4
    indep_modes = (dims ** 2 - own_modes) // 2 + own_modes
    if int(np.sum(Nmodes)) != indep_modes:
        print("WARNING: Not all modes counted")
        print("Counted  %d independent modes" % (int(np.sum(Nmodes))))
        print("Expected %d independent modes" % indep_modes)
        sys.exit()


def _check_square(a, what):
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise ValueError("%s must be a (grid, grid) array, got %s" % (what, tuple(a.shape)))


def FFT2Dr_f(a, threads=1):
    """r2c 2D FFT, unnormalised, complex64 (grid, grid//2+1) (:181-196)."""
    require_dtype(a, "float32", "a")
    _check_square(a, "a")
    g = int(a.shape[0])
    return _call_grid("pyl_fft2_r2c", a, (g, g // 2 + 1), "complex64", g)


def IFFT2Dr_f(a, threads=1):
    """c2r 2D FFT normalised by 1/grid^2, float32 (grid, grid) (:213-228)."""
    require_dtype(a, "complex64", "a")
    g = int(a.shape[0])
    if a.ndim != 2 or tuple(int(s) for s in a.shape) != (g, g // 2 + 1):
        raise ValueError("a must be (grid, grid//2+1), got %s" % (tuple(a.shape),))
    return _call_grid("pyl_fft2_c2r", a, (g, g), "float32", g)


class Pk_plane:
    """Power spectrum of a 2D field (Pk_library.pyx:435-511): k, Pk, Nmodes."""

    def __init__(self, delta, BoxSize, MAS="CIC", threads=1, verbose=True):
        start = time.time()
        require_dtype(delta, "float32", "delta")
        _check_square(delta, "delta")
        if verbose:
            print("\nComputing power spectrum of the field...")
        grid = int(delta.shape[0])
        kmax = frequencies_2D(BoxSize, grid)[4]
        k, Pk, Nmodes = np.zeros(kmax), np.zeros(kmax), np.zeros(kmax)
        ptrs = [ctypes.c_void_p(x.ctypes.data) for x in (k, Pk, Nmodes)]
        start2 = time.time()
        if is_cuda_tensor(delta):
            ctx = _native.context(delta.device.index or 0)
            src = delta.contiguous()
            torch_sync(src)
            rc = ctx.lib.pyl_pk_plane(ctx.ptr, dev_ptr(src), grid, float(BoxSize),
                                      MAS_function(MAS), *ptrs, _native.PYL_DEVICE_PTRS)
        else:
            ctx = _native.context(0)
            src = np.ascontiguousarray(delta.cpu().numpy() if is_tensor(delta) else delta)
            rc = ctx.lib.pyl_pk_plane(ctx.ptr, host_ptr(src), grid, float(BoxSize),
                                      MAS_function(MAS), *ptrs, 0)
        _raise_or_exit(ctx, rc)
        if verbose:
            print("Time to complete loop = %.2f" % (time.time() - start2))
        self.k, self.Pk, self.Nmodes = k, Pk, Nmodes
        if verbose:
            print("Time taken = %.2f seconds" % (time.time() - start))


class XPk:
    """Auto- and cross-power spectra of several fields (Pk_library.pyx:529-735).

    delta: list of (dims, dims, dims) float32 fields (numpy or CUDA tensors);
    MAS: list with the scheme of each field.  Attributes: k3D, Pk (kmax, 3,
    fields), XPk (kmax, 3, pairs), Nmodes3D; k1D, Pk1D, PkX1D, Nmodes1D; kpar,
    kper, Pk2D, PkX2D, Nmodes2D (pairs i < j in row order).
    """

    def __init__(self, delta, BoxSize, axis=2, MAS=None, threads=1):
        start = time.time()
        print("\nComputing power spectra of the fields...")
        dims = len(delta[0])
        fields = len(delta)
        for i in range(1, fields):
            if len(delta[i]) != dims:
                print("Fields have different grid sizes!!!")
                sys.exit()
        if MAS is None or len(MAS) != fields:
            raise ValueError("MAS must list one scheme per field")
        for i, d in enumerate(delta):
            require_dtype(d, "float32", "delta[%d]" % i)
            _check_cube(d, "delta[%d]" % i)
        if not 1 <= fields <= 8:
            raise ValueError("XPk takes 1 to 8 fields on the GPU")
        kmax, kmax_par, kmax_per = _native.pk_sizes(dims)
        X = fields * (fields - 1) // 2
        n2 = (kmax_par + 1) * (kmax_per + 1)
        arr = dict(k3D=np.zeros(kmax), Pk=np.zeros((kmax, 3, fields)),
                   XPk=np.zeros((kmax, 3, X)), Nmodes3D=np.zeros(kmax),
                   k1D=np.zeros(kmax_par), Pk1D=np.zeros((kmax_par, fields)),
                   PkX1D=np.zeros((kmax_par, X)), Nmodes1D=np.zeros(kmax_par),
                   kpar=np.zeros(n2), kper=np.zeros(n2), Pk2D=np.zeros((n2, fields)),
                   PkX2D=np.zeros((n2, X)), Nmodes2D=np.zeros(n2))
        out = _native.XPkOut(*[arr[k].ctypes.data for k in _native.XPkOut.names])
        mas = (ctypes.c_int * fields)(*[MAS_function(m) for m in MAS])
        cuda = [is_cuda_tensor(d) for d in delta]
        if any(cuda) and not all(cuda):
            raise ValueError("fields must be all host arrays or all CUDA tensors")
        if all(cuda):
            ctx = _native.context(delta[0].device.index or 0)
            srcs = [d.contiguous() for d in delta]
            for s in srcs:
                torch_sync(s)
            ptrs = (ctypes.c_void_p * fields)(*[s.data_ptr() for s in srcs])
            flags = _native.PYL_DEVICE_PTRS
        else:
            ctx = _native.context(0)
            srcs = [np.ascontiguousarray(d.cpu().numpy() if is_tensor(d) else d) for d in delta]
            ptrs = (ctypes.c_void_p * fields)(*[s.ctypes.data for s in srcs])
            flags = 0
        print("Time FFTS = %.2f" % (time.time() - start))
        start2 = time.time()
        rc = ctx.lib.pyl_xpk(ctx.ptr, ptrs, fields, dims, float(BoxSize), int(axis), mas,
                             ctypes.byref(out), flags)
        _raise_or_exit(ctx, rc)
        print("Time loop = %.2f" % (time.time() - start2))
        for k, v in arr.items():
            setattr(self, k, v)
        print("Time taken = %.2f seconds" % (time.time() - start))
