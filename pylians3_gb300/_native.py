"""ctypes binding of libpylgpu.so (the C ABI declared in include/pylgpu.h).

The library is built in-tree by ``pylians3_gb300.build_native``.  There is no
CPU fallback: if the shared library is missing or no CUDA device is present,
the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
SO_PATH = os.path.join(_PKG, "libpylgpu.so")

PYL_OK = 0
PYL_ERR_ARG = -1
PYL_ERR_CUDA = -2
PYL_ERR_OOM = -3
PYL_ERR_MODES = -4
PYL_ERR_TIMEOUT = -5
PYL_ERR_BUDGET = -6
PYL_ERR_UNSUPPORTED = -7
PYL_ERR_STATE = -8

MAS_CODE = {"NGP": 1, "CIC": 2, "TSC": 3, "PCS": 4}
PYL_DEVICE_PTRS = 0x01
PYL_COMPENSATED = 0x02
PYL_DEPOSIT_ATOMIC = 0x04
PYL_DEPOSIT_SORTED = 0x08
PYL_SORT_TWO_PASS = 0x10
PYL_SORT_FRONTIER = 0x20
PYL_DEPOSIT_FLOAT = 0x40
PYL_NO_GRAPH = 0x80
PYL_SORT_EXACT = 0x100
PYL_PK_1D, PYL_PK_2D, PYL_PK_PHASE, PYL_PK_ALL = 0x01, 0x02, 0x04, 0x07

# every symbol include/pylgpu.h declares (checked by the tests)
EXPORTS = (
    "pyl_ctx_create", "pyl_ctx_destroy", "pyl_ctx_set_stream", "pyl_ctx_get_stream",
    "pyl_synchronize", "pyl_last_error", "pyl_ctx_workspace_bytes", "pyl_ctx_trim",
    "pyl_ctx_launch_count", "pyl_ctx_last_sort", "pyl_host_alloc", "pyl_host_free", "pyl_ma", "pyl_ma_f64",
    "pyl_fft_r2c", "pyl_fft_c2r", "pyl_pk_sizes", "pyl_pk", "pyl_pk_particles",
    "pyl_ctx_set_timing", "pyl_ctx_stage_times", "pyl_stage_name", "pyl_pk_noalloc",
    "pyl_pk_particles_enqueue", "pyl_pk_query", "pyl_pk_collect",
    "pyl_correct_mas", "pyl_fft2_r2c", "pyl_fft2_c2r", "pyl_pk_plane", "pyl_cic_interp",
    "pyl_xpk", "pyl_rsd", "pyl_pk_batch", "pyl_set_tile_shape", "pyl_get_tile_shape",
)


class PylError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libpylgpu error %d: %s" % (code, msg))
        self.code = code


class PkOut(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in (
        "k3D", "Pk", "Nmodes3D", "k1D", "Pk1D", "Nmodes1D", "kpar", "kper",
        "Pk2D", "Nmodes2D", "Pkphase")]


class PkRequest(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_void_p), ("n", ctypes.c_int64), ("W", ctypes.c_void_p),
                ("dims", ctypes.c_int), ("BoxSize", ctypes.c_float), ("mas_deposit", ctypes.c_int),
                ("axis", ctypes.c_int), ("mas_window", ctypes.c_int), ("what", ctypes.c_int)]


class XPkOut(ctypes.Structure):
    names = ("k3D", "Pk", "XPk", "Nmodes3D", "k1D", "Pk1D", "PkX1D", "Nmodes1D",
             "kpar", "kper", "Pk2D", "PkX2D", "Nmodes2D")
    _fields_ = [(name, ctypes.c_void_p) for name in names]


_lib = None
_lock = threading.Lock()


def load():
    """Load libpylgpu.so and declare its signatures (no GPU needed)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(SO_PATH):
            raise ImportError(
                "libpylgpu.so is not built (expected at %s); run "
                "`python -m pylians3_gb300.build_native`" % SO_PATH)
        lib = ctypes.CDLL(SO_PATH)
        vp, i32, i64, f32, f64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                  ctypes.c_float, ctypes.c_double)
        sz = ctypes.c_size_t
        sig = {
            "pyl_ctx_create": [ctypes.POINTER(vp), i32, vp],
            "pyl_ctx_destroy": [vp],
            "pyl_ctx_set_stream": [vp, vp],
            "pyl_ctx_get_stream": [vp, ctypes.POINTER(vp)],
            "pyl_synchronize": [vp],
            "pyl_ctx_workspace_bytes": [vp, ctypes.POINTER(sz)],
            "pyl_ctx_trim": [vp],
            "pyl_ctx_launch_count": [vp, ctypes.POINTER(i64)],
            "pyl_ctx_last_sort": [vp, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_uint)],
            "pyl_ctx_set_timing": [vp, i32],
            "pyl_ctx_stage_times": [vp, ctypes.POINTER(f64), ctypes.POINTER(i64), i32, i32],
            "pyl_host_alloc": [ctypes.POINTER(vp), sz],
            "pyl_host_free": [vp],
            "pyl_ma": [vp, vp, i64, i32, vp, vp, i32, f32, i32, i32, i32],
            "pyl_ma_f64": [vp, vp, i64, i32, vp, vp, i32, f32, i32, i32, i32],
            "pyl_fft_r2c": [vp, vp, vp, i32, i32],
            "pyl_fft_c2r": [vp, vp, vp, i32, i32],
            "pyl_pk_sizes": [i32, ctypes.POINTER(i32), ctypes.POINTER(i32),
                             ctypes.POINTER(i32)],
            "pyl_pk": [vp, vp, i32, f64, i32, i32, i32, ctypes.POINTER(PkOut), i32],
            "pyl_pk_noalloc": [vp, vp, i32, f64, i32, i32, i32, ctypes.POINTER(PkOut)],
            "pyl_pk_particles": [vp, vp, i64, vp, i32, f32, i32, i32, i32, i32,
                                 ctypes.POINTER(PkOut), i32],
            "pyl_pk_particles_enqueue": [vp, vp, i64, vp, i32, f32, i32, i32, i32, i32, i32],
            "pyl_pk_query": [vp],
            "pyl_pk_collect": [vp, ctypes.POINTER(PkOut), i32],
            "pyl_correct_mas": [vp, vp, vp, i32, i32, i32],
            "pyl_fft2_r2c": [vp, vp, vp, i32, i32],
            "pyl_fft2_c2r": [vp, vp, vp, i32, i32],
            "pyl_pk_plane": [vp, vp, i32, f64, i32, vp, vp, vp, i32],
            "pyl_cic_interp": [vp, vp, i32, f32, vp, i64, vp, i32],
            "pyl_xpk": [vp, vp, i32, i32, f64, i32, vp, ctypes.POINTER(XPkOut), i32],
            "pyl_rsd": [vp, vp, vp, i64, f32, f32, f32, i32, i32],
            "pyl_pk_batch": [vp, ctypes.POINTER(PkRequest), i32, ctypes.POINTER(PkOut), i32],
            "pyl_set_tile_shape": [i32, i32, i32, i32, i32, i32],
            "pyl_get_tile_shape": [i32, i32] + [ctypes.POINTER(i32)] * 4,
        }
        for name, args in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        lib.pyl_last_error.argtypes = [vp]
        lib.pyl_last_error.restype = ctypes.c_char_p
        lib.pyl_stage_name.argtypes = [i32]
        lib.pyl_stage_name.restype = ctypes.c_char_p
        _lib = lib
        return lib


class Context:
    """Owns one pyl_ctx (device workspaces, FFT plans, mode tables, a stream)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load()
        self.ptr = ctypes.c_void_p()
        rc = self.lib.pyl_ctx_create(ctypes.byref(self.ptr), int(device),
                                     ctypes.c_void_p(stream) if stream else None)
        if rc != PYL_OK:
            raise PylError(rc, "cannot create a context on CUDA device %d" % device)
        self.device = device

    def check(self, rc):
        if rc != PYL_OK:
            msg = self.lib.pyl_last_error(self.ptr)
            raise PylError(rc, msg.decode() if msg else "")
        return rc

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        self.check(self.lib.pyl_ctx_get_stream(self.ptr, ctypes.byref(s)))
        return s.value or 0

    def set_stream(self, stream: int | None):
        self.check(self.lib.pyl_ctx_set_stream(
            self.ptr, ctypes.c_void_p(stream) if stream else None))

    def synchronize(self):
        self.check(self.lib.pyl_synchronize(self.ptr))

    def launches(self) -> int:
        v = ctypes.c_int64()
        self.check(self.lib.pyl_ctx_launch_count(self.ptr, ctypes.byref(v)))
        return v.value

    def last_sort(self):
        """(count_free, spilled) of the last collected particles request:
        count_free 1 = the sort without a counting pass, 0 = the exact
        counting sort, -1 = no sorted deposit."""
        cf, sp = ctypes.c_int(), ctypes.c_uint()
        self.check(self.lib.pyl_ctx_last_sort(self.ptr, ctypes.byref(cf), ctypes.byref(sp)))
        return cf.value, sp.value

    def set_timing(self, on: bool):
        self.check(self.lib.pyl_ctx_set_timing(self.ptr, 1 if on else 0))

    def stage_times(self, reset: bool = False) -> dict:
        """{stage name: (total ms, launches)} of the timed stages."""
        n = 16
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int64 * n)()
        k = self.lib.pyl_ctx_stage_times(self.ptr, ms, cnt, n, 1 if reset else 0)
        if k < 0:
            self.check(k)
        return {self.lib.pyl_stage_name(i).decode(): (ms[i], cnt[i])
                for i in range(k) if cnt[i]}

    def workspace_bytes(self) -> int:
        v = ctypes.c_size_t()
        self.check(self.lib.pyl_ctx_workspace_bytes(self.ptr, ctypes.byref(v)))
        return v.value

    def trim(self):
        self.check(self.lib.pyl_ctx_trim(self.ptr))

    def close(self):
        if self.ptr:
            self.lib.pyl_ctx_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_contexts: dict = {}


def context(device: int = 0) -> Context:
    """The process-wide default context of a device."""
    with _lock:
        c = _contexts.get(device)
    if c is None:
        c = Context(device)
        with _lock:
            _contexts.setdefault(device, c)
            c = _contexts[device]
    return c


def pk_sizes(dims: int):
    lib = load()
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = lib.pyl_pk_sizes(int(dims), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    if rc != PYL_OK:
        raise PylError(rc, "bad dims %r" % dims)
    return a.value, b.value, c.value


class PinnedArray:
    """A numpy array in pinned (page-locked) host memory from cudaHostAlloc."""

    def __init__(self, shape, dtype=np.float32):
        lib = load()
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        self._ptr = ctypes.c_void_p()
        rc = lib.pyl_host_alloc(ctypes.byref(self._ptr), max(1, nbytes))
        if rc != PYL_OK:
            raise PylError(rc, "pinned allocation of %d bytes failed" % nbytes)
        buf = (ctypes.c_byte * max(1, nbytes)).from_address(self._ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
        self._lib = lib

    def __del__(self):
        try:
            if self._ptr:
                self._lib.pyl_host_free(self._ptr)
        except Exception:
            pass


class _PinnedNDArray(np.ndarray):
    """ndarray that keeps its pinned allocation alive (views keep it via .base)."""
    _pinned_holder = None


def pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    """numpy array backed by pinned host memory (freed with the array)."""
    holder = PinnedArray(shape, dtype)
    arr = holder.array.view(_PinnedNDArray)
    arr._pinned_holder = holder
    return arr
