"""CPU oracle for the Pylians3 density-field + power-spectrum hot path.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only as the
checker (or the timed CPU baseline) -- never as the thing measured or shipped.
The product package ``pylians3_gb300`` never imports it.

It restates, with the reference's floating-point types:
  * ``MA`` / ``NGP`` ... ``PCSW``   -- library/MAS_library/MAS_library.pyx:57-545
    (loops in oracle/pyl_oracle.c, dispatch and 2D renormalisation here, :57-112)
  * ``deposit_omp``                -- library/MAS_library/MAS_c.c:8-266
  * ``Pk``                         -- library/Pk_library/Pk_library.pyx:263-418
    (mode loop in C; normalisation here, :384-418)
  * ``FFT3Dr_f`` / ``IFFT3Dr_f``   -- Pk_library.pyx:117-130, :149-162.  The
    reference calls pyFFTW (FFTW3f), which is not installed here; the
    oracle uses scipy.fft (pocketfft) in float32 with the same conventions
    (forward unnormalised, inverse normalised by 1/N^3).
  * ``MA_f64`` / ``Pk_f64``        -- a float64 restatement (grid, FFT, window
    and sums all in float64), the precision oracle.

Parity of this restatement with the compiled reference is pinned by the
golden vectors in tests/golden/ (see tests/test_oracle_golden.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liborc.so")
_SRC = os.path.join(_HERE, "pyl_oracle.c")

_lib = None


def build(force: bool = False) -> str:
    """Compile pyl_oracle.c into oracle/_build/liborc.so (gcc, OpenMP).

    ``-ffp-contract=off`` keeps every float operation separately rounded, as
    the reference's C semantics state them.
    """
    os.makedirs(_BUILD, exist_ok=True)
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= os.path.getmtime(_SRC)):
        return _SO
    tmp = _SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-o", tmp, _SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _SO)
    return _SO


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(_SO)
    fp = ctypes.c_void_p
    for name in ("orc_ngp", "orc_cic", "orc_tsc", "orc_pcs",
                 "orc_ngp_d", "orc_cic_d", "orc_tsc_d", "orc_pcs_d"):
        f = getattr(lib, name)
        f.argtypes = [fp, ctypes.c_long, ctypes.c_int, fp, fp, ctypes.c_int,
                      ctypes.c_float]
        f.restype = None
    lib.orc_deposit_omp.argtypes = [ctypes.c_int, fp, ctypes.c_long, fp, fp,
                                    ctypes.c_int, ctypes.c_float, ctypes.c_int]
    lib.orc_deposit_omp.restype = None
    lib.orc_deposit_d_omp.argtypes = lib.orc_deposit_omp.argtypes
    lib.orc_deposit_d_omp.restype = None
    lib.orc_pk_bin.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.c_int, ctypes.c_int] + [fp] * 9
    lib.orc_pk_bin.restype = None
    lib.orc_pk_bin_d.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 fp, fp, fp]
    lib.orc_pk_bin_d.restype = None
    lib.orc_pk_bin_mt.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int] + [fp] * 9
    lib.orc_pk_bin_mt.restype = None
    lib.orc_pk_bin_d_mt.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, fp, fp, fp]
    lib.orc_pk_bin_d_mt.restype = None
    lib.orc_mode_counts.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [fp] * 5
    lib.orc_mode_counts.restype = None
    lib.orc_num_threads.restype = ctypes.c_int
    _lib = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data


# --------------------------------------------------------------------------
# Mass assignment (MAS_library.pyx:57-112)
# --------------------------------------------------------------------------
_MAS_FN = {"NGP": "orc_ngp", "CIC": "orc_cic", "TSC": "orc_tsc", "PCS": "orc_pcs"}


def _deposit(MAS, pos, grid, BoxSize, W, f64=False):
    lib = _load()
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    if W is not None:
        W = np.ascontiguousarray(W, dtype=np.float32)
    dims = grid.shape[0]
    assert grid.flags.c_contiguous
    fn = getattr(lib, _MAS_FN[MAS] + ("_d" if f64 else ""))
    fn(pos.ctypes.data, pos.shape[0], pos.shape[1], _ptr(W), grid.ctypes.data,
       dims, float(np.float32(BoxSize)))


def MA(pos, number, BoxSize, MAS="CIC", W=None, verbose=False,
       renormalize_2D=True):
    """Restatement of MA (MAS_library.pyx:57-112): accumulates into `number`."""
    coord, coord_aux = pos.shape[1], number.ndim
    if coord != coord_aux:
        print("pos have %d dimensions and the density %d!!!" % (coord, coord_aux))
        sys.exit()
    if MAS not in _MAS_FN:
        print("option not valid!!!")
        sys.exit()
    f64 = number.dtype == np.float64
    if coord == 3:
        _deposit(MAS, pos, number, BoxSize, W, f64)
    else:
        number2 = np.expand_dims(number, axis=2)
        _deposit(MAS, pos, number2, BoxSize, W, f64)
        if renormalize_2D and MAS != "NGP":
            number2 /= {"CIC": 2.0, "TSC": 3.0, "PCS": 4.0}[MAS]


def MA_f64(pos, dims, BoxSize, MAS="CIC", W=None, threads=1):
    """Float64 grid deposit (precision oracle); weights computed as the
    reference computes them, accumulation in float64 (cf. CICW_d :229-266).
    threads != 1: the same taps added on all cores (threads=0) or that many
    (3D positions only)."""
    grid = np.zeros((dims, dims, dims), np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    if threads != 1 and pos.shape[1] == 3:
        lib = _load()
        Wc = None if W is None else np.ascontiguousarray(W, dtype=np.float32)
        lib.orc_deposit_d_omp({"NGP": 1, "CIC": 2, "TSC": 3, "PCS": 4}[MAS], pos.ctypes.data,
                              pos.shape[0], _ptr(Wc), grid.ctypes.data, dims,
                              float(np.float32(BoxSize)), int(threads))
        return grid
    _deposit(MAS, pos, grid, BoxSize, W, f64=True)
    return grid


def deposit_omp(MAS, pos, grid, BoxSize, W=None, threads=0):
    """OpenMP atomic deposit (MAS_c.c:8-266), 3D; threads=0 uses all cores."""
    lib = _load()
    mas = {"NGP": 1, "CIC": 2, "TSC": 3, "PCS": 4}[MAS]
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    lib.orc_deposit_omp(mas, pos.ctypes.data, pos.shape[0], _ptr(W),
                        grid.ctypes.data, grid.shape[0],
                        float(np.float32(BoxSize)), int(threads))


def num_threads() -> int:
    return int(_load().orc_num_threads())


# --------------------------------------------------------------------------
# Power spectrum (Pk_library.pyx:56-130, 263-418)
# --------------------------------------------------------------------------
def frequencies(BoxSize, dims):
    """Pk_library.pyx:56-61."""
    kF = 2.0 * np.pi / BoxSize
    middle = dims // 2
    kN = middle * kF
    kmax_par = middle
    kmax_per = int(np.sqrt(middle ** 2 + middle ** 2))
    kmax = int(np.sqrt(middle ** 2 + middle ** 2 + middle ** 2))
    return kF, kN, kmax_par, kmax_per, kmax


def MAS_function(MAS):
    """Pk_library.pyx:72-78."""
    return {"NGP": 1, "CIC": 2, "TSC": 3, "PCS": 4}.get(MAS, 0)


def expected_modes(dims):
    """Independent-mode count asserted by check_number_modes (:87-99)."""
    own = 1 if dims % 2 == 1 else 8
    return (dims ** 3 - own) // 2 + own


def FFT3Dr_f(a, threads=1):
    """r2c over (0,1,2), unnormalised, complex64 (Pk_library.pyx:117-130)."""
    import scipy.fft as sf
    return sf.rfftn(np.asarray(a, np.float32), axes=(0, 1, 2),
                    workers=max(1, int(threads))).astype(np.complex64, copy=False)


def IFFT3Dr_f(a, threads=1):
    """c2r normalised by 1/N^3, float32 (Pk_library.pyx:149-162)."""
    import scipy.fft as sf
    dims = a.shape[0]
    return sf.irfftn(np.asarray(a, np.complex64), s=(dims, dims, dims),
                     axes=(0, 1, 2), workers=max(1, int(threads))
                     ).astype(np.float32, copy=False)


class Pk:
    """Restatement of class Pk (Pk_library.pyx:263-418)."""

    def __init__(self, delta, BoxSize, axis=2, MAS="CIC", threads=1,
                 verbose=False, delta_k=None, rows=None, bin_threads=1):
        """bin_threads != 1 runs the mode loop's rows on that many cores (0:
        all), private float64 sums added at the end: the same per-mode
        values, another order of the float64 sums (large test grids)."""
        lib = _load()
        dims = len(delta) if delta is not None else delta_k.shape[0]
        kF, kN, kmax_par, kmax_per, kmax = frequencies(BoxSize, dims)
        MAS_index = MAS_function(MAS)
        if delta_k is None:
            delta_k = FFT3Dr_f(delta, threads)
        delta_k = np.ascontiguousarray(delta_k, np.complex64)
        k1D = np.zeros(kmax_par + 1)
        Pk1D = np.zeros(kmax_par + 1)
        N1D = np.zeros(kmax_par + 1)
        Pk2D = np.zeros((kmax_par + 1) * (kmax_per + 1))
        N2D = np.zeros((kmax_par + 1) * (kmax_per + 1))
        k3D = np.zeros(kmax + 1)
        Pk3D = np.zeros((kmax + 1, 3))
        Pkphase = np.zeros(kmax + 1)
        N3D = np.zeros(kmax + 1)
        r0, r1 = (0, dims) if rows is None else rows
        outs = (k1D.ctypes.data, Pk1D.ctypes.data, N1D.ctypes.data,
                Pk2D.ctypes.data, N2D.ctypes.data, k3D.ctypes.data,
                Pk3D.ctypes.data, Pkphase.ctypes.data, N3D.ctypes.data)
        if bin_threads != 1 and rows is None:
            lib.orc_pk_bin_mt(delta_k.ctypes.data, dims, int(axis), MAS_index,
                              int(bin_threads), *outs)
        else:
            lib.orc_pk_bin(delta_k.ctypes.data, dims, int(axis), MAS_index, r0, r1, *outs)
        self.raw = dict(k3D=k3D.copy(), Pk3D=Pk3D.copy(), N3D=N3D.copy())
        if rows is not None:          # bounded sample for timing: no finalisation
            return
        # --- normalisation, :384-418 ---
        k1D, N1D, Pk1D = k1D[1:], N1D[1:], Pk1D[1:]
        with np.errstate(divide="ignore", invalid="ignore"):
            Pk1D = Pk1D * (BoxSize / dims ** 2) ** 3
            k1D = (k1D / N1D) * kF
            kmaxper = np.sqrt(kN ** 2 - k1D ** 2)
            Pk1D = Pk1D * (np.pi * kmaxper ** 2 / N1D) / (2.0 * np.pi) ** 2
        self.k1D, self.Pk1D, self.Nmodes1D = k1D, Pk1D, N1D
        kp = np.arange(kmax_par + 1)
        kq = np.arange(kmax_per + 1)
        self.kpar = np.tile(0.5 * (2 * kp + 1) * kF, kmax_per + 1)
        self.kper = np.repeat(0.5 * (2 * kq + 1) * kF, kmax_par + 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            self.Pk2D = Pk2D * (BoxSize / dims ** 2) ** 3 / N2D
        self.Nmodes2D = N2D
        if int(np.sum(N3D)) != expected_modes(dims):
            print("WARNING: Not all modes counted")
            sys.exit()
        k3D, N3D, Pk3D, Pkphase = k3D[1:], N3D[1:], Pk3D[1:, :], Pkphase[1:]
        unit = (BoxSize / dims ** 2) ** 3
        self.k3D = (k3D / N3D) * kF
        P = np.empty_like(Pk3D)
        P[:, 0] = (Pk3D[:, 0] / N3D) * unit
        P[:, 1] = (Pk3D[:, 1] * 5.0 / N3D) * unit
        P[:, 2] = (Pk3D[:, 2] * 9.0 / N3D) * unit
        self.Pk = P
        self.Pkphase = (Pkphase / N3D) * unit
        self.Nmodes3D = N3D


def mode_counts(dims, axis=2, threads=0):
    """Mode counts and k sums of class Pk without the data (the index part of
    Pk_library.pyx:311-378 on all cores) with the reference's finalisation
    of k3D / k1D (:384-409): returns dict k3D, Nmodes3D (DC bin dropped),
    k1D, Nmodes1D, Nmodes2D, as the attributes of class Pk for BoxSize 2 pi
    (kF = 1)."""
    lib = _load()
    kF, kN, kmax_par, kmax_per, kmax = frequencies(2.0 * np.pi, dims)
    k1D = np.zeros(kmax_par + 1)
    N1D = np.zeros(kmax_par + 1)
    N2D = np.zeros((kmax_par + 1) * (kmax_per + 1))
    k3D = np.zeros(kmax + 1)
    N3D = np.zeros(kmax + 1)
    lib.orc_mode_counts(int(dims), int(axis), int(threads), k1D.ctypes.data, N1D.ctypes.data,
                        N2D.ctypes.data, k3D.ctypes.data, N3D.ctypes.data)
    if int(np.sum(N3D)) != expected_modes(dims):
        raise AssertionError("oracle mode count %d != %d" % (int(np.sum(N3D)), expected_modes(dims)))
    with np.errstate(divide="ignore", invalid="ignore"):
        return dict(k3D=(k3D[1:] / N3D[1:]) * kF, Nmodes3D=N3D[1:],
                    k1D=(k1D[1:] / N1D[1:]) * kF, Nmodes1D=N1D[1:], Nmodes2D=N2D)


class Pk_f64:
    """Float64 precision oracle: float64 FFT of a float64 grid, window and
    sums in float64 (k3D, Pk[:,0:3], Nmodes3D as class Pk)."""

    def __init__(self, delta, BoxSize, axis=2, MAS="CIC", threads=1, bin_threads=1):
        import scipy.fft as sf
        lib = _load()
        dims = delta.shape[0]
        kF, kN, kmax_par, kmax_per, kmax = frequencies(BoxSize, dims)
        dk = np.ascontiguousarray(
            sf.rfftn(np.asarray(delta, np.float64), axes=(0, 1, 2),
                     workers=max(1, int(threads))), np.complex128)
        k3D = np.zeros(kmax + 1)
        Pk3D = np.zeros((kmax + 1, 3))
        N3D = np.zeros(kmax + 1)
        if bin_threads != 1:
            lib.orc_pk_bin_d_mt(dk.ctypes.data, dims, int(axis), MAS_function(MAS),
                                int(bin_threads), k3D.ctypes.data, Pk3D.ctypes.data,
                                N3D.ctypes.data)
        else:
            lib.orc_pk_bin_d(dk.ctypes.data, dims, int(axis), MAS_function(MAS),
                             k3D.ctypes.data, Pk3D.ctypes.data, N3D.ctypes.data)
        unit = (BoxSize / dims ** 2) ** 3
        k3D, N3D, Pk3D = k3D[1:], N3D[1:], Pk3D[1:]
        self.k3D = k3D / N3D * kF
        self.Pk = np.stack([Pk3D[:, 0] / N3D * unit, Pk3D[:, 1] * 5.0 / N3D * unit,
                            Pk3D[:, 2] * 9.0 / N3D * unit], axis=1)
        self.Nmodes3D = N3D


# --------------------------------------------------------------------------
# Rows around the spectrum (numpy restatements; small grids)
# --------------------------------------------------------------------------
def _window_1d(dims, MAS_index, nonneg=False):
    """MAS_correction(pi k / dims, p) in double for every index (Pk_library.pyx:83-84)."""
    middle = dims // 2
    idx = np.arange(dims // 2 + 1 if nonneg else dims)
    k = idx if nonneg else np.where(idx > middle, idx - dims, idx)
    x = (np.pi / dims) * k
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where(x == 0.0, 1.0, np.power(x / np.sin(np.where(x == 0, 1.0, x)), MAS_index))
    return k, w


def _independent(kx, ky, kz, dims):
    """Hermitian half-space selection of the mode loops (Pk_library.pyx:324-327)."""
    middle, even = dims // 2, dims % 2 == 0
    plane = (kz == 0) | ((kz == middle) & even)
    edge = (kx == 0) | ((kx == middle) & even)
    return ~(plane & ((kx < 0) | (edge & (ky < 0))))


def correct_MAS(delta, BoxSize, MAS="CIC", threads=1):
    """Restatement of correct_MAS (Pk_library.pyx:1882-1939)."""
    dims = delta.shape[0]
    p = MAS_function(MAS)
    dk = FFT3Dr_f(delta, threads)
    kx, wx = _window_1d(dims, p)
    kz, wz = _window_1d(dims, p, nonneg=True)
    KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
    fac = ((wx[:, None, None] * wx[None, :, None]) * wz[None, None, :]).astype(np.float32)
    m = _independent(KX, KY, KZ, dims)
    dk[m] = dk[m] * fac[m]
    return IFFT3Dr_f(dk, threads)


def FFT2Dr_f(a, threads=1):
    """r2c over (0,1), unnormalised, complex64 (Pk_library.pyx:181-196)."""
    import scipy.fft as sf
    return sf.rfftn(np.asarray(a, np.float32), axes=(0, 1),
                    workers=max(1, int(threads))).astype(np.complex64, copy=False)


def IFFT2Dr_f(a, threads=1):
    """c2r normalised by 1/N^2, float32 (Pk_library.pyx:213-228)."""
    import scipy.fft as sf
    g = a.shape[0]
    return sf.irfftn(np.asarray(a, np.complex64), s=(g, g), axes=(0, 1),
                     workers=max(1, int(threads))).astype(np.float32, copy=False)


class Pk_plane:
    """Restatement of class Pk_plane (Pk_library.pyx:435-511): k, Pk, Nmodes."""

    def __init__(self, delta, BoxSize, MAS="CIC", threads=1, verbose=False):
        grid = delta.shape[0]
        middle, even = grid // 2, grid % 2 == 0
        kF = 2.0 * np.pi / BoxSize
        kmax = int(np.sqrt(middle ** 2 + middle ** 2))
        p = MAS_function(MAS)
        dk = FFT2Dr_f(delta, threads)
        kx, wx = _window_1d(grid, p)
        ky, wy = _window_1d(grid, p, nonneg=True)
        KX, KY = np.meshgrid(kx, ky, indexing="ij")
        keep = ~(((KY == 0) | ((KY == middle) & even)) & (KX < 0))
        k = np.sqrt((KX * KX + KY * KY).astype(np.float64))
        kidx = k.astype(np.int64)
        fac = (wx[:, None] * wy[None, :]).astype(np.float32)
        v = (dk * fac)[keep]
        d2 = v.real.astype(np.float64) ** 2 + v.imag.astype(np.float64) ** 2
        ki = kidx[keep]
        N = np.bincount(ki, minlength=kmax + 1).astype(np.float64)
        ks = np.bincount(ki, weights=k[keep], minlength=kmax + 1)
        P = np.bincount(ki, weights=d2, minlength=kmax + 1)
        if int(N.sum()) != (grid * grid - (1 if grid % 2 else 4)) // 2 + (1 if grid % 2 else 4):
            raise RuntimeError("not all modes counted")
        N, ks, P = N[1:], ks[1:], P[1:]
        self.k = ks / N * kF
        self.Pk = P / N * (BoxSize / grid ** 2) ** 2
        self.Nmodes = N


class XPk:
    """Restatement of class XPk (Pk_library.pyx:529-735), vectorised over the
    modes (float64 sums in another order than the reference's loop)."""

    def __init__(self, delta, BoxSize, axis=2, MAS=None, threads=1):
        fields = len(delta)
        dims = delta[0].shape[0]
        middle = dims // 2
        kF, kN, kmax_par, kmax_per, kmax = frequencies(BoxSize, dims)
        kx, _ = _window_1d(dims, 0)
        kz, _ = _window_1d(dims, 0, nonneg=True)
        KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
        keep = _independent(KX, KY, KZ, dims)
        KX, KY, KZ = KX[keep], KY[keep], KZ[keep]
        k = np.sqrt((KX * KX + KY * KY + KZ * KZ).astype(np.float64))
        kidx = k.astype(np.int64)
        kpar = {0: KX, 1: KY}.get(axis, KZ)
        kper2 = {0: KY * KY + KZ * KZ, 1: KX * KX + KZ * KZ}.get(axis, KX * KX + KY * KY)
        kper = np.sqrt(kper2.astype(np.float64)).astype(np.int64)
        with np.errstate(invalid="ignore", divide="ignore"):
            mu = np.where(k == 0, 0.0, kpar / np.where(k == 0, 1.0, k))
        mu2 = mu * mu
        val1 = (3.0 * mu2 - 1.0) / 2.0
        val2 = (35.0 * mu2 * mu2 - 30.0 * mu2 + 3.0) / 8.0
        apar = np.abs(kpar)
        in1 = k <= middle
        i2 = (kmax_par + 1) * kper + apar
        re, im = [], []
        for f, m in zip(delta, MAS):
            p = MAS_function(m)
            _, wx = _window_1d(dims, p)
            _, wz = _window_1d(dims, p, nonneg=True)
            fac = ((wx[:, None, None] * wx[None, :, None]) * wz[None, None, :]).astype(np.float32)
            v = (FFT3Dr_f(f, threads) * fac)[keep]
            re.append(v.real.astype(np.float64))
            im.append(v.imag.astype(np.float64))
        series = [re[i] * re[i] + im[i] * im[i] for i in range(fields)]
        for i in range(fields):
            for j in range(i + 1, fields):
                series.append(re[i] * re[j] + im[i] * im[j])
        n2d = (kmax_par + 1) * (kmax_per + 1)

        def binned(idx, w, n):
            return np.bincount(idx, weights=w, minlength=n)

        N3 = binned(kidx, None, kmax + 1).astype(np.float64)
        k3 = binned(kidx, k, kmax + 1)
        N1 = binned(apar[in1], None, kmax_par + 1).astype(np.float64)
        k1 = binned(apar[in1], apar[in1].astype(np.float64), kmax_par + 1)
        N2 = binned(i2, None, n2d).astype(np.float64)
        S = len(series)
        P3 = np.zeros((kmax + 1, 3, S))
        P1 = np.zeros((kmax_par + 1, S))
        P2 = np.zeros((n2d, S))
        for s, d2 in enumerate(series):
            P3[:, 0, s] = binned(kidx, d2, kmax + 1)
            P3[:, 1, s] = binned(kidx, d2 * val1, kmax + 1)
            P3[:, 2, s] = binned(kidx, d2 * val2, kmax + 1)
            P1[:, s] = binned(apar[in1], d2[in1], kmax_par + 1)
            P2[:, s] = binned(i2, d2, n2d)
        if int(N3.sum()) != expected_modes(dims):
            raise RuntimeError("not all modes counted")
        fact = (BoxSize / dims ** 2) ** 3
        k1D = k1[1:] / N1[1:] * kF
        kmaxper = np.sqrt(kN ** 2 - k1D ** 2)
        P1 = P1[1:] * fact
        P1 = P1 * (np.pi * kmaxper[:, None] ** 2 / N1[1:, None]) / (2.0 * np.pi) ** 2
        self.k1D, self.Nmodes1D = k1D, N1[1:]
        self.Pk1D, self.PkX1D = P1[:, :fields], P1[:, fields:]
        pp = np.arange(kmax_par + 1)
        qq = np.arange(kmax_per + 1)
        idx2 = (kmax_par + 1) * qq[None, :] + pp[:, None]
        self.kpar = np.zeros(n2d)
        self.kper = np.zeros(n2d)
        self.kpar[idx2] = (0.5 * (pp + pp + 1) * kF)[:, None]
        self.kper[idx2] = (0.5 * (qq + qq + 1) * kF)[None, :]
        P2 = P2 * fact / N2[:, None]
        self.Pk2D, self.PkX2D, self.Nmodes2D = P2[:, :fields], P2[:, fields:], N2
        N3, k3, P3 = N3[1:], k3[1:], P3[1:]
        self.k3D = k3 / N3 * kF
        scale = np.array([1.0, 5.0, 9.0])[None, :, None]
        P3 = (P3 * scale / N3[:, None, None]) * fact
        self.Pk, self.XPk, self.Nmodes3D = P3[:, :, :fields], P3[:, :, fields:], N3


def CIC_interp(density, BoxSize, pos, den):
    """Restatement of CIC_interp (MAS_library.pyx:558-599), float32 steps in
    the written order; writes den in place."""
    dims = density.shape[0]
    inv = np.float32(np.float32(dims) / np.float32(BoxSize))
    pos = np.asarray(pos, np.float32)
    dist = pos * inv
    c = dist.astype(np.int32)
    u = (dist - c.astype(np.float32)).astype(np.float32)
    d = (np.float32(1.0) - u).astype(np.float32)
    lo = c % dims
    hi = (lo + 1) % dims
    g = density
    terms = [
        (lo, lo, lo, d, d, d), (lo, lo, hi, d, d, u), (lo, hi, lo, d, u, d), (lo, hi, hi, d, u, u),
        (hi, lo, lo, u, d, d), (hi, lo, hi, u, d, u), (hi, hi, lo, u, u, d), (hi, hi, hi, u, u, u)]
    s = None
    for ix, iy, iz, a, b, cc in terms:
        t = g[ix[:, 0], iy[:, 1], iz[:, 2]] * a[:, 0] * b[:, 1] * cc[:, 2]
        s = t if s is None else (s + t).astype(np.float32)
    den[:len(s)] = s


def pos_redshift_space(pos, vel, BoxSize, Hubble, redshift, axis):
    """Restatement of pos_redshift_space (redshift_space_library.pyx:29-50),
    in place, float32 steps as written."""
    factor = np.float32((1.0 + float(np.float32(redshift))) / float(np.float32(Hubble)))
    box = np.float32(BoxSize)
    p = (pos[:, axis] + vel[:, axis] * factor).astype(np.float32)
    neg = p < 0
    while neg.any():
        p[neg] = p[neg] + box
        neg = p < 0
    big = p > box
    p[big] = np.fmod(p[big], box)
    pos[:, axis] = p
