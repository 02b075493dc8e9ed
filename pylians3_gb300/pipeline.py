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
    "auto": 0,                                   # fixed-point tiles (PCS: where 24 bits fit)
    "float": _native.PYL_DEPOSIT_FLOAT,          # float32 shared atomics
    "compensated": _native.PYL_COMPENSATED,      # float32 + TwoSum error grid
}


def power_spectrum(pos, dims, BoxSize, MAS="CIC", axis=2, W=None, window=None,
                   what=0, ctx=None, deposit="auto", sort="auto"):
    """Spectrum of the particles' overdensity field on a dims^3 grid.

    pos: (n, 3) float32 numpy array (pinned memory copies fastest, see
    ``pinned_empty``) or torch CUDA tensor.  MAS is the deposit scheme;
    ``window`` the window to deconvolve (default: the same as MAS).
    ``what``: extra outputs (Pk_library.PK_1D | PK_2D | PK_PHASE).
    ``deposit``: accumulation of the grid, one of DEPOSIT_FLAGS.
    ``sort``: "auto" takes the count-free tile sort where the previous
    request of the same dims, scheme and weighting allows it; "exact" always
    counts first.
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
    if sort not in ("auto", "exact"):
        raise ValueError('sort must be "auto" or "exact"')
    if sort == "exact":
        dflags |= _native.PYL_SORT_EXACT
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


_pools: dict = {}


def _pool(device, depth):
    """Contexts (each with its own stream and workspaces) kept per device."""
    key = (device, depth)
    if key not in _pools:
        _pools[key] = [_native.Context(device) for _ in range(depth)]
    return _pools[key]


def power_spectra(pos_sets, dims, BoxSize, MAS="CIC", axis=2, W_sets=None, window=None,
                  what=0, deposit="auto", depth=2, device=0):
    """Spectra of several particle sets (the power_spectrum path for each),
    with up to ``depth`` sets in flight on separate contexts: the copy of one
    set's host positions to the device overlaps the computation of the set
    before it (the copy engine and the SMs work at the same time), and each
    set's spectrum comes back as soon as it is done.  Host arrays should be
    in pinned memory (``pinned_empty``) for the copies to run asynchronously.
    Returns the spectra in input order."""
    if MAS not in _native.MAS_CODE:
        raise ValueError("option not valid!!! (MAS must be NGP, CIC, TSC or PCS)")
    if deposit not in DEPOSIT_FLAGS:
        raise ValueError("deposit must be one of %s" % sorted(DEPOSIT_FLAGS))
    win = MAS_function(MAS if window is None else window)
    ctxs = _pool(int(device), int(depth))
    pos_sets = list(pos_sets)
    W_sets = [None] * len(pos_sets) if W_sets is None else list(W_sets)
    results = [None] * len(pos_sets)
    inflight = []     # (index, context, outputs, keep-alive)

    def finish():
        i, ctx, out, _ = inflight.pop(0)
        _raise_or_exit(ctx, ctx.lib.pyl_pk_collect(ctx.ptr, ctypes.byref(out.struct), -1))
        res = Spectrum()
        out.assign(res)
        results[i] = res

    for i, (pos, W) in enumerate(zip(pos_sets, W_sets)):
        require_dtype(pos, "float32", "pos")
        if pos.ndim != 2 or int(pos.shape[1]) != 3:
            raise ValueError("pos must be (n, 3)")
        n = int(pos.shape[0])
        if len(inflight) == len(ctxs):
            finish()
        ctx = ctxs[i % len(ctxs)]
        out = _Outputs(int(dims), what)
        if is_cuda_tensor(pos):
            p = pos.contiguous()
            w = None if W is None else W.contiguous()
            torch_sync(p)
            pp, wp, flags = dev_ptr(p), (dev_ptr(w) if w is not None else None), _native.PYL_DEVICE_PTRS
        else:
            p = np.ascontiguousarray(pos)
            w = None if W is None else np.ascontiguousarray(W, np.float32)
            pp, wp, flags = host_ptr(p), (host_ptr(w) if w is not None else None), 0
        rc = ctx.lib.pyl_pk_particles_enqueue(ctx.ptr, pp, n, wp, int(dims), ctypes.c_float(BoxSize),
                                              _native.MAS_CODE[MAS], int(axis), win, int(what),
                                              flags | DEPOSIT_FLAGS[deposit])
        _raise_or_exit(ctx, rc)
        inflight.append((i, ctx, out, (p, w)))
    while inflight:
        finish()
    return results


def spectra_batch(requests, ctx=None, graph=True, lanes=0):
    """Spectra of a list of requests issued at once and waited for once
    (pyl_pk_batch), spread over ``lanes`` streams that run side by side
    (0: the library's default, 4): the first call with a given list captures the launch
    sequence into a CUDA graph, later calls with the same list (same arrays,
    sizes and options) launch it as one graph.  requests: dicts with the
    arguments of ``power_spectrum`` (pos, dims, BoxSize, MAS, axis, W,
    window, what); the positions are all CUDA tensors or all pinned host
    arrays.  Returns the spectra in order."""
    reqs = (_native.PkRequest * len(requests))()
    outs = [_Outputs(int(r["dims"]), int(r.get("what", 0))) for r in requests]
    outa = (_native.PkOut * len(requests))(*[o.struct for o in outs])
    keep = []
    dev = None
    for i, r in enumerate(requests):
        pos, W, MAS = r["pos"], r.get("W"), r.get("MAS", "CIC")
        require_dtype(pos, "float32", "pos")
        if MAS not in _native.MAS_CODE:
            raise ValueError("option not valid!!! (MAS must be NGP, CIC, TSC or PCS)")
        cuda = is_cuda_tensor(pos)
        if dev is None:
            dev = cuda
        elif dev != cuda:
            raise ValueError("positions must be all CUDA tensors or all host arrays")
        if cuda:
            p = pos.contiguous()
            w = None if W is None else W.contiguous()
            torch_sync(p)
            pp, wp = p.data_ptr(), (w.data_ptr() if w is not None else None)
        else:
            p = np.ascontiguousarray(pos)
            w = None if W is None else np.ascontiguousarray(W, np.float32)
            pp, wp = p.ctypes.data, (w.ctypes.data if w is not None else None)
        keep.append((p, w))
        win = MAS_function(MAS if r.get("window") is None else r["window"])
        reqs[i] = _native.PkRequest(pp, int(pos.shape[0]), wp, int(r["dims"]),
                                    float(r["BoxSize"]), _native.MAS_CODE[MAS],
                                    int(r.get("axis", 2)), win, int(r.get("what", 0)))
    if ctx is None:
        ctx = _native.context(requests[0]["pos"].device.index or 0 if dev else 0)
    flags = ((_native.PYL_DEVICE_PTRS if dev else 0) | (0 if graph else _native.PYL_NO_GRAPH)
             | ((int(lanes) & 0xF) << 16))
    _raise_or_exit(ctx, ctx.lib.pyl_pk_batch(ctx.ptr, reqs, len(requests), outa, flags))
    res = []
    for o in outs:
        s = Spectrum()
        o.assign(s)
        res.append(s)
    return res
