"""Autotuner of the sorted deposit's tile shape and sort granularity.

For a (dims, MAS) workload the deposit's cost depends on the tile extents
(shared footprint per CTA, halo overhead, number of tiles) and on F, the
tiles per coarse bucket of the first partition pass (the fan-out of each of
the two passes).  ``tune(dims, MAS, n)`` times the whole sorted deposit
(counting pass, both partition passes, tile accumulation; pyl_ma on device
arrays, CUDA events on the context stream) for every candidate shape that
fits the kernels' limits, then the best shape for a few values of F, sets
the winner for the process with pyl_set_tile_shape and returns it.  Results
are kept in a JSON cache (``cache_path()``) keyed by device, dims, MAS, the
particle count rounded to a power of two and whether the particles carry
weights, so that later processes reuse them (``load_cache()`` applies every
entry of the current device).
"""
from __future__ import annotations

import ctypes
import json
import math
import os

from . import _native

_CACHE_ENV = "PYLGPU_TUNE_CACHE"


def cache_path() -> str:
    return os.environ.get(_CACHE_ENV) or os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                      "_tune_cache.json")


def current_shape(dims: int, mas: str):
    lib = _native.load()
    v = [ctypes.c_int() for _ in range(4)]
    rc = lib.pyl_get_tile_shape(int(dims), _native.MAS_CODE[mas], *[ctypes.byref(x) for x in v])
    if rc != _native.PYL_OK:
        raise _native.PylError(rc, "pyl_get_tile_shape")
    return tuple(x.value for x in v)


def set_shape(dims: int, mas: str, shape) -> bool:
    """Applies (TX, TY, TZ, F) for the process; False if the kernels cannot
    take it.  shape = None restores the built-in rule."""
    lib = _native.load()
    TX, TY, TZ, F = shape if shape is not None else (0, 0, 0, 0)
    return lib.pyl_set_tile_shape(int(dims), _native.MAS_CODE[mas], TX, TY, TZ, F) == _native.PYL_OK


def candidates(dims: int):
    """Tile extents to try: powers of two from 8 to 32 (z from 16) within the grid."""
    out = []
    for TZ in (16, 32):
        for TY in (8, 16, 32):
            for TX in (8, 16, 32):
                if max(TX, TY, TZ) <= max(8, dims):
                    out.append((TX, TY, TZ))
    return out


def _key(dims, mas, n, weighted, device):
    import torch
    name = torch.cuda.get_device_name(device)
    return "%s|%d|%s|%d|%d" % (name, dims, mas, int(round(math.log2(max(n, 1)))), int(weighted))


def _time_deposit(ctx, pos, W, grid, dims, mas, reps):
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream)
    n = int(pos.shape[0])
    wp = ctypes.c_void_p(W.data_ptr()) if W is not None else None
    flags = _native.PYL_DEVICE_PTRS | _native.PYL_DEPOSIT_SORTED

    def run():
        ctx.check(ctx.lib.pyl_ma(ctx.ptr, ctypes.c_void_p(pos.data_ptr()), n, 3, wp,
                                 ctypes.c_void_p(grid.data_ptr()), dims, ctypes.c_float(1000.0),
                                 _native.MAS_CODE[mas], 1, flags))
    run()
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(dims: int, mas: str, n: int, weighted: bool = False, reps: int = 3, device: int = 0,
         positions=None, use_cache: bool = True):
    """Best (TX, TY, TZ, F) for the sorted deposit of n particles on a dims^3
    grid with scheme mas; sets it for the process and returns
    (shape, {shape: ms}).  positions: a CUDA (n, 3) tensor to time on
    (default: seeded uniform positions)."""
    import torch
    key = _key(dims, mas, n, weighted, device)
    cache = _read_cache() if use_cache else {}
    if key in cache:
        shape = tuple(cache[key]["shape"])
        if set_shape(dims, mas, shape):
            return shape, {}
    ctx = _native.Context(device)
    g = torch.Generator(device="cuda").manual_seed(1234)
    pos = positions if positions is not None else (
        torch.rand((int(n), 3), generator=g, device="cuda") * 1000.0)
    W = (torch.exp(0.5 * torch.randn(pos.shape[0], generator=g, device="cuda"))
         if weighted else None)
    grid = torch.zeros((dims,) * 3, device="cuda")
    timings = {}
    default = current_shape(dims, mas)
    best, best_ms = None, float("inf")
    for TX, TY, TZ in candidates(dims):
        shape = (TX, TY, TZ, 0)
        if not set_shape(dims, mas, shape):
            continue
        ms = _time_deposit(ctx, pos, W, grid, dims, mas, reps)
        full = current_shape(dims, mas)
        timings[full] = ms
        if ms < best_ms:
            best, best_ms = full, ms
    if best is not None:
        for F in sorted({max(1, best[3] // 2), best[3] * 2}):
            shape = best[:3] + (F,)
            if F > 256 or not set_shape(dims, mas, shape):
                continue
            ms = _time_deposit(ctx, pos, W, grid, dims, mas, reps)
            timings[current_shape(dims, mas)] = ms
            if ms < best_ms:
                best, best_ms = current_shape(dims, mas), ms
    ctx.close()
    if best is None:
        set_shape(dims, mas, None)
        return default, timings
    set_shape(dims, mas, best)
    if use_cache:
        cache = _read_cache()
        cache[key] = {"shape": list(best), "ms": best_ms,
                      "default": list(default), "default_ms": timings.get(default)}
        _write_cache(cache)
    return best, timings


def _read_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _write_cache(cache):
    tmp = cache_path() + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, cache_path())


def load_cache(device: int = 0) -> int:
    """Applies every cached shape of this device; returns how many."""
    import torch
    name = torch.cuda.get_device_name(device)
    k = 0
    for key, v in _read_cache().items():
        dev, dims, mas, _, _ = key.split("|")
        if dev == name and set_shape(int(dims), mas, tuple(v["shape"])):
            k += 1
    return k
