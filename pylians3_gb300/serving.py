"""Continuous batching of power-spectrum requests on one GPU.

A request is a particle set to turn into a spectrum (the pyl_pk_particles
path: deposit, FFT, window, multipoles, binning).  ``Server`` keeps a pool of
contexts ("slots"), each with its own CUDA stream and its own resident
workspaces (sorted particles, grid, half-complex grid, FFT twiddles, mode
tables), and a dispatcher thread that

  * admits queued requests in arrival order as soon as a slot is free and
    the device memory the slots would then hold stays within the HBM budget
    (idle slots are trimmed first when it would not);
  * issues each admitted request with ``pyl_pk_particles_enqueue`` on its
    slot's stream, so requests of different sizes run on the device at the
    same time;
  * polls the slots with ``pyl_pk_query`` and finishes a request with
    ``pyl_pk_collect`` as soon as its work is done, freeing the slot for the
    next request.

Every request's result depends only on its own input: it uses its slot's
buffers alone, so the spectrum is the same whether it ran alone or among
other requests (up to the order of floating-point atomic additions).

``run_batch`` is the batched form for a fixed list of realizations (all
submitted at once, collected when done).
"""
from __future__ import annotations

import ctypes
import threading
import time
from collections import deque
from concurrent.futures import Future

import numpy as np

from . import _native
from ._arrays import dev_ptr, host_ptr, is_cuda_tensor
from .Pk_library import MAS_function, _Outputs


def request_bytes(n: int, dims: int, weighted: bool, host_positions: bool) -> int:
    """Device bytes a request needs in a slot: the sort buffers (the
    count-free sort's coarse and tile slots with their margins and its spill
    list: about 3.2 records per particle), grid, half-complex grid, staging
    of host positions, small tables."""
    rs = (dims // 2 + 1 + 7) // 8 * 8
    b = int(12 * n * 3.2) + 4 * dims ** 3 + 8 * dims * dims * rs + (64 << 20)
    if weighted:
        b += int(4 * n * 3.2)
    if host_positions:
        b += 12 * n + (4 * n if weighted else 0)
    return b


class _Request:
    __slots__ = ("pos", "n", "W", "dims", "box", "mas", "axis", "window", "what", "flags",
                 "future", "t_submit", "t_start", "t_done", "bytes", "out", "keep")

    def __init__(self, **kw):
        for k, v in kw.items():
            setattr(self, k, v)


class Server:
    """Continuous-batching spectrum server on one device.

    ``slots``: requests that may be on the device at once.
    ``hbm_budget``: bytes of device memory the slots' workspaces may hold.
    ``contexts``: the slots' contexts, if the caller builds them (default:
    ``slots`` new contexts on ``device``); a context needs ``lib``, ``ptr``,
    ``workspace_bytes()``, ``trim()`` and ``close()``.
    """

    def __init__(self, slots: int = 8, hbm_budget: float = 150e9, device: int = 0,
                 contexts=None):
        self.device = device
        self.budget = int(hbm_budget)
        self.ctx = (list(contexts) if contexts is not None
                    else [_native.Context(device) for _ in range(slots)])
        self.busy: list = [None] * len(self.ctx)
        self.q: deque = deque()
        self.cv = threading.Condition()
        self.running = True
        self.failure = None          # set when the dispatcher dies: no more requests
        self.done_latencies: list = []
        self.completed = 0
        self.thread = threading.Thread(target=self._loop, name="pyl-server", daemon=True)
        self.thread.start()

    # ------------------------------------------------------------ client
    def submit(self, pos, dims, BoxSize, MAS="CIC", axis=2, W=None, window=None, what=0):
        """Queue a spectrum request; returns a Future of an object with the
        attributes of class Pk that were requested (k3D, Pk, Nmodes3D, ...).
        pos: (n, 3) float32 torch CUDA tensor, or numpy array (pinned host
        memory keeps the upload asynchronous)."""
        if MAS not in _native.MAS_CODE:
            raise ValueError("option not valid!!! (MAS must be NGP, CIC, TSC or PCS)")
        n = int(pos.shape[0])
        dev = is_cuda_tensor(pos)
        if not dev:
            pos = np.ascontiguousarray(pos, np.float32)
            if W is not None:
                W = np.ascontiguousarray(W, np.float32)
        elif W is not None:
            W = W.contiguous()
        nbytes = request_bytes(n, int(dims), W is not None, not dev)
        if nbytes > self.budget:
            raise _native.PylError(_native.PYL_ERR_BUDGET,
                                   "request needs %d bytes, budget %d" % (nbytes, self.budget))
        fut = Future()
        if self.failure is not None:
            raise RuntimeError("the server's dispatcher stopped: %r" % (self.failure,))
        r = _Request(pos=pos, n=n, W=W, dims=int(dims), box=float(BoxSize),
                     mas=_native.MAS_CODE[MAS], axis=int(axis),
                     window=MAS_function(MAS if window is None else window), what=int(what),
                     flags=_native.PYL_DEVICE_PTRS if dev else 0, future=fut,
                     t_submit=time.perf_counter(), t_start=None, t_done=None, bytes=nbytes,
                     out=None, keep=None)
        with self.cv:
            if self.failure is not None:
                raise RuntimeError("the server's dispatcher stopped: %r" % (self.failure,))
            self.q.append(r)
            self.cv.notify()
        return fut

    def close(self, wait: bool = True):
        with self.cv:
            self.running = False
            self.cv.notify()
        if wait:
            self.thread.join()
        for c in self.ctx:
            c.close()

    def latencies(self) -> np.ndarray:
        return np.asarray(self.done_latencies, dtype=np.float64)

    # ---------------------------------------------------------- internals
    def _held(self, skip=None) -> int:
        return sum(c.workspace_bytes() for i, c in enumerate(self.ctx) if i != skip)

    def _admit(self, slot: int, r: _Request) -> bool:
        c = self.ctx[slot]
        need = max(c.workspace_bytes(), r.bytes)
        if self._held(skip=slot) + need > self.budget:
            for i, other in enumerate(self.ctx):          # trim idle slots first
                if i != slot and self.busy[i] is None and other.workspace_bytes():
                    other.trim()
            if self._held(skip=slot) + need > self.budget:
                return False
        out = _Outputs(r.dims, r.what)
        p = dev_ptr(r.pos) if r.flags & _native.PYL_DEVICE_PTRS else host_ptr(r.pos)
        w = None
        if r.W is not None:
            w = dev_ptr(r.W) if r.flags & _native.PYL_DEVICE_PTRS else host_ptr(r.W)
        r.t_start = time.perf_counter()
        rc = c.lib.pyl_pk_particles_enqueue(c.ptr, p, r.n, w, r.dims, ctypes.c_float(r.box),
                                            r.mas, r.axis, r.window, r.what, r.flags)
        if rc != _native.PYL_OK:
            msg = c.lib.pyl_last_error(c.ptr)
            r.future.set_exception(_native.PylError(rc, msg.decode() if msg else ""))
            return True
        r.out = out
        self.busy[slot] = r
        return True

    def _finish(self, slot: int):
        r = self.busy[slot]
        c = self.ctx[slot]
        rc = c.lib.pyl_pk_collect(c.ptr, ctypes.byref(r.out.struct), -1)
        r.t_done = time.perf_counter()
        if rc != _native.PYL_OK:
            msg = c.lib.pyl_last_error(c.ptr)
            self.busy[slot] = None
            r.future.set_exception(_native.PylError(rc, msg.decode() if msg else ""))
            return
        res = _Result()
        r.out.assign(res)
        res.latency = r.t_done - r.t_submit
        res.service = r.t_done - r.t_start
        self.done_latencies.append(res.latency)
        self.completed += 1
        self.busy[slot] = None     # cleared last: a failure above leaves r in busy
        r.future.set_result(res)

    def _loop(self):
        try:
            self._dispatch()
        except BaseException as e:   # noqa: BLE001 -- every future must learn of it
            self._fail_all(e)

    def _fail_all(self, exc):
        """The dispatcher died: every request in flight or queued fails with
        the exception, and submit() refuses new requests."""
        with self.cv:
            self.failure = exc
            self.running = False
            pending = [r for r in self.busy if r is not None] + list(self.q)
            self.q.clear()
            self.busy = [None] * len(self.ctx)
        for r in pending:
            if not r.future.done():
                r.future.set_exception(exc)

    def _dispatch(self):
        while True:
            progressed = False
            for i, r in enumerate(self.busy):
                if r is not None:
                    c = self.ctx[i]
                    rc = c.lib.pyl_pk_query(c.ptr)
                    if rc != 0:
                        self._finish(i)
                        progressed = True
            with self.cv:
                while self.q:
                    free = [i for i, r in enumerate(self.busy) if r is None]
                    if not free:
                        break
                    r = self.q[0]
                    if not self._admit(free[0], r):
                        break
                    self.q.popleft()
                    progressed = True
                idle = all(b is None for b in self.busy)
                if not self.running and not self.q and idle:
                    return
                if not progressed:
                    if idle and not self.q:
                        self.cv.wait(timeout=0.01)
                    else:
                        self.cv.wait(timeout=2e-5)


class _Result:
    """Spectrum of one served request (attributes as class Pk)."""


def run_batch(requests, slots: int = 8, hbm_budget: float = 150e9, device: int = 0):
    """Spectra of a list of realizations, overlapped on the device.

    requests: iterable of dicts with the arguments of ``Server.submit``.
    Returns the results in request order and the wall time."""
    srv = Server(slots=slots, hbm_budget=hbm_budget, device=device)
    t0 = time.perf_counter()
    futs = [srv.submit(**r) for r in requests]
    res = [f.result() for f in futs]
    t1 = time.perf_counter()
    srv.close()
    return res, t1 - t0
