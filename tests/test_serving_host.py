"""Host logic of the continuous-batching server, on the CPU: arrival-order
admission, the HBM budget (with idle slots trimmed first), error
propagation, draining on close, and a dispatcher that dies (every future
fails, new submissions are refused).  The slots are fake contexts whose
"device work" completes after a few polls; no GPU is touched (the library
is loaded only for its host-side mode-count sizes)."""
import ctypes
import threading

import numpy as np
import pytest

from pylians3_gb300 import _native, serving


class _FakeLib:
    def __init__(self, owner):
        self.o = owner

    def pyl_pk_particles_enqueue(self, ptr, p, n, w, dims, box, mas, axis, window, what, flags):
        o = self.o
        if n == 13:                       # a request the fake device refuses
            o.err = b"fake enqueue failure"
            return _native.PYL_ERR_ARG
        with o.log_mu:
            o.ws = max(o.ws, serving.request_bytes(n, dims, w is not None, True))
            o.log.append(("enqueue", o.slot, n))
            o.held_log.append(sum(c.ws for c in o.all))
        o.pending = (n, 3)                # done after three polls
        return _native.PYL_OK

    def pyl_pk_query(self, ptr):
        n, left = self.o.pending
        if n == 666:                      # a fault inside the dispatcher
            raise OSError("fake query fault")
        gate = self.o.gates.get(n)
        if gate is not None and not gate.is_set():   # held by the test
            return 0
        self.o.pending = (n, left - 1)
        return 1 if left <= 1 else 0

    def pyl_pk_collect(self, ptr, out, timeout_ms):
        o = self.o
        n, _ = o.pending
        o.pending = None
        s = ctypes.cast(out, ctypes.POINTER(_native.PkOut)).contents
        ctypes.cast(s.k3D, ctypes.POINTER(ctypes.c_double))[0] = float(n)   # tag the result
        with o.log_mu:
            o.log.append(("collect", o.slot, n))
        return _native.PYL_OK

    def pyl_last_error(self, ptr):
        return self.o.err


class _FakeContext:
    def __init__(self, slot, peers, log, held_log, log_mu, gates):
        self.slot, self.all, self.log, self.held_log, self.log_mu = slot, peers, log, held_log, log_mu
        self.gates = gates
        self.ws = 0
        self.pending = None
        self.err = b""
        self.trims = 0
        self.ptr = ctypes.c_void_p(1)
        self.lib = _FakeLib(self)

    def workspace_bytes(self):
        return self.ws

    def trim(self):
        self.trims += 1
        self.ws = 0

    def close(self):
        pass


def _server(slots, budget, gates=None):
    log, held, mu, peers = [], [], threading.Lock(), []
    for i in range(slots):
        peers.append(_FakeContext(i, peers, log, held, mu, gates if gates is not None else {}))
    return serving.Server(hbm_budget=budget, contexts=peers), peers, log, held


def _pos(n):
    return np.zeros((n, 3), np.float32)


def test_all_requests_complete_with_their_own_results():
    srv, _, log, _ = _server(slots=2, budget=150e9)
    sizes = [100 + i for i in range(12)]
    futs = [srv.submit(_pos(n), 16, 1000.0, "CIC", axis=0) for n in sizes]
    res = [f.result(timeout=10) for f in futs]
    srv.close()
    assert [int(r.k3D[0]) for r in res] == sizes
    assert [e[2] for e in log if e[0] == "enqueue"] == sizes        # arrival order
    assert srv.completed == len(sizes) and len(srv.latencies()) == len(sizes)


def test_request_over_budget_is_refused_at_submit():
    srv, _, _, _ = _server(slots=2, budget=1e6)
    with pytest.raises(_native.PylError) as e:
        srv.submit(_pos(1 << 20), 64, 1000.0, "CIC")
    assert e.value.code == _native.PYL_ERR_BUDGET
    srv.close()


def test_budget_holds_and_idle_slots_are_trimmed():
    big = serving.request_bytes(1 << 22, 64, False, True)
    small = serving.request_bytes(64, 16, False, True)
    budget = int(1.5 * big)               # one big request, plus a small one
    assert big + small <= budget < 2 * big
    gate = threading.Event()
    srv, peers, log, held = _server(slots=3, budget=budget, gates={64: gate})
    # slot 0 ends up holding a small workspace, slot 1 a big one, both idle:
    # the small request stays on the device until the big one is enqueued
    s0 = srv.submit(_pos(64), 16, 1000.0, "CIC")
    b1 = srv.submit(_pos(1 << 22), 64, 1000.0, "TSC", axis=2)
    b1.result(timeout=10)
    gate.set()
    s0.result(timeout=10)
    assert peers[0].ws == small and peers[1].ws == big
    # the next big request goes to the first free slot (0); slot 1's idle
    # workspace has to be trimmed to keep both under the budget
    b2 = srv.submit(_pos(1 << 22), 64, 1000.0, "TSC", axis=2)
    assert int(b2.result(timeout=10).k3D[0]) == 1 << 22
    srv.close()
    assert peers[1].trims == 1 and peers[1].ws == 0
    assert ("enqueue", 0, 1 << 22) in log
    assert max(held) <= budget            # never more than the budget resident


def test_budget_serialises_big_requests():
    one = serving.request_bytes(4096, 64, False, True)
    srv, peers, log, held = _server(slots=3, budget=int(1.5 * one))
    futs = [srv.submit(_pos(4096), 64, 1000.0, "TSC", axis=2) for _ in range(6)]
    for f in futs:
        f.result(timeout=10)
    srv.close()
    assert max(held) <= int(1.5 * one)
    # one big request on the device at a time: enqueues and collects alternate
    kinds = [e[0] for e in log]
    assert kinds == ["enqueue", "collect"] * 6


def test_enqueue_error_reaches_the_future():
    srv, _, _, _ = _server(slots=2, budget=150e9)
    bad = srv.submit(_pos(13), 16, 1000.0, "CIC")
    good = srv.submit(_pos(14), 16, 1000.0, "CIC")
    with pytest.raises(_native.PylError) as e:
        bad.result(timeout=10)
    assert e.value.code == _native.PYL_ERR_ARG and "fake enqueue failure" in str(e.value)
    assert int(good.result(timeout=10).k3D[0]) == 14
    srv.close()


def test_close_drains_the_queue():
    srv, _, _, _ = _server(slots=1, budget=150e9)
    futs = [srv.submit(_pos(50 + i), 16, 1000.0, "NGP") for i in range(5)]
    srv.close(wait=True)                  # the loop returns only when all are done
    assert all(f.done() for f in futs)
    assert [int(f.result().k3D[0]) for f in futs] == [50 + i for i in range(5)]


def test_invalid_scheme_is_rejected():
    srv, _, _, _ = _server(slots=1, budget=150e9)
    with pytest.raises(ValueError):
        srv.submit(_pos(10), 16, 1000.0, "XYZ")
    srv.close()


def test_dispatcher_failure_fails_every_future():
    gate = threading.Event()
    srv, _, _, _ = _server(slots=2, budget=150e9, gates={70: gate})
    held = srv.submit(_pos(70), 16, 1000.0, "CIC")      # in flight, held by the gate
    boom = srv.submit(_pos(666), 16, 1000.0, "CIC")     # its poll raises
    queued = [srv.submit(_pos(80 + i), 16, 1000.0, "CIC") for i in range(4)]
    for f in [held, boom] + queued:
        with pytest.raises(OSError, match="fake query fault"):
            f.result(timeout=10)
    with pytest.raises(RuntimeError, match="dispatcher stopped"):
        srv.submit(_pos(90), 16, 1000.0, "CIC")
    gate.set()
    srv.close(wait=True)                  # returns: the loop has ended
