"""Both deposit paths (unsorted global atomics and tile-sorted shared memory,
the latter with fixed-point or float32 shared accumulation), forced through
the C ABI flags, against the oracle on uniform, clustered and edge-case
inputs.  Grids agree to float32 rounding of a different summation order (or
the fixed point's rounding of each tap): |diff| <= 1e-5 * max(1, |value|)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOX = 1000.0


@pytest.fixture(scope="module")
def native():
    import torch
    assert torch.cuda.is_available()
    from pylians3_gb300 import build_native, _native
    build_native.build()
    return _native


def run_ma(native, pos, dims, MAS, W=None, flags=0, grid=None):
    ctx = native.context(0)
    g = np.zeros((dims,) * 3, np.float32) if grid is None else grid
    p = np.ascontiguousarray(pos, np.float32)
    w = None if W is None else np.ascontiguousarray(W, np.float32)
    ctx.check(ctx.lib.pyl_ma(ctx.ptr, ctypes.c_void_p(p.ctypes.data), len(p), 3,
                             None if w is None else ctypes.c_void_p(w.ctypes.data),
                             ctypes.c_void_p(g.ctypes.data), dims, ctypes.c_float(BOX),
                             native.MAS_CODE[MAS], 0, flags))
    return g


def inputs(kind, n, rng):
    if kind == "uniform":
        return rng.random((n, 3), dtype=np.float32) * np.float32(BOX)
    if kind == "clustered":
        c = rng.random((20, 3)) * BOX
        p = c[rng.integers(0, 20, n)] + rng.standard_normal((n, 3)) * 8.0
        return np.mod(p, BOX).astype(np.float32)
    # edges: exact cell boundaries, 0 and BoxSize and the last float below it
    vals = np.array([0.0, BOX / 64, BOX / 2, BOX - BOX / 64, BOX,
                     np.nextafter(np.float32(BOX), np.float32(0))], np.float32)
    e = np.stack(np.meshgrid(vals, vals, vals, indexing="ij"), -1).reshape(-1, 3)
    return np.concatenate([e, rng.random((n, 3), dtype=np.float32) * np.float32(BOX)])


@pytest.mark.parametrize("dims", [32, 48, 50, 64, 128])
@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS"])
@pytest.mark.parametrize("kind", ["uniform", "clustered", "edges"])
def test_paths_match_oracle(native, oracle, dims, MAS, kind):
    rng = np.random.default_rng(dims * 7 + len(kind))
    pos = inputs(kind, 200000, rng)
    W = rng.lognormal(0, 0.5, len(pos)).astype(np.float32)
    for w in (None, W):
        ref = np.zeros((dims,) * 3, np.float32)
        oracle.MA(pos, ref, BOX, MAS, W=w)
        # Dense clustered cells sum ~1e4 float32 terms: the oracle's own
        # rounding (vs its float64 deposit) can exceed 1e-5 of the maximum.
        # Every path must be as close to the float64 grid as 3x that, or
        # within 1e-5 of the maximum of the float32 oracle.
        ref64 = oracle.MA_f64(pos, dims, BOX, MAS, W=w)
        own = float(np.abs(ref - ref64).max())
        tol = 1e-5 * max(1.0, float(np.abs(ref).max()))
        for flags in (native.PYL_DEPOSIT_SORTED,
                      native.PYL_DEPOSIT_SORTED | native.PYL_SORT_TWO_PASS,
                      native.PYL_DEPOSIT_SORTED | native.PYL_SORT_FRONTIER,
                      native.PYL_DEPOSIT_SORTED | native.PYL_DEPOSIT_FLOAT,
                      native.PYL_DEPOSIT_ATOMIC):
            g = run_ma(native, pos, dims, MAS, w, flags)
            ok = (float(np.abs(g - ref).max()) <= tol or
                  float(np.abs(g - ref64).max()) <= 3 * own)
            assert ok, (flags, w is None, float(np.abs(g - ref).max()), own)


def test_sorted_accumulates(native, oracle):
    rng = np.random.default_rng(1)
    pos = rng.random((300000, 3), dtype=np.float32) * np.float32(BOX)
    base = rng.random((64,) * 3, dtype=np.float32)
    g = run_ma(native, pos, 64, "TSC", flags=native.PYL_DEPOSIT_SORTED, grid=base.copy())
    ref = base.copy()
    oracle.MA(pos, ref, BOX, "TSC")
    assert float(np.abs(g - ref).max()) <= 1e-5 * float(np.abs(ref).max())


def test_sorted_unaligned_device_grid(native, oracle):
    """A grid that is a view at a 4-byte offset takes the scalar flush."""
    import torch
    rng = np.random.default_rng(2)
    pos = rng.random((300000, 3), dtype=np.float32) * np.float32(BOX)
    dims = 64
    buf = torch.zeros(dims ** 3 + 1, device="cuda")
    view = buf[1:]
    tp = torch.from_numpy(pos).cuda()
    ctx = native.context(0)
    ctx.check(ctx.lib.pyl_ma(ctx.ptr, ctypes.c_void_p(tp.data_ptr()), len(pos), 3, None,
                             ctypes.c_void_p(view.data_ptr()), dims, ctypes.c_float(BOX),
                             native.MAS_CODE["CIC"], 0,
                             native.PYL_DEVICE_PTRS | native.PYL_DEPOSIT_SORTED))
    ctx.synchronize()
    ref = np.zeros((dims,) * 3, np.float32)
    oracle.MA(pos, ref, BOX, "CIC")
    assert float(buf[0].item()) == 0.0
    got = view.cpu().numpy().reshape((dims,) * 3)
    assert float(np.abs(got - ref).max()) <= 1e-5 * float(ref.max())


@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS"])
@pytest.mark.parametrize("path", ["sorted", "atomic"])
def test_compensated_matches_float64(native, oracle, MAS, path):
    """PYL_COMPENSATED: every cell is the float64 sum of its taps rounded
    once to float32, also in cells holding thousands of particles (where the
    plain float32 sums drift by many ulps).  NGP/CIC/TSC taps equal the
    reference's; PCS taps carry the float32 evaluation of the cubic (a few
    ulps each), which the bound adds for PCS."""
    rng = np.random.default_rng(17)
    c = rng.random((8, 3)) * BOX
    pos = np.concatenate([
        np.mod(c[rng.integers(0, 8, 400000)] + rng.standard_normal((400000, 3)) * 3.0, BOX),
        rng.random((200000, 3)) * BOX]).astype(np.float32)
    W = rng.lognormal(0, 0.5, len(pos)).astype(np.float32)
    flag = native.PYL_DEPOSIT_SORTED if path == "sorted" else native.PYL_DEPOSIT_ATOMIC
    for w in (None, W):
        ref64 = oracle.MA_f64(pos, 64, BOX, MAS, W=w)
        g = run_ma(native, pos, 64, MAS, w, flag | native.PYL_COMPENSATED)
        ulp = np.spacing(np.abs(ref64).astype(np.float32)).astype(np.float64)
        tol = 1.0 * ulp + (8 * 2.0 ** -24 * np.abs(ref64) if MAS == "PCS" else 0.0)
        err = np.abs(g.astype(np.float64) - ref64)
        assert np.all(err <= tol), (MAS, path, w is None, float((err / ulp).max()))


def test_sorted_unaligned_device_positions(native, oracle):
    """Positions at a 4-byte offset: the counting pass and the first
    partition pass take their plain-load forms (no 16-byte vector or bulk
    loads); the grid equals the aligned case."""
    import torch
    rng = np.random.default_rng(12)
    n = 1 << 20
    pos = rng.random((n, 3), dtype=np.float32) * np.float32(BOX)
    buf = torch.zeros(3 * n + 1, device="cuda")
    buf[1:] = torch.from_numpy(pos.reshape(-1)).cuda()
    view = buf[1:]
    assert view.data_ptr() % 16 != 0
    ctx = native.context(0)
    for MAS in ("CIC", "TSC"):
        g = torch.zeros((64,) * 3, device="cuda")
        ctx.check(ctx.lib.pyl_ma(ctx.ptr, ctypes.c_void_p(view.data_ptr()), n, 3, None,
                                 ctypes.c_void_p(g.data_ptr()), 64, ctypes.c_float(BOX),
                                 native.MAS_CODE[MAS], 1,
                                 native.PYL_DEVICE_PTRS | native.PYL_DEPOSIT_SORTED))
        ctx.synchronize()
        ref = np.zeros((64,) * 3, np.float32)
        oracle.MA(pos, ref, BOX, MAS)
        assert np.abs(g.cpu().numpy() - ref).max() <= 1e-5 * np.abs(ref).max()
