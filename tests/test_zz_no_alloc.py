"""pyl_pk_noalloc -- the power spectrum of a device grid computed without
allocating device memory, for callers that cannot call cudaMalloc (a host
application whose pool allocator owns the device, a plugin host that forbids
outside allocations, a loop where cudaMalloc would synchronise the device).

Checked through the C ABI:
  * on a fresh context (on a caller-provided stream) that runs nothing but
    pyl_pk_noalloc: two calls in a row give pyl_pk's spectrum (computed on a
    separate context), the context holds no workspace afterwards, and the
    device's free memory is the same before and after the two calls (the
    first, warm-up call loads the kernels and resolves the scratch address);
  * against the reference's golden spectrum (dims 16) and the oracle (128^3,
    the same seeded overdensity).
The shared scratch array keeps the previous call's contents, so every call
must clear what it needs.  Tolerances are those of the other spectrum tests:
mode counts exact, k3D to float64 rounding, per-bin
|P_ell - P_ell,ref| / |P0_ref| <= 1e-4.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOX = 1000.0
TOL_PK = 1e-4


@pytest.fixture(scope="module")
def env():
    import torch
    assert torch.cuda.is_available(), "needs a CUDA device"
    from pylians3_gb300 import build_native, _native
    build_native.build()
    return torch, _native


def _ctx(torch, native):
    """A fresh context on a caller-provided stream (creates no stream)."""
    stream = torch.cuda.Stream()
    return native.Context(0, stream=stream.cuda_stream), stream


def run(native, ctx, fn_name, grid, dims, axis, mas, what):
    from pylians3_gb300.Pk_library import _Outputs
    out = _Outputs(dims, what)
    args = [ctx.ptr, ctypes.c_void_p(grid.data_ptr()), dims, BOX, axis, mas, what,
            ctypes.byref(out.struct)]
    if fn_name == "pyl_pk":
        args.append(native.PYL_DEVICE_PTRS)
    ctx.check(getattr(ctx.lib, fn_name)(*args))
    return out


def same_spectrum(got, ref):
    assert np.array_equal(got.Nmodes3D, ref.Nmodes3D)
    assert np.array_equal(got.Nmodes1D, ref.Nmodes1D)
    assert np.array_equal(got.Nmodes2D, ref.Nmodes2D)
    np.testing.assert_allclose(got.k3D, ref.k3D, rtol=1e-12)
    err = np.abs(got.Pk - ref.Pk).max(axis=1) / np.abs(ref.Pk[:, 0])
    assert float(err.max()) <= TOL_PK
    np.testing.assert_allclose(got.Pk1D, ref.Pk1D, rtol=TOL_PK,
                               atol=1e-12 * np.abs(ref.Pk1D).max())
    np.testing.assert_allclose(got.Pkphase, ref.Pkphase, rtol=TOL_PK)
    fin = np.isfinite(ref.Pk2D)
    assert np.array_equal(fin, np.isfinite(got.Pk2D))
    assert np.all(np.abs(got.Pk2D[fin] - ref.Pk2D[fin])
                  <= TOL_PK * np.abs(ref.Pk2D[fin]) + 1e-12)


@pytest.mark.parametrize("dims,axis,mas", [(64, 0, 2), (128, 2, 3), (32, 1, 4), (16, 2, 1)])
def test_noalloc_matches_pk_and_allocates_nothing(env, dims, axis, mas):
    torch, native = env
    g = torch.Generator(device="cuda").manual_seed(dims + axis)
    grid = torch.randn((dims,) * 3, generator=g, device="cuda")
    torch.cuda.synchronize()
    ref_ctx, _ = _ctx(torch, native)
    ref = run(native, ref_ctx, "pyl_pk", grid, dims, axis, mas, native.PYL_PK_ALL)
    ref_ctx.close()

    ctx, stream = _ctx(torch, native)
    run(native, ctx, "pyl_pk_noalloc", grid, dims, axis, mas, native.PYL_PK_ALL)  # warm-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        got = run(native, ctx, "pyl_pk_noalloc", grid, dims, axis, mas, native.PYL_PK_ALL)
        same_spectrum(got, ref)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert ctx.workspace_bytes() == 0
    ctx.close()


def test_noalloc_golden_and_oracle(env, golden, oracle):
    torch, native = env
    from pylians3_gb300.Pk_library import MAS_function
    ctx, _ = _ctx(torch, native)
    # the reference's own spectrum of the golden overdensity (dims 16)
    gp = golden["pk"]
    d16 = torch.from_numpy(np.ascontiguousarray(gp["delta_d16"])).cuda()
    for MAS in ("CIC", "PCS"):
        for axis in (0, 2):
            key = lambda k: "%s_d16_%s_a%d" % (k, MAS, axis)
            for _ in range(2):
                got = run(native, ctx, "pyl_pk_noalloc", d16, 16, axis, MAS_function(MAS), 0)
                assert np.array_equal(got.Nmodes3D, gp[key("Nmodes3D")])
                np.testing.assert_allclose(got.k3D, gp[key("k3D")], rtol=1e-12)
                err = np.abs(got.Pk - gp[key("Pk")]).max(axis=1) / np.abs(gp[key("Pk")][:, 0])
                assert float(err.max()) <= TOL_PK
    # the oracle on a seeded 128^3 overdensity
    rng = np.random.default_rng(77)
    pos = rng.random((2 * 128 ** 3, 3), dtype=np.float32) * np.float32(BOX)
    d = np.zeros((128,) * 3, np.float32)
    oracle.MA(pos, d, BOX, "TSC")
    d /= np.mean(d, dtype=np.float64)
    d -= 1.0
    ref = oracle.Pk(d, BOX, axis=1, MAS="TSC", threads=8)
    dt = torch.from_numpy(d).cuda()
    for _ in range(2):
        got = run(native, ctx, "pyl_pk_noalloc", dt, 128, 1, MAS_function("TSC"), 0)
        assert np.array_equal(got.Nmodes3D, ref.Nmodes3D)
        np.testing.assert_allclose(got.k3D, ref.k3D, rtol=1e-12)
        err = np.abs(got.Pk - ref.Pk).max(axis=1) / np.abs(ref.Pk[:, 0])
        assert float(err.max()) <= TOL_PK
    ctx.close()


def test_noalloc_rejects_sizes_beyond_the_scratch(env):
    torch, native = env
    ctx, _ = _ctx(torch, native)
    for dims in (256, 100):
        grid = torch.zeros((dims,) * 3, device="cuda")
        from pylians3_gb300.Pk_library import _Outputs
        out = _Outputs(dims, 0)
        rc = ctx.lib.pyl_pk_noalloc(ctx.ptr, ctypes.c_void_p(grid.data_ptr()), dims, BOX, 2, 2,
                                    0, ctypes.byref(out.struct))
        assert rc == native.PYL_ERR_UNSUPPORTED
        assert b"power of two" in ctx.lib.pyl_last_error(ctx.ptr)
    ctx.close()
