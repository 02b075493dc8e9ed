"""pyl_pk_noalloc -- the power spectrum of a device grid computed without
allocating device memory, for callers that cannot call cudaMalloc (a host
application whose pool allocator owns the device, a plugin host that forbids
outside allocations, a loop where cudaMalloc would synchronise the device).

Checked through the C ABI against pyl_pk on the same device grid, on two
calls in a row (the shared scratch array keeps the previous call's contents,
so the second call must clear what it needs).  Tolerances are those of the
other spectrum tests: mode counts exact, k3D to float64 rounding, per-bin
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
    # a context on a caller-provided stream creates no stream of its own
    stream = torch.cuda.Stream()
    ctx = _native.Context(0, stream=stream.cuda_stream)
    return torch, _native, ctx, stream


def run(native, ctx, fn_name, grid, dims, axis, mas, what):
    from pylians3_gb300.Pk_library import _Outputs
    out = _Outputs(dims, what)
    args = [ctx.ptr, ctypes.c_void_p(grid.data_ptr()), dims, BOX, axis, mas, what,
            ctypes.byref(out.struct)]
    if fn_name == "pyl_pk":
        args.append(native.PYL_DEVICE_PTRS)
    ctx.check(getattr(ctx.lib, fn_name)(*args))
    return out


@pytest.mark.parametrize("dims,axis,mas", [(64, 0, 2), (128, 2, 3), (32, 1, 4), (16, 2, 1)])
def test_noalloc_matches_pk(env, dims, axis, mas):
    torch, native, ctx, stream = env
    g = torch.Generator(device="cuda").manual_seed(dims + axis)
    with torch.cuda.stream(stream):
        grid = torch.randn((dims,) * 3, generator=g, device="cuda")
    stream.synchronize()
    ref = run(native, ctx, "pyl_pk", grid, dims, axis, mas, native.PYL_PK_ALL)
    for _ in range(2):
        got = run(native, ctx, "pyl_pk_noalloc", grid, dims, axis, mas, native.PYL_PK_ALL)
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


def test_noalloc_rejects_sizes_beyond_the_scratch(env):
    torch, native, ctx, stream = env
    for dims in (256, 100):
        grid = torch.zeros((dims,) * 3, device="cuda")
        from pylians3_gb300.Pk_library import _Outputs
        out = _Outputs(dims, 0)
        rc = ctx.lib.pyl_pk_noalloc(ctx.ptr, ctypes.c_void_p(grid.data_ptr()), dims, BOX, 2, 2,
                                    0, ctypes.byref(out.struct))
        assert rc == native.PYL_ERR_UNSUPPORTED
        assert b"power of two" in ctx.lib.pyl_last_error(ctx.ptr)
