"""The autotuner picks a tile shape among the candidates, and the deposit's
results do not depend on the tile shape or the coarse bucket size."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOX = 1000.0


@pytest.fixture(scope="module")
def env():
    import torch
    assert torch.cuda.is_available()
    from pylians3_gb300 import build_native
    build_native.build()
    from pylians3_gb300 import _native, autotune
    return torch, _native, autotune


def test_tune_returns_a_valid_shape(env, tmp_path, monkeypatch):
    torch, N, at = env
    monkeypatch.setenv("PYLGPU_TUNE_CACHE", str(tmp_path / "cache.json"))
    shape, times = at.tune(64, "CIC", 1 << 20, reps=1)
    assert shape in times and len(times) >= 4
    assert at.current_shape(64, "CIC") == shape
    again, t2 = at.tune(64, "CIC", 1 << 20, reps=1)       # from the cache
    assert again == shape and t2 == {}
    at.set_shape(64, "CIC", None)


@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS"])
@pytest.mark.parametrize("shape", [(8, 32, 16, 0), (32, 8, 32, 4), (16, 16, 16, 64)])
def test_deposit_independent_of_shape(env, oracle, MAS, shape):
    torch, N, at = env
    rng = np.random.default_rng(3)
    pos = rng.random((300000, 3), dtype=np.float32) * np.float32(BOX)
    W = rng.lognormal(0, 0.5, len(pos)).astype(np.float32)
    ctx = N.context(0)
    assert at.set_shape(64, MAS, shape)
    try:
        for w in (None, W):
            ref = oracle.MA_f64(pos, 64, BOX, MAS, W=w)
            g = np.zeros((64,) * 3, np.float32)
            ctx.check(ctx.lib.pyl_ma(ctx.ptr, ctypes.c_void_p(pos.ctypes.data), len(pos), 3,
                                     None if w is None else ctypes.c_void_p(w.ctypes.data),
                                     ctypes.c_void_p(g.ctypes.data), 64, ctypes.c_float(BOX),
                                     N.MAS_CODE[MAS], 1, N.PYL_DEPOSIT_SORTED))
            assert np.abs(g - ref).max() <= 1e-5 * np.abs(ref).max()
    finally:
        at.set_shape(64, MAS, None)
