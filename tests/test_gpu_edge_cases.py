"""Edge cases of the deposit and the spectrum on the GPU: empty input, a
single dense clump (tiles split into many work items, fixed-point scales
set by huge box sums), non-finite positions and weights, a zero field."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOX = 1000.0


@pytest.fixture(scope="module")
def gpu():
    import torch
    assert torch.cuda.is_available()
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    return P


def test_empty_input_leaves_grid(gpu):
    g = np.full((32,) * 3, 3.0, np.float32)
    gpu.MAS_library.MA(np.zeros((0, 3), np.float32), g, BOX, "CIC")
    assert np.all(g == 3.0)


@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS"])
@pytest.mark.parametrize("weighted", [False, True])
def test_dense_clump(gpu, oracle, MAS, weighted):
    """2^21 particles within one cell's width: one tile holds them all (32
    work items).  Mass is conserved to 1e-5 (the reference's own known-answer
    bound, library/tests/test.py:30-33), and every cell is as close to
    the float64 deposit as 1e-5 of the maximum or 3x the error of the
    oracle's own float32 sum (cells here sum ~10^6 terms of ~0.1)."""
    rng = np.random.default_rng(21)
    n = 1 << 21
    pos = (np.float32(500.0) + rng.random((n, 3), dtype=np.float32) * np.float32(10.0))
    W = rng.lognormal(0, 0.5, n).astype(np.float32) if weighted else None
    ref = oracle.MA_f64(pos, 64, BOX, MAS, W=W)
    ref32 = np.zeros((64,) * 3, np.float32)
    oracle.MA(pos, ref32, BOX, MAS, W=W)
    own = float(np.abs(ref32 - ref).max())
    g = np.zeros((64,) * 3, np.float32)
    gpu.MAS_library.MA(pos, g, BOX, MAS, W=W)
    assert abs(g.sum(dtype=np.float64) / ref.sum() - 1) < 1e-5
    assert np.abs(g - ref).max() <= max(1e-5 * np.abs(ref).max(), 3 * own)


def test_non_finite_inputs_stay_bounded(gpu):
    """NaN/inf positions are taken as 0 (their cells stay in the grid) and
    the call completes; a NaN weight makes its cells NaN, as float adds do,
    without touching other cells."""
    rng = np.random.default_rng(4)
    pos = rng.random((1 << 20, 3), dtype=np.float32) * np.float32(BOX)
    pos[:10] = np.nan
    pos[10:20] = np.inf
    g = np.zeros((64,) * 3, np.float32)
    gpu.MAS_library.MA(pos, g, BOX, "CIC")
    assert np.isfinite(g).all()
    assert abs(g.sum(dtype=np.float64) - len(pos)) < 1e-3 * len(pos)
    W = np.ones(len(pos), np.float32)
    W[100] = np.nan
    g2 = np.zeros((64,) * 3, np.float32)
    gpu.MAS_library.MA(pos, g2, BOX, "CIC", W=W)
    assert 0 < np.isnan(g2).sum() <= 8


def test_zero_field_spectrum(gpu):
    r = gpu.Pk_library.Pk(np.zeros((32,) * 3, np.float32), BOX, axis=0, MAS="CIC", verbose=False)
    assert np.all(r.Pk == 0.0)
    assert int(r.Nmodes3D.sum()) + 1 == (32 ** 3 - 8) // 2 + 8


def test_power_spectrum_rejects_empty(gpu):
    from pylians3_gb300 import PylError
    with pytest.raises(PylError):
        gpu.power_spectrum(np.zeros((0, 3), np.float32), 32, BOX, "CIC")
