"""GPU parity of the rows around the spectrum: correct_MAS, the 2D FFTs and
Pk_plane, XPk and CIC_interp, against the reference's golden vectors and the
oracle on larger seeded inputs (including 3*2^k and odd grid lengths)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOX = 1000.0
TOL_PK = 1e-4


@pytest.fixture(scope="module")
def gpu():
    import torch
    assert torch.cuda.is_available()
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    return P


@pytest.fixture(scope="module")
def nxt():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "next_golden.npz"))


# ------------------------------------------------------------ correct_MAS
@pytest.mark.parametrize("dims", [16, 17])
@pytest.mark.parametrize("MAS", ["CIC", "TSC", "PCS", "None"])
def test_correct_mas_golden(gpu, nxt, dims, MAS):
    delta = nxt["cm_delta_d%d" % dims]
    before = delta.copy()
    got = gpu.Pk_library.correct_MAS(delta, BOX, MAS=MAS)
    want = nxt["cm_out_d%d_%s" % (dims, MAS)]
    assert got.dtype == np.float32 and got.shape == want.shape
    assert np.abs(got - want).max() <= 2e-5 * np.abs(want).max()
    assert np.array_equal(delta, before)


@pytest.mark.parametrize("dims", [64, 96, 100])
def test_correct_mas_vs_oracle(gpu, oracle, dims):
    import torch
    rng = np.random.default_rng(dims)
    delta = rng.standard_normal((dims,) * 3).astype(np.float32)
    want = oracle.correct_MAS(delta, BOX, MAS="PCS")
    got = gpu.Pk_library.correct_MAS(delta, BOX, MAS="PCS")
    assert np.abs(got - want).max() <= 2e-5 * np.abs(want).max()
    t = gpu.Pk_library.correct_MAS(torch.from_numpy(delta).cuda(), BOX, MAS="PCS")
    assert t.is_cuda and np.abs(t.cpu().numpy() - want).max() <= 2e-5 * np.abs(want).max()


# ------------------------------------------------------ 2D FFTs, Pk_plane
@pytest.mark.parametrize("grid", [16, 17, 48, 100, 256, 1024])
def test_fft2_r2c_c2r(gpu, grid):
    rng = np.random.default_rng(grid)
    a = rng.standard_normal((grid, grid)).astype(np.float32)
    f = gpu.Pk_library.FFT2Dr_f(a, 1)
    ref = np.fft.rfft2(a.astype(np.float64))
    assert f.shape == ref.shape and f.dtype == np.complex64
    assert np.abs(f - ref).max() / np.sqrt(np.mean(np.abs(ref) ** 2)) < 2e-5
    back = gpu.Pk_library.IFFT2Dr_f(f, 1)
    assert np.abs(back - a).max() < 2e-5


@pytest.mark.parametrize("grid", [16, 17, 32])
@pytest.mark.parametrize("MAS", ["NGP", "CIC", "PCS", "None"])
def test_pk_plane_golden(gpu, nxt, grid, MAS):
    r = gpu.Pk_library.Pk_plane(nxt["pp_delta_g%d" % grid], BOX, MAS=MAS, verbose=False)
    np.testing.assert_array_equal(r.Nmodes, nxt["pp_Nmodes_g%d_%s" % (grid, MAS)])
    np.testing.assert_allclose(r.k, nxt["pp_k_g%d_%s" % (grid, MAS)], rtol=1e-12)
    np.testing.assert_allclose(r.Pk, nxt["pp_Pk_g%d_%s" % (grid, MAS)], rtol=TOL_PK)


@pytest.mark.parametrize("grid", [255, 384, 2048])
def test_pk_plane_vs_oracle(gpu, oracle, grid):
    rng = np.random.default_rng(grid)
    delta = rng.standard_normal((grid, grid)).astype(np.float32)
    ref = oracle.Pk_plane(delta, BOX, MAS="CIC")
    r = gpu.Pk_library.Pk_plane(delta, BOX, MAS="CIC", verbose=False)
    np.testing.assert_array_equal(r.Nmodes, ref.Nmodes)
    np.testing.assert_allclose(r.k, ref.k, rtol=1e-12)
    np.testing.assert_allclose(r.Pk, ref.Pk, rtol=TOL_PK)


# ------------------------------------------------------------------ XPk
def _xpk_close(r, want, keys=("Pk", "XPk", "Pk1D", "PkX1D", "Pk2D", "PkX2D")):
    """Per bin, every series within TOL_PK of the auto spectra's scale."""
    for key in ("Nmodes3D", "Nmodes1D", "Nmodes2D"):
        np.testing.assert_array_equal(getattr(r, key), want(key))
    for key in ("k3D", "k1D", "kpar", "kper"):
        np.testing.assert_allclose(getattr(r, key), want(key), rtol=1e-12)
    for key in keys:
        w = want(key)
        g = getattr(r, key)
        assert g.shape == w.shape, key
        auto = want({"XPk": "Pk", "PkX1D": "Pk1D", "PkX2D": "Pk2D"}.get(key, key))
        scale = np.abs(auto).max(axis=tuple(range(1, auto.ndim)), keepdims=True)
        scale = scale.reshape(scale.shape[:1] + (1,) * (w.ndim - 1))
        err = np.abs(g - w) / np.maximum(scale, 1e-300)
        assert err.max() <= TOL_PK, (key, float(err.max()))


@pytest.mark.parametrize("dims", [16, 17])
@pytest.mark.parametrize("axis", [0, 2])
def test_xpk_golden(gpu, nxt, dims, axis):
    fields = [nxt["xp_delta%d_d%d" % (i, dims)] for i in range(3)]
    r = gpu.Pk_library.XPk(fields, BOX, axis=axis, MAS=["CIC", "PCS", "CIC"])
    _xpk_close(r, lambda k: nxt["xp_%s_d%d_a%d" % (k, dims, axis)])


@pytest.mark.parametrize("dims,axis", [(64, 1), (96, 2)])
def test_xpk_vs_oracle_and_pk(gpu, oracle, dims, axis):
    import torch
    rng = np.random.default_rng(dims)
    a = rng.standard_normal((dims,) * 3).astype(np.float32)
    b = (0.3 * a + rng.standard_normal((dims,) * 3)).astype(np.float32)
    MAS = ["TSC", "CIC"]
    ref = oracle.XPk([a, b], BOX, axis=axis, MAS=MAS)
    r = gpu.Pk_library.XPk([torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()], BOX,
                           axis=axis, MAS=MAS)
    _xpk_close(r, lambda k: getattr(ref, k))
    # the auto spectra are class Pk's
    p = gpu.Pk_library.Pk(a, BOX, axis=axis, MAS="TSC", verbose=False)
    err = np.abs(r.Pk[:, :, 0] - p.Pk).max(axis=1) / np.abs(p.Pk[:, 0])
    assert err.max() <= TOL_PK


# ------------------------------------------------------------ CIC_interp
@pytest.mark.parametrize("dims", [16, 17])
def test_cic_interp_golden(gpu, nxt, dims):
    pos = nxt["ci_pos_d%d" % dims]
    den = np.zeros(len(pos), np.float32)
    gpu.MAS_library.CIC_interp(nxt["ci_grid_d%d" % dims], BOX, pos, den)
    want = nxt["ci_den_d%d" % dims]
    assert np.abs(den - want).max() <= 1e-6 * np.abs(want).max()


def test_cic_interp_vs_oracle_exact(gpu, oracle):
    """Same float32 steps in the same order as the restatement: bit-exact."""
    import torch
    rng = np.random.default_rng(5)
    grid = rng.standard_normal((128,) * 3).astype(np.float32)
    pos = rng.random((1 << 20, 3), dtype=np.float32) * np.float32(BOX)
    want = np.zeros(len(pos), np.float32)
    oracle.CIC_interp(grid, BOX, pos, want)
    den = np.zeros(len(pos), np.float32)
    gpu.MAS_library.CIC_interp(grid, BOX, pos, den)
    assert np.array_equal(den, want)
    dt = torch.zeros(len(pos), device="cuda")
    gpu.MAS_library.CIC_interp(torch.from_numpy(grid).cuda(), BOX, torch.from_numpy(pos).cuda(), dt)
    assert np.array_equal(dt.cpu().numpy(), want)


def test_cic_interp_inverts_constant_and_linear(gpu):
    """Interpolating a constant grid gives the constant; a grid linear in x
    (away from the periodic seam) gives the linear function of position."""
    dims = 64
    g = np.full((dims,) * 3, 2.5, np.float32)
    rng = np.random.default_rng(6)
    pos = rng.random((100000, 3), dtype=np.float32) * np.float32(BOX)
    den = np.zeros(len(pos), np.float32)
    gpu.MAS_library.CIC_interp(g, BOX, pos, den)
    assert np.abs(den - 2.5).max() < 1e-5
    lin = np.broadcast_to(np.arange(dims, dtype=np.float32)[:, None, None], (dims,) * 3).copy()
    pos[:, 0] = rng.random(len(pos), dtype=np.float32) * np.float32(BOX * (dims - 2) / dims)
    gpu.MAS_library.CIC_interp(lin, BOX, pos, den)
    assert np.abs(den - pos[:, 0] * (dims / BOX)).max() < 1e-3
