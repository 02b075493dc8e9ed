"""Pin the CPU oracle (oracle/) to the golden vectors made by the reference.

The golden vectors (tests/golden/*.npz) were produced by the reference's own
compiled MAS_library / Pk_library (tests/golden/make_golden.py).  The oracle
must reproduce them: mode counts and k-bins exactly, grids to float32
rounding (the reference was built with -ffast-math, which contracts some
multiply-adds), spectra to float64 rounding.
"""
import os

import numpy as np
import pytest

BOX = 1000.0
KEYS = ("k3D", "Pk", "Nmodes3D", "k1D", "Pk1D", "Nmodes1D", "kpar", "kper",
        "Pk2D", "Nmodes2D", "Pkphase")


@pytest.mark.parametrize("dims", [16, 17])
@pytest.mark.parametrize("coord", [3, 2])
@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS"])
@pytest.mark.parametrize("wt", [0, 1])
def test_ma_matches_reference(golden, oracle, dims, coord, MAS, wt):
    g = golden["ma"]
    tag = "d%d_c%d" % (dims, coord)
    pos, W = g["pos_" + tag], g["W_" + tag]
    ref = g["grid_%s_%s_w%d" % (tag, MAS, wt)]
    grid = np.zeros((dims,) * coord, np.float32)
    oracle.MA(pos, grid, BOX, MAS, W=W if wt else None)
    scale = max(1.0, float(np.abs(ref).max()))
    assert np.abs(grid - ref).max() <= 2e-6 * scale * (4 if coord == 2 else 1)
    # mass conservation, as library/tests/test.py asserts
    mass = float(W.astype(np.float64).sum()) if wt else float(len(pos))
    assert abs(grid.sum(dtype=np.float64) / mass - 1.0) < 1e-5


@pytest.mark.parametrize("dims", [16, 17, 24])
@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS", "None"])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_pk_matches_reference(golden, oracle, dims, MAS, axis):
    g = golden["pk"]
    delta = g["delta_d%d" % dims]
    r = oracle.Pk(delta, BOX, axis=axis, MAS=MAS, threads=1)
    for k in KEYS:
        ref = g["%s_d%d_%s_a%d" % (k, dims, MAS, axis)]
        got = np.asarray(getattr(r, k))
        assert got.shape == ref.shape, k
        if k.startswith("Nmodes"):
            assert np.array_equal(got, ref), k
        elif k == "Pk":
            # multipoles cross zero: compare against |P0| of the bin
            err = np.abs(got - ref).max(axis=1) / np.abs(ref[:, 0])
            assert err.max() < 1e-12, (k, err.max())
        else:
            fin = np.isfinite(ref)
            assert np.array_equal(fin, np.isfinite(got)), k
            scale = np.abs(ref[fin]).max() if fin.any() else 1.0
            assert np.abs(got[fin] - ref[fin]).max(initial=0.0) <= 1e-12 * scale, k


@pytest.mark.parametrize("dims", [8, 9, 63, 64, 128])
def test_mode_counts_match_reference(golden, oracle, dims):
    g = golden["nmodes"]
    z = np.zeros((dims,) * 3, np.float32)
    r = oracle.Pk(z, BOX, axis=2, MAS="CIC")
    assert np.array_equal(r.Nmodes3D, g["Nmodes3D_d%d" % dims])
    assert np.array_equal(r.Nmodes1D, g["Nmodes1D_d%d" % dims])
    assert np.array_equal(r.Nmodes2D, g["Nmodes2D_d%d" % dims])
    np.testing.assert_allclose(r.k3D, g["k3D_d%d" % dims], rtol=1e-13)
    assert int(r.Nmodes3D.sum()) + 1 == oracle.expected_modes(dims)


@pytest.mark.parametrize("dims", [8, 9, 63, 64, 128, 192, 256])
def test_data_free_mode_counts_match_reference(golden, oracle, dims):
    """oracle.mode_counts (the index part of the mode loop on all cores, the
    source of the 512 / 1024 known answers) against the reference's counts."""
    g = golden["nmodes"]
    m = oracle.mode_counts(dims, axis=2)
    assert np.array_equal(m["Nmodes3D"], g["Nmodes3D_d%d" % dims])
    assert np.array_equal(m["Nmodes1D"], g["Nmodes1D_d%d" % dims])
    assert np.array_equal(m["Nmodes2D"], g["Nmodes2D_d%d" % dims])
    np.testing.assert_allclose(m["k3D"] * (2 * np.pi / BOX), g["k3D_d%d" % dims], rtol=1e-12)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_threaded_binning_matches_serial(golden, oracle, axis):
    """The mode loop with its rows on several cores gives the serial loop's
    spectra (float64 sums in another order) and the same counts."""
    delta = golden["pk"]["delta_d24"]
    a = oracle.Pk(delta, BOX, axis=axis, MAS="TSC")
    b = oracle.Pk(delta, BOX, axis=axis, MAS="TSC", bin_threads=3)
    for k in ("Nmodes3D", "Nmodes1D", "Nmodes2D"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    for k in ("k3D", "Pk", "k1D", "Pk1D", "Pkphase"):
        np.testing.assert_allclose(getattr(b, k), getattr(a, k), rtol=1e-12, atol=0)
    fin = np.isfinite(a.Pk2D)
    np.testing.assert_allclose(b.Pk2D[fin], a.Pk2D[fin], rtol=1e-12)
    d64 = delta.astype(np.float64)
    c = oracle.Pk_f64(d64, BOX, axis=axis, MAS="TSC")
    d = oracle.Pk_f64(d64, BOX, axis=axis, MAS="TSC", bin_threads=3)
    np.testing.assert_allclose(d.Pk, c.Pk, rtol=1e-12)
    assert np.array_equal(c.Nmodes3D, d.Nmodes3D)


def test_pipeline_matches_reference(golden, oracle):
    g = golden["pipeline"]
    dims = g["delta"].shape[0]
    delta = np.zeros((dims,) * 3, np.float32)
    oracle.MA(g["pos"], delta, BOX, "CIC")
    delta /= np.mean(delta, dtype=np.float64)
    delta -= 1.0
    assert np.abs(delta - g["delta"]).max() < 1e-5
    r = oracle.Pk(delta, BOX, axis=0, MAS="CIC")
    p0 = np.abs(g["Pk"][:, 0])
    assert np.all(np.abs(r.Pk - g["Pk"]).max(axis=1) / p0 < 1e-5)
    assert np.array_equal(r.Nmodes3D, g["Nmodes3D"])


def test_fft_conventions(oracle):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((12, 12, 12)).astype(np.float32)
    f = oracle.FFT3Dr_f(a)
    assert f.dtype == np.complex64 and f.shape == (12, 12, 7)
    np.testing.assert_allclose(f, np.fft.rfftn(a.astype(np.float64)), rtol=1e-4, atol=1e-4)
    back = oracle.IFFT3Dr_f(f)
    np.testing.assert_allclose(back, a, atol=1e-5)


def test_f64_oracle_close_to_f32(golden, oracle):
    g = golden["pk"]
    delta = g["delta_d24"]
    r32 = oracle.Pk(delta, BOX, axis=2, MAS="CIC")
    r64 = oracle.Pk_f64(delta.astype(np.float64), BOX, axis=2, MAS="CIC")
    p0 = np.abs(r64.Pk[:, 0])
    assert np.max(np.abs(r32.Pk - r64.Pk).max(axis=1) / p0) < 1e-5
    assert np.array_equal(r32.Nmodes3D, r64.Nmodes3D)


def test_omp_deposit_matches_serial(oracle):
    rng = np.random.default_rng(9)
    pos = rng.random((20000, 3), dtype=np.float32) * np.float32(BOX)
    for MAS in ("NGP", "CIC", "TSC", "PCS"):
        a = np.zeros((20,) * 3, np.float32)
        b = np.zeros_like(a)
        oracle.MA(pos, a, BOX, MAS)
        oracle.deposit_omp(MAS, pos, b, BOX, threads=2)
        assert np.abs(a - b).max() < 1e-5


def test_f64_omp_deposit_matches_serial(oracle):
    """The all-cores float64 deposit adds the same taps as the serial one."""
    rng = np.random.default_rng(10)
    pos = rng.random((20000, 3), dtype=np.float32) * np.float32(BOX)
    W = rng.lognormal(0, 0.5, len(pos)).astype(np.float32)
    for MAS in ("NGP", "CIC", "TSC", "PCS"):
        for w in (None, W):
            a = oracle.MA_f64(pos, 20, BOX, MAS, W=w)
            b = oracle.MA_f64(pos, 20, BOX, MAS, W=w, threads=2)
            assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()


# ------------------------------------------------------------- next rows
@pytest.fixture(scope="module")
def nxt():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "next_golden.npz"))


@pytest.mark.parametrize("dims", [16, 17])
@pytest.mark.parametrize("MAS", ["CIC", "TSC", "PCS", "None"])
def test_correct_mas_matches_reference(nxt, oracle, dims, MAS):
    got = oracle.correct_MAS(nxt["cm_delta_d%d" % dims], BOX, MAS=MAS)
    want = nxt["cm_out_d%d_%s" % (dims, MAS)]
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


@pytest.mark.parametrize("grid", [16, 17, 32])
@pytest.mark.parametrize("MAS", ["NGP", "CIC", "PCS", "None"])
def test_pk_plane_matches_reference(nxt, oracle, grid, MAS):
    r = oracle.Pk_plane(nxt["pp_delta_g%d" % grid], BOX, MAS=MAS)
    np.testing.assert_array_equal(r.Nmodes, nxt["pp_Nmodes_g%d_%s" % (grid, MAS)])
    np.testing.assert_allclose(r.k, nxt["pp_k_g%d_%s" % (grid, MAS)], rtol=1e-12)
    np.testing.assert_allclose(r.Pk, nxt["pp_Pk_g%d_%s" % (grid, MAS)], rtol=1e-6)


@pytest.mark.parametrize("dims", [16, 17])
@pytest.mark.parametrize("axis", [0, 2])
def test_xpk_matches_reference(nxt, oracle, dims, axis):
    fields = [nxt["xp_delta%d_d%d" % (i, dims)] for i in range(3)]
    r = oracle.XPk(fields, BOX, axis=axis, MAS=["CIC", "PCS", "CIC"])
    for key in ("Nmodes3D", "Nmodes1D", "Nmodes2D"):
        np.testing.assert_array_equal(getattr(r, key), nxt["xp_%s_d%d_a%d" % (key, dims, axis)])
    for key in ("k3D", "k1D", "kpar", "kper"):
        np.testing.assert_allclose(getattr(r, key), nxt["xp_%s_d%d_a%d" % (key, dims, axis)],
                                   rtol=1e-12)
    scale = np.abs(nxt["xp_Pk_d%d_a%d" % (dims, axis)]).max()
    for key in ("Pk", "XPk", "Pk1D", "PkX1D", "Pk2D", "PkX2D"):
        want = nxt["xp_%s_d%d_a%d" % (key, dims, axis)]
        assert getattr(r, key).shape == want.shape, key
        assert np.abs(getattr(r, key) - want).max() <= 1e-6 * max(scale, np.abs(want).max()), key


@pytest.mark.parametrize("dims", [16, 17])
def test_cic_interp_matches_reference(nxt, oracle, dims):
    pos = nxt["ci_pos_d%d" % dims]
    den = np.zeros(len(pos), np.float32)
    oracle.CIC_interp(nxt["ci_grid_d%d" % dims], BOX, pos, den)
    want = nxt["ci_den_d%d" % dims]
    assert np.abs(den - want).max() <= 1e-6 * np.abs(want).max()
