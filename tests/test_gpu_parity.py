"""GPU parity: libpylgpu (through the drop-in API / C ABI) vs the golden
vectors of the reference and vs the CPU oracle on the same seeded inputs.

Tolerances (stated per check):
  * Nmodes / k-bin counts: bit-exact.  k3D: float64 rounding (rtol 1e-12).
  * grids: float32 rounding of a different summation order
    (|diff| <= 1e-5 * max(1, |value|)).
  * Pk multipoles per bin: |P_ell - P_ell,ref| / |P0_ref| <= 1e-4; beyond
    the Nyquist wavenumber of a GPU-deposited grid, the gate of
    tests/gates.py (a multiple of the reference's own float32 error).
"""
import numpy as np
import pytest

from gates import check, per_bin_err

pytestmark = pytest.mark.gpu

BOX = 1000.0
TOL_PK = 1e-4


@pytest.fixture(scope="module")
def gpu():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    return P


def pk_err(got, ref):
    return float((np.abs(got - ref).max(axis=1) / np.abs(ref[:, 0])).max())


def grid_ok(got, ref, tol=1e-5):
    return float(np.abs(got - ref).max()) <= tol * max(1.0, float(np.abs(ref).max()))


# ------------------------------------------------------------------ deposit
@pytest.mark.parametrize("dims", [16, 17])
@pytest.mark.parametrize("coord", [3, 2])
@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS"])
@pytest.mark.parametrize("wt", [0, 1])
def test_ma_golden(gpu, golden, dims, coord, MAS, wt):
    g = golden["ma"]
    tag = "d%d_c%d" % (dims, coord)
    pos, W = g["pos_" + tag], g["W_" + tag]
    ref = g["grid_%s_%s_w%d" % (tag, MAS, wt)]
    grid = np.zeros((dims,) * coord, np.float32)
    gpu.MAS_library.MA(pos, grid, BOX, MAS, W=W if wt else None)
    assert grid_ok(grid, ref)


@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS"])
@pytest.mark.parametrize("wt", [0, 1])
def test_ma_vs_oracle_64(gpu, oracle, MAS, wt):
    rng = np.random.default_rng(11)
    pos = rng.random((300000, 3), dtype=np.float32) * np.float32(BOX)
    W = rng.lognormal(0, 0.5, len(pos)).astype(np.float32) if wt else None
    a = np.zeros((64,) * 3, np.float32)
    b = np.zeros_like(a)
    gpu.MAS_library.MA(pos, a, BOX, MAS, W=W)
    oracle.MA(pos, b, BOX, MAS, W=W)
    assert grid_ok(a, b)
    mass = float(W.sum(dtype=np.float64)) if wt else float(len(pos))
    assert abs(a.sum(dtype=np.float64) / mass - 1) < 1e-5


def test_ma_accumulates_and_torch_path(gpu, oracle):
    import torch
    rng = np.random.default_rng(12)
    pos = rng.random((50000, 3), dtype=np.float32) * np.float32(BOX)
    a = np.ones((32,) * 3, np.float32)
    gpu.MAS_library.MA(pos, a, BOX, "TSC")
    gpu.MAS_library.MA(pos, a, BOX, "TSC")
    b = np.zeros_like(a)
    oracle.MA(pos, b, BOX, "TSC")
    assert grid_ok(a, 1 + 2 * b)
    t = torch.zeros((32,) * 3, dtype=torch.float32, device="cuda")
    gpu.MAS_library.MA(torch.from_numpy(pos).cuda(), t, BOX, "TSC")
    assert grid_ok(t.cpu().numpy(), b)


def test_ma_f64_grid(gpu, oracle):
    rng = np.random.default_rng(13)
    pos = rng.random((40000, 3), dtype=np.float32) * np.float32(BOX)
    W = rng.random(len(pos), dtype=np.float32)
    for name, MAS in (("CICW_d", "CIC"), ("NGPW_d", "NGP")):
        a = np.zeros((24,) * 3, np.float64)
        getattr(gpu.MAS_library, name)(pos, a, BOX, W)
        b = np.zeros_like(a)
        oracle.MA(pos, b, BOX, MAS, W=W)
        assert np.abs(a - b).max() < 1e-9 * max(1, np.abs(b).max())


def test_ma_edge_positions(gpu, oracle):
    """Cell edges, 0 and BoxSize land in the reference's cells."""
    dims = 16
    cell = np.float32(BOX) / np.float32(dims)
    vals = np.array([0, cell, 2 * cell, 0.5 * cell, 1.5 * cell,
                     np.nextafter(np.float32(BOX), np.float32(0)), BOX,
                     np.nextafter(0.5 * cell, np.float32(0))], np.float32)
    pos = np.stack(np.meshgrid(vals, vals, vals, indexing="ij"), -1).reshape(-1, 3)
    for MAS in ("NGP", "CIC", "TSC", "PCS"):
        a = np.zeros((dims,) * 3, np.float32)
        b = np.zeros_like(a)
        gpu.MAS_library.MA(pos, a, BOX, MAS)
        oracle.MA(pos, b, BOX, MAS)
        assert grid_ok(a, b), MAS


# ------------------------------------------------------------------ spectra
@pytest.mark.parametrize("dims", [16, 17, 24])
@pytest.mark.parametrize("MAS", ["NGP", "CIC", "TSC", "PCS", "None"])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_pk_golden(gpu, golden, dims, MAS, axis):
    g = golden["pk"]
    delta = g["delta_d%d" % dims]
    r = gpu.Pk_library.Pk(delta, BOX, axis=axis, MAS=MAS, verbose=False)
    key = lambda k: "%s_d%d_%s_a%d" % (k, dims, MAS, axis)
    for k in ("Nmodes3D", "Nmodes1D", "Nmodes2D"):
        assert np.array_equal(getattr(r, k), g[key(k)]), k
    np.testing.assert_allclose(r.k3D, g[key("k3D")], rtol=1e-12)
    np.testing.assert_allclose(r.k1D, g[key("k1D")], rtol=1e-12)
    np.testing.assert_allclose(r.kpar, g[key("kpar")], rtol=1e-15)
    np.testing.assert_allclose(r.kper, g[key("kper")], rtol=1e-15)
    assert pk_err(r.Pk, g[key("Pk")]) <= TOL_PK
    # the last 1D bin (k_par = kN) is 0 * (kN^2 - k^2): compare with a scale
    ref1 = g[key("Pk1D")]
    assert np.all(np.abs(r.Pk1D - ref1) <= TOL_PK * np.abs(ref1) + 1e-12 * np.abs(ref1).max())
    ref2 = g[key("Pk2D")]
    fin = np.isfinite(ref2)
    assert np.array_equal(fin, np.isfinite(r.Pk2D))
    assert np.all(np.abs(r.Pk2D[fin] - ref2[fin]) <= TOL_PK * np.abs(ref2[fin]) + 1e-12)
    np.testing.assert_allclose(r.Pkphase, g[key("Pkphase")], rtol=TOL_PK)


@pytest.mark.parametrize("dims", [8, 9, 63, 64, 128, 192, 256])
def test_nmodes_known_answers(gpu, golden, dims):
    g = golden["nmodes"]
    z = np.zeros((dims,) * 3, np.float32)
    r = gpu.Pk_library.Pk(z, BOX, axis=2, MAS="CIC", verbose=False)
    assert np.array_equal(r.Nmodes3D, g["Nmodes3D_d%d" % dims])
    assert np.array_equal(r.Nmodes1D, g["Nmodes1D_d%d" % dims])
    assert np.array_equal(r.Nmodes2D, g["Nmodes2D_d%d" % dims])
    np.testing.assert_allclose(r.k3D, g["k3D_d%d" % dims], rtol=1e-12)


def test_pipeline_golden(gpu, golden):
    g = golden["pipeline"]
    dims = g["delta"].shape[0]
    delta = np.zeros((dims,) * 3, np.float32)
    gpu.MAS_library.MA(g["pos"], delta, BOX, "CIC")
    delta /= np.mean(delta, dtype=np.float64)
    delta -= 1.0
    r = gpu.Pk_library.Pk(delta, BOX, axis=0, MAS="CIC", verbose=False)
    assert pk_err(r.Pk, g["Pk"]) <= TOL_PK
    assert np.array_equal(r.Nmodes3D, g["Nmodes3D"])
    # fused particles -> spectrum path
    s = gpu.power_spectrum(g["pos"], dims, BOX, "CIC", axis=0)
    assert pk_err(s.Pk, g["Pk"]) <= TOL_PK
    np.testing.assert_allclose(s.k3D, g["k3D"], rtol=1e-12)


@pytest.mark.parametrize("MAS,axis", [("CIC", 0), ("TSC", 2), ("PCS", 1), ("NGP", 2)])
def test_small_plain_config_vs_oracle(gpu, oracle, MAS, axis):
    """128^3 uniform particles -> 128^3 grid -> delta/mean-1 -> Pk (the small
    plain configuration) against the oracle on the same seeded input."""
    rng = np.random.default_rng(2026)
    pos = rng.random((128 ** 3, 3), dtype=np.float32) * np.float32(BOX)
    ref_d = np.zeros((128,) * 3, np.float32)
    oracle.MA(pos, ref_d, BOX, MAS)
    ref_d /= np.mean(ref_d, dtype=np.float64)
    ref_d -= 1.0
    ref = oracle.Pk(ref_d, BOX, axis=axis, MAS=MAS, threads=8)
    d = np.zeros((128,) * 3, np.float32)
    gpu.MAS_library.MA(pos, d, BOX, MAS)
    d /= np.mean(d, dtype=np.float64)
    d -= 1.0
    r = gpu.Pk_library.Pk(d, BOX, axis=axis, MAS=MAS, verbose=False)
    assert pk_err(r.Pk, ref.Pk) <= TOL_PK
    assert np.array_equal(r.Nmodes3D, ref.Nmodes3D)
    s = gpu.power_spectrum(pos, 128, BOX, MAS, axis=axis)
    assert pk_err(s.Pk, ref.Pk) <= TOL_PK


@pytest.mark.parametrize("dims", [48, 96, 192])
@pytest.mark.parametrize("MAS,axis", [("CIC", 0), ("PCS", 2)])
def test_pk_3x2k_lengths_vs_oracle(gpu, oracle, dims, MAS, axis):
    """Grids of 3 * 2^k cells take the radix-3 register FFT: Pk of the same
    seeded overdensity and the fused particles path against the oracle."""
    rng = np.random.default_rng(dims + 7)
    pos = rng.random((4 * dims ** 3, 3), dtype=np.float32) * np.float32(BOX)
    ref_d = np.zeros((dims,) * 3, np.float32)
    oracle.MA(pos, ref_d, BOX, MAS)
    ref_d /= np.mean(ref_d, dtype=np.float64)
    ref_d -= 1.0
    ref = oracle.Pk(ref_d, BOX, axis=axis, MAS=MAS, threads=8)
    r = gpu.Pk_library.Pk(ref_d, BOX, axis=axis, MAS=MAS, verbose=False)
    assert pk_err(r.Pk, ref.Pk) <= TOL_PK
    assert np.array_equal(r.Nmodes3D, ref.Nmodes3D)
    np.testing.assert_allclose(r.Pk1D, ref.Pk1D, rtol=TOL_PK, atol=TOL_PK * np.abs(ref.Pk1D).max())
    # The fused path deposits on the GPU: float32 sums in another order than
    # the oracle's (as the reference's own OpenMP deposit does from run to
    # run).  That order noise is white on the grid and the PCS window
    # deconvolution amplifies it up to ~5e4-fold at the grid corner: bins up
    # to the Nyquist wavenumber (|k| <= dims/2) are held to TOL_PK, the corner
    # bins beyond it to the gate derived from the reference's own float32
    # error (tests/gates.py: the oracle's float32 spectrum against its
    # float64 one on the same particles, in several of the reference's own
    # float32 summation orders: the serial MA and the OpenMP deposit of
    # MAS_c.c on all cores and on 2, 3 and 5 threads).  In the single-mode
    # corner bin of 192^3 PCS those orders alone scatter from 1e-4 to 2.5e-3
    # of P0 against float64, so the gate takes the envelope over all of them.
    s = gpu.power_spectrum(pos, dims, BOX, MAS, axis=axis)
    err = per_bin_err(s.Pk, ref.Pk)
    assert err[:dims // 2 + 1].max() <= TOL_PK
    refs32 = [ref.Pk]
    for nt in (0, 2, 3, 5):
        omp_d = np.zeros((dims,) * 3, np.float32)
        oracle.deposit_omp(MAS, pos, omp_d, BOX, threads=nt)
        omp_d /= np.mean(omp_d, dtype=np.float64)
        omp_d -= 1.0
        refs32.append(oracle.Pk(omp_d, BOX, axis=axis, MAS=MAS, threads=8).Pk)
    g64 = oracle.MA_f64(pos, dims, BOX, MAS, threads=0)
    g64 /= g64.mean()
    g64 -= 1.0
    ref64 = oracle.Pk_f64(g64, BOX, axis=axis, MAS=MAS, threads=8)
    check(s.Pk, ref.Pk, ref64.Pk, ref.Nmodes3D, "fused %d^3 %s" % (dims, MAS), refs32=refs32)


# ------------------------------------------------------------------ FFTs
@pytest.mark.parametrize("dims", [8, 16, 17, 24, 48, 61, 64, 96, 100, 128, 192, 384])
def test_fft_r2c_c2r(gpu, dims):
    rng = np.random.default_rng(dims)
    a = rng.standard_normal((dims,) * 3).astype(np.float32)
    f = gpu.Pk_library.FFT3Dr_f(a, 1)
    ref = np.fft.rfftn(a.astype(np.float64))
    scale = np.sqrt(np.mean(np.abs(ref) ** 2))
    assert f.shape == ref.shape and f.dtype == np.complex64
    assert np.abs(f - ref).max() / scale < 2e-5
    back = gpu.Pk_library.IFFT3Dr_f(f, 1)
    assert np.abs(back - a).max() < 2e-5
    # c2r of an arbitrary (non-Hermitian) half spectrum follows pocketfft/FFTW
    import scipy.fft as sf
    z = (rng.standard_normal(f.shape) + 1j * rng.standard_normal(f.shape)).astype(np.complex64)
    got = gpu.Pk_library.IFFT3Dr_f(z, 1)
    want = sf.irfftn(z.astype(np.complex128), s=(dims,) * 3, axes=(0, 1, 2))
    assert np.abs(got - want).max() < 2e-5 * max(1.0, np.abs(want).max())


def test_fft_torch_zero_copy(gpu):
    import torch
    a = torch.randn((32, 32, 32), device="cuda")
    f = gpu.Pk_library.FFT3Dr_f(a, 1)
    ref = torch.fft.rfftn(a.double())     # cuFFT, as an oracle only
    assert f.is_cuda and f.dtype == torch.complex64
    assert (f.cdouble() - ref).abs().max().item() / ref.abs().pow(2).mean().sqrt().item() < 2e-5
    back = gpu.Pk_library.IFFT3Dr_f(f, 1)
    assert (back - a).abs().max().item() < 2e-5


@pytest.mark.parametrize("dims", [256, 512])
def test_fft_headline_sizes(gpu, dims):
    """r2c and c2r at the grid sizes of the benchmarked spectra, against a
    float64 cuFFT transform (test oracle only).  A float32 FFT's error here
    is ~1e-6 of the rms (forward) and ~2e-6 (round trip)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(dims)
    a = torch.randn((dims,) * 3, generator=g, device="cuda")
    f = gpu.Pk_library.FFT3Dr_f(a, 1)
    ref = torch.fft.rfftn(a.double())
    assert (f.cdouble() - ref).abs().max().item() / ref.abs().pow(2).mean().sqrt().item() < 2e-5
    del ref
    back = gpu.Pk_library.IFFT3Dr_f(f, 1)
    assert (back - a).abs().max().item() < 2e-5


# ------------------------------------------------------- large properties
def test_512_cic_mass_conservation(gpu):
    """Full-size headline deposit (512^3 grid, 2^27 particles): the deposited
    mass equals the particle count (library/tests/test.py:30-33 checks the
    same to 1e-5).  Per-bin spectrum parity at this size is in
    test_gpu_headline_parity.py."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(5)
    pos = torch.rand((512 ** 3, 3), generator=g, device="cuda") * BOX
    grid = torch.zeros((512,) * 3, device="cuda")
    gpu.MAS_library.MA(pos, grid, BOX, "CIC")
    assert abs(grid.double().sum().item() / 512 ** 3 - 1) < 1e-5
