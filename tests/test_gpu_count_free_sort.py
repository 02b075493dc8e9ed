"""The count-free tile sort of the fused particles path.

After an exact (counting) sort, the next request of the same dims, scheme
and weighting (in any context of the process) takes fixed slots sized from
the occupancy the exact sort saw, and needs no counting pass.  Checked
through the public API (sort="exact" forces the counting sort) and
pyl_ctx_last_sort:
  * on uniform input the count-free sort runs without spilling and gives the
    exact sort's spectrum to 1e-5 of P0 per bin up to the Nyquist wavenumber
    and 1e-4 beyond (the grid differs by float32 rounding: tile halos reach
    it through float reductions in any order);
  * on a coherent (displaced-lattice) input it takes the one-pass frontier
    form and again matches the exact sort;
  * when a request's tiles hold more than the slots allow (a clustered input
    after a uniform one), the overflow goes to the spill list, the spectrum
    still matches the oracle (per bin, 1e-4 of P0 up to the Nyquist
    wavenumber), and the next request takes the exact sort again.
"""
import numpy as np
import pytest

from gates import TOL_PK, per_bin_err

pytestmark = pytest.mark.gpu

BOX = 1000.0


@pytest.fixture(scope="module")
def P():
    import torch
    assert torch.cuda.is_available()
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    return P


def spectra(P, ctx, pos, dims, MAS, axis, W=None, sort="auto"):
    s = P.power_spectrum(pos, dims, BOX, MAS, axis=axis, W=W, ctx=ctx, sort=sort)
    return s, ctx.last_sort()


@pytest.mark.parametrize("MAS,weighted", [("CIC", False), ("TSC", True), ("PCS", False)])
def test_uniform_count_free_equals_exact(P, MAS, weighted):
    from pylians3_gb300 import _native, synth
    import torch
    ctx = _native.Context(0)
    dims = 256
    pos = synth.uniform(dims ** 3, BOX, seed=11)         # one work item per tile
    W = None
    if weighted:
        g = torch.Generator(device="cuda").manual_seed(12)
        W = torch.exp(0.5 * torch.randn(pos.shape[0], generator=g, device="cuda"))
    a, (cf0, _) = spectra(P, ctx, pos, dims, MAS, 0, W, sort="exact")   # learns the slots
    b, (cf1, sp1) = spectra(P, ctx, pos, dims, MAS, 0, W)
    c, (cf2, sp2) = spectra(P, ctx, pos, dims, MAS, 0, W)
    assert cf0 == 0 and cf1 == 1 and cf2 == 1 and sp1 == 0 and sp2 == 0
    assert np.array_equal(a.Nmodes3D, b.Nmodes3D)
    # the tiles' halos reach the grid through float reductions in any order
    # (in both sorts), and dense PCS tiles accumulate in float atomics:
    # float32 rounding of the grid, ~1e-7 of P0 up to the Nyquist wavenumber;
    # beyond it the PCS deconvolution amplifies it in bins of a few modes
    mid = dims // 2
    for x in (b, c):
        e = per_bin_err(x.Pk, a.Pk)
        assert e[:mid].max() <= 1e-5
        assert e.max() <= TOL_PK
    ctx.close()


def test_lattice_count_free_frontier_equals_exact(P):
    from pylians3_gb300 import _native, synth
    ctx = _native.Context(0)
    dims = 128
    pos = synth.zeldovich(dims, BOX, sigma=3.0, seed=5)      # lattice order: frontier sort
    a, (cf0, _) = spectra(P, ctx, pos, dims, "CIC", 2, sort="exact")
    b, (cf1, sp1) = spectra(P, ctx, pos, dims, "CIC", 2)
    assert cf0 == 0 and cf1 == 1 and sp1 == 0
    assert per_bin_err(b.Pk, a.Pk).max() <= 1e-5
    ctx.close()


def test_overflow_spills_and_falls_back(P, oracle):
    from pylians3_gb300 import _native, synth
    import torch
    ctx = _native.Context(0)
    dims, n = 128, 2 * 128 ** 3
    uni = synth.uniform(n, BOX, seed=21)
    spectra(P, ctx, uni, dims, "CIC", 1, sort="exact")       # learns uniform occupancy
    _, (cf, sp) = spectra(P, ctx, uni, dims, "CIC", 1)
    assert cf == 1 and sp == 0
    # the same size and scheme, but a third of the particles in 30 clumps
    rng = np.random.default_rng(9)
    pos = rng.random((n, 3), dtype=np.float32) * np.float32(BOX)
    k = n // 3
    centres = rng.random((30, 3)) * BOX
    pos[:k] = np.mod(centres[rng.integers(0, 30, k)] + rng.standard_normal((k, 3)) * 6.0,
                     BOX).astype(np.float32)
    clumped = torch.from_numpy(pos).cuda()
    s, (cf, sp) = spectra(P, ctx, clumped, dims, "CIC", 1)
    assert cf == 1 and sp > 0                                # slots overflowed
    ref_d = np.zeros((dims,) * 3, np.float32)
    oracle.MA(pos, ref_d, BOX, "CIC")
    ref_d /= np.mean(ref_d, dtype=np.float64)
    ref_d -= 1.0
    ref = oracle.Pk(ref_d, BOX, axis=1, MAS="CIC", threads=8)
    err = per_bin_err(s.Pk, ref.Pk)
    assert err[:dims // 2].max() <= TOL_PK
    assert np.array_equal(s.Nmodes3D, ref.Nmodes3D)
    t, (cf, sp) = spectra(P, ctx, clumped, dims, "CIC", 1)
    assert cf == 0 and sp == 0                               # back to the exact sort
    assert per_bin_err(t.Pk, ref.Pk)[:dims // 2].max() <= TOL_PK
    ctx.close()
