"""Parity at the benchmarked sizes: per-bin spectra and bit-exact mode counts.

* 512^3 CIC, 2^27 uniform particles, axis 0 (the benchmarked spectrum) and
  512^3 Zel'dovich lattice (sigma 3 Mpc/h, RSD shift along z), TSC, axis 2:
  the fused particles -> spectrum path (what bench.py times) and the drop-in
  MA -> delta/mean - 1 -> Pk sequence on the device, against the oracle on
  the same seeded positions.  The oracle deposit is the reference's OpenMP
  one (MAS_c.c:8-266 restated; float32 atomics on all cores; its serial MA,
  MAS_library.pyx:123-166 / 369-404, is a second summation order for the
  gate), its overdensity and its Pk (Pk_library.pyx:311-418; mode-loop rows
  on all cores).  Mode
  counts are compared exactly, k3D to float64 rounding, and P_ell per bin
  against the gate of tests/gates.py: |dP_ell| / |P0| <= 1e-4, or a small
  multiple of the reference's own float32-vs-float64 error where that is
  larger (corner bins beyond the Nyquist wavenumber).
* Nmodes3D / Nmodes1D / Nmodes2D at dims 512 and 1024 (axes 0 and 2) against
  the oracle's integer mode counts, bit-exact; k3D and k1D to rtol 1e-12.
"""
import os

import numpy as np
import pytest

from gates import TOL_PK, check, float32_gate, per_bin_err

pytestmark = pytest.mark.gpu

BOX = 1000.0
NCPU = os.cpu_count() or 1


@pytest.fixture(scope="module")
def gpu():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    return P


@pytest.mark.parametrize("dims", [512, 1024])
@pytest.mark.parametrize("axis", [0, 2])
def test_mode_counts_bit_exact(gpu, oracle, dims, axis):
    import torch
    z = torch.zeros((dims,) * 3, device="cuda")
    r = gpu.Pk_library.Pk(z, BOX, axis=axis, MAS="CIC", verbose=False)
    del z
    torch.cuda.empty_cache()
    m = oracle.mode_counts(dims, axis)
    kF = 2.0 * np.pi / BOX
    assert np.array_equal(r.Nmodes3D, m["Nmodes3D"])
    assert np.array_equal(r.Nmodes1D, m["Nmodes1D"])
    assert np.array_equal(r.Nmodes2D, m["Nmodes2D"])
    np.testing.assert_allclose(r.k3D, m["k3D"] * kF, rtol=1e-12)
    np.testing.assert_allclose(r.k1D, m["k1D"] * kF, rtol=1e-12)


def _oracle_spectra(oracle, pos_np, dims, MAS, axis):
    """Oracle spectra of the same positions: float32 (the reference's
    arithmetic) with the OpenMP deposit (MAS_c.c) and with the serial one
    (MA), and float64 (the precision restatement)."""
    refs = []
    for dep in ("omp", "serial"):
        g = np.zeros((dims,) * 3, np.float32)
        if dep == "omp":
            oracle.deposit_omp(MAS, pos_np, g, BOX, threads=0)
        else:
            oracle.MA(pos_np, g, BOX, MAS)
        g /= np.mean(g, dtype=np.float64)
        g -= 1.0
        refs.append(oracle.Pk(g, BOX, axis=axis, MAS=MAS, threads=NCPU, bin_threads=0))
        del g
    g64 = oracle.MA_f64(pos_np, dims, BOX, MAS, threads=0)
    g64 /= g64.mean()
    g64 -= 1.0
    ref64 = oracle.Pk_f64(g64, BOX, axis=axis, MAS=MAS, threads=NCPU, bin_threads=0)
    return refs, ref64


def _compare(gpu, oracle, pos, dims, MAS, axis, label):
    import torch
    fused = gpu.power_spectrum(pos, dims, BOX, MAS, axis=axis)
    grid = torch.zeros((dims,) * 3, device="cuda")
    gpu.MAS_library.MA(pos, grid, BOX, MAS)
    grid /= grid.double().mean().float()
    grid -= 1.0
    dropin = gpu.Pk_library.Pk(grid, BOX, axis=axis, MAS=MAS, verbose=False)
    del grid
    pos_np = pos.cpu().numpy()
    torch.cuda.empty_cache()
    refs, ref64 = _oracle_spectra(oracle, pos_np, dims, MAS, axis)
    ref32 = refs[0]
    for name, r in (("fused", fused), ("drop-in", dropin)):
        assert np.array_equal(r.Nmodes3D, ref32.Nmodes3D), name
        np.testing.assert_allclose(r.k3D, ref32.k3D, rtol=1e-12)
        err = per_bin_err(r.Pk, ref32.Pk)
        mid = dims // 2
        e_ref = np.max([per_bin_err(q.Pk, ref64.Pk) for q in refs], axis=0)
        gate = float32_gate([q.Pk for q in refs], ref64.Pk, ref32.Nmodes3D)
        print("\n%s %s: max err <= k_N %.2e, all bins %.2e (bins > 1e-4: %d; last bin %.2e, "
              "gate %.2e, Nmodes %d); reference float32 vs float64: <= k_N %.2e, all %.2e, "
              "bins > 1e-4: %d"
              % (label, name, err[:mid].max(), err.max(), int((err > TOL_PK).sum()), err[-1],
                 gate[-1], int(ref32.Nmodes3D[-1]), e_ref[:mid].max(), e_ref.max(),
                 int((e_ref > TOL_PK).sum())))
        check(r.Pk, ref32.Pk, ref64.Pk, ref32.Nmodes3D, "%s %s" % (label, name),
              refs32=[q.Pk for q in refs])
        # up to the Nyquist wavenumber the flat tolerance holds everywhere
        assert err[:mid].max() <= TOL_PK


def test_headline_512_cic_uniform_axis0(gpu, oracle):
    from pylians3_gb300 import synth
    pos = synth.uniform(512 ** 3, BOX, seed=1234)    # the benchmark's seeded positions
    _compare(gpu, oracle, pos, 512, "CIC", 0, "512^3 CIC uniform axis 0")


def test_c2_512_zeldovich_rsd_tsc_axis2(gpu, oracle):
    from pylians3_gb300 import synth
    pos = synth.zeldovich(512, BOX, sigma=3.0, seed=1234)
    _compare(gpu, oracle, pos, 512, "TSC", 2, "512^3 Zel'dovich+RSD TSC axis 2")
