"""The per-bin parity gate (tests/gates.py) on the CPU: the 1e-4 floor, the
per-mode scaling with sqrt(Nmodes), and that the reference's own float32
path in one summation order passes the gate built from another order (the
gate is not tighter than the reference against itself)."""
import numpy as np

from gates import TOL_PK, check, float32_gate, per_bin_err

BOX = 1000.0


def test_floor_and_per_mode_scaling():
    # float32 noise of one per-mode level (5e-5) averaged over Nmodes modes
    n = np.array([1e6, 1e4, 100, 16, 4, 1])
    ref64 = np.ones((6, 3))
    ref32 = ref64.copy()
    ref32[:, 0] += 5e-5 / np.sqrt(n)
    g = float32_gate([ref32], ref64, n)
    assert np.allclose(g, np.maximum(TOL_PK, 8.0 * 5e-5 / np.sqrt(n)))
    # where the reference errs by more in one bin, its neighbours' gates follow
    ref32[2, 1] += 1e-4
    g2 = float32_gate([ref32], ref64, n)
    assert np.all(g2 >= g) and g2[-1] > g[-1]


def test_reference_orders_pass_each_others_gate(oracle):
    """PCS on 64^3 (its corner bins amplify float32 noise ~5e4-fold): the
    oracle's serial-order spectrum passes the gate built from its OpenMP
    order and the float64 restatement."""
    rng = np.random.default_rng(31)
    pos = rng.random((3 * 64 ** 3, 3), dtype=np.float32) * np.float32(BOX)
    spectra = []
    for dep in ("omp", "serial"):
        g = np.zeros((64,) * 3, np.float32)
        if dep == "omp":
            oracle.deposit_omp("PCS", pos, g, BOX, threads=4)
        else:
            oracle.MA(pos, g, BOX, "PCS")
        g /= np.mean(g, dtype=np.float64)
        g -= 1.0
        spectra.append(oracle.Pk(g, BOX, axis=1, MAS="PCS"))
    g64 = oracle.MA_f64(pos, 64, BOX, "PCS")
    g64 /= g64.mean()
    g64 -= 1.0
    ref64 = oracle.Pk_f64(g64, BOX, axis=1, MAS="PCS")
    omp, serial = spectra
    check(serial.Pk, omp.Pk, ref64.Pk, omp.Nmodes3D, "serial vs omp")
    assert per_bin_err(serial.Pk, omp.Pk)[:32].max() <= TOL_PK
