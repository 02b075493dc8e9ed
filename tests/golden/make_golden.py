"""Generate the golden vectors in tests/golden/ from the compiled reference.

Run here, where the reference sources are readable:
    python oracle/build_ref.py            # compiles the reference into oracle/_ref
    python tests/golden/make_golden.py    # writes tests/golden/*.npz

Every fixture stores its inputs next to the reference's outputs, so that the
tests never need the reference (or the random generator that made the
inputs) at run time.  Inputs are small and seeded:

  ma_golden.npz        MA(pos, grid, BoxSize, MAS, W) for MAS in NGP/CIC/TSC/PCS,
                       with and without weights, dims 16 (even) and 17 (odd),
                       3D and 2D, uniform positions plus edge-case positions
                       (0, exact cell edges, BoxSize - ulp, BoxSize).
                       [library/MAS_library/MAS_library.pyx:57-545]
  pk_golden.npz        Pk(delta, BoxSize, axis, MAS) for dims 16, 17, 24,
                       MAS in NGP/CIC/TSC/PCS/None, axis 0/1/2: k3D, Pk,
                       Nmodes3D, k1D, Pk1D, Nmodes1D, kpar, kper, Pk2D,
                       Nmodes2D, Pkphase.  [Pk_library.pyx:263-418]
  nmodes_golden.npz    Nmodes3D and k3D for dims 8, 9, 63, 64, 128, 192, 256
                       (the bit-exact mode-count / k-binning known answers).
  pipeline_golden.npz  The canonical caller in miniature (Pk_snapshot.py:81-89):
                       uniform positions -> MA CIC -> delta/mean-1 -> Pk,
                       dims 32, axis 0.
  next_golden.npz      The rows around the spectrum: correct_MAS (dims 16, 17;
                       CIC/TSC/PCS/None) [Pk_library.pyx:1882-1939], Pk_plane
                       (grid 16, 17, 32; NGP/CIC/PCS/None) [:435-511], XPk of
                       three fields with mixed schemes (dims 16, 17; axis 0, 2)
                       [:529-735], CIC_interp (dims 16, 17; uniform and edge
                       positions) [MAS_library.pyx:558-599].
                       `python tests/golden/make_golden.py next` writes only it.
The reference's Pk calls pyFFTW; here it runs on the scipy.fft stand-in in
oracle/pyfftw_shim (float32 in, complex64 out, as FFTW3f).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402

BOX = 1000.0
PK_KEYS = ("k3D", "Pk", "Nmodes3D", "k1D", "Pk1D", "Nmodes1D", "kpar", "kper",
           "Pk2D", "Nmodes2D", "Pkphase")


def edge_positions(dims, coord):
    cell = np.float32(BOX) / np.float32(dims)
    vals = np.array([0.0, cell, 0.5 * cell, 1.5 * cell, 2.5 * cell,
                     np.nextafter(np.float32(BOX), np.float32(0)),
                     (dims - 1) * cell, (dims - 0.5) * cell], np.float32)
    g = np.stack(np.meshgrid(*([vals] * coord), indexing="ij"), -1)
    return g.reshape(-1, coord).astype(np.float32)


def main():
    if not build_ref.built():
        build_ref.build(build_ref.default_reference())   # $PYLIANS3_REFERENCE or the default
    MASL, PKL = build_ref.load()
    rng = np.random.default_rng(20261203)

    # ---------------- MA ----------------
    out = {}
    for dims in (16, 17):
        for coord in (3, 2):
            n = 6000 if coord == 3 else 3000
            pos = (rng.random((n, coord), dtype=np.float32) * np.float32(BOX))
            pos = np.concatenate([pos, edge_positions(dims, coord)]).astype(np.float32)
            W = rng.lognormal(0.0, 0.5, len(pos)).astype(np.float32)
            tag = "d%d_c%d" % (dims, coord)
            out["pos_" + tag] = pos
            out["W_" + tag] = W
            for MAS in ("NGP", "CIC", "TSC", "PCS"):
                for wt in (0, 1):
                    g = np.zeros((dims,) * coord, np.float32)
                    MASL.MA(pos, g, BOX, MAS, W=W if wt else None)
                    out["grid_%s_%s_w%d" % (tag, MAS, wt)] = g
    np.savez_compressed(os.path.join(HERE, "ma_golden.npz"), **out)

    # ---------------- Pk ----------------
    out = {}
    for dims in (16, 17, 24):
        delta = rng.standard_normal((dims,) * 3).astype(np.float32)
        out["delta_d%d" % dims] = delta
        for MAS in ("NGP", "CIC", "TSC", "PCS", "None"):
            for axis in (0, 1, 2):
                r = PKL.Pk(delta, BOX, axis=axis, MAS=MAS, threads=1, verbose=False)
                for k in PK_KEYS:
                    out["%s_d%d_%s_a%d" % (k, dims, MAS, axis)] = np.asarray(getattr(r, k))
    np.savez_compressed(os.path.join(HERE, "pk_golden.npz"), **out)

    # ---------------- Nmodes / k3D KAT ----------------
    out = {}
    for dims in (8, 9, 63, 64, 128, 192, 256):
        z = np.zeros((dims,) * 3, np.float32)
        r = PKL.Pk(z, BOX, axis=2, MAS="CIC", threads=os.cpu_count(), verbose=False)
        out["Nmodes3D_d%d" % dims] = np.asarray(r.Nmodes3D)
        out["k3D_d%d" % dims] = np.asarray(r.k3D)
        out["Nmodes1D_d%d" % dims] = np.asarray(r.Nmodes1D)
        out["Nmodes2D_d%d" % dims] = np.asarray(r.Nmodes2D)
    np.savez_compressed(os.path.join(HERE, "nmodes_golden.npz"), **out)

    # ---------------- canonical pipeline ----------------
    dims = 32
    pos = rng.random((dims ** 3, 3), dtype=np.float32) * np.float32(BOX)
    delta = np.zeros((dims,) * 3, np.float32)
    MASL.MA(pos, delta, BOX, "CIC")
    delta /= np.mean(delta, dtype=np.float64)
    delta -= 1.0
    r = PKL.Pk(delta, BOX, axis=0, MAS="CIC", threads=1, verbose=False)
    out = {"pos": pos, "delta": delta}
    for k in PK_KEYS:
        out[k] = np.asarray(getattr(r, k))
    np.savez_compressed(os.path.join(HERE, "pipeline_golden.npz"), **out)
    next_rows(MASL, PKL)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


XPK_KEYS = ("k3D", "Pk", "XPk", "Nmodes3D", "k1D", "Pk1D", "PkX1D", "Nmodes1D", "kpar",
            "kper", "Pk2D", "PkX2D", "Nmodes2D")


def next_rows(MASL, PKL):
    rng = np.random.default_rng(20261204)
    out = {}
    # correct_MAS
    for dims in (16, 17):
        delta = rng.standard_normal((dims,) * 3).astype(np.float32)
        out["cm_delta_d%d" % dims] = delta
        for MAS in ("CIC", "TSC", "PCS", "None"):
            out["cm_out_d%d_%s" % (dims, MAS)] = np.asarray(
                PKL.correct_MAS(delta, BOX, MAS=MAS, threads=1))
    # Pk_plane
    for grid in (16, 17, 32):
        delta = rng.standard_normal((grid, grid)).astype(np.float32)
        out["pp_delta_g%d" % grid] = delta
        for MAS in ("NGP", "CIC", "PCS", "None"):
            r = PKL.Pk_plane(delta, BOX, MAS=MAS, threads=1, verbose=False)
            for k in ("k", "Pk", "Nmodes"):
                out["pp_%s_g%d_%s" % (k, grid, MAS)] = np.asarray(getattr(r, k))
    # XPk: three fields, the third correlated with the first
    for dims in (16, 17):
        a = rng.standard_normal((dims,) * 3).astype(np.float32)
        b = rng.standard_normal((dims,) * 3).astype(np.float32)
        c = (0.5 * a + 0.5 * rng.standard_normal((dims,) * 3)).astype(np.float32)
        for i, f in enumerate((a, b, c)):
            out["xp_delta%d_d%d" % (i, dims)] = f
        for axis in (0, 2):
            r = PKL.XPk([a, b, c], BOX, axis=axis, MAS=["CIC", "PCS", "CIC"], threads=1)
            for k in XPK_KEYS:
                out["xp_%s_d%d_a%d" % (k, dims, axis)] = np.asarray(getattr(r, k))
    # CIC_interp
    for dims in (16, 17):
        grid = rng.standard_normal((dims,) * 3).astype(np.float32)
        pos = (rng.random((4000, 3), dtype=np.float32) * np.float32(BOX))
        pos = np.concatenate([pos, edge_positions(dims, 3)]).astype(np.float32)
        den = np.zeros(len(pos), np.float32)
        MASL.CIC_interp(grid, BOX, pos, den)
        out["ci_grid_d%d" % dims] = grid
        out["ci_pos_d%d" % dims] = pos
        out["ci_den_d%d" % dims] = den
    np.savez_compressed(os.path.join(HERE, "next_golden.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "next":
        next_rows(*build_ref.load())
    else:
        main()
