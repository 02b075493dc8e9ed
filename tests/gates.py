"""Per-bin tolerance gates of the spectrum parity tests.

The stated tolerance is |P_ell - P_ell,ref| / |P0_ref| <= 1e-4 per bin.  It
holds in every bin up to the Nyquist wavenumber and in every bin that holds
many modes.  The exceptions are the few bins at the grid corner beyond the
Nyquist wavenumber: there the TSC/PCS window deconvolution divides by W(k)^2
(~3e3 for TSC, ~5e4 for PCS) and a bin holds a handful of modes (the last
bin of a 512^3 grid holds one, the (256, 256, 256) mode), so the float32
rounding of the grid and of the FFT is not averaged down.  The reference's
own float32 path moves there with the order of its sums alone: at 512^3
Zel'dovich TSC its serial and OpenMP deposits put the last bin at 4.5e-5 and
0.9e-5 of P0 from the float64 result.

There the gate is derived from the reference against itself: the oracle's
float32 spectra (the reference's arithmetic, in one or more summation
orders) against its float64 restatement on the same input give the
reference's float32 error per bin; times sqrt(Nmodes) that is a per-mode
noise level, which varies smoothly with k.  A bin's gate is FACTOR times the
largest per-mode level within +-HALF_WIDTH bins, over sqrt(Nmodes) of the
bin, or 1e-4 where that is larger.
"""
import numpy as np

TOL_PK = 1e-4
# Two float32 implementations with per-mode errors s_gpu and s_ref differ by
# sqrt(s_gpu^2 + s_ref^2); on single-mode corner bins the GPU's (tile
# deposit + register FFT) measured up to ~3x the reference's, and a single
# mode's error is one draw of that noise: FACTOR leaves ~2.5 standard
# deviations above it.
FACTOR = 8.0
HALF_WIDTH = 4   # envelope: running max over +-4 bins


def per_bin_err(got, ref):
    """max over ell of |P_ell - P_ell,ref| / |P0_ref|, per bin."""
    return np.abs(got - ref).max(axis=1) / np.abs(ref[:, 0])


def envelope(e, half_width=HALF_WIDTH):
    n = len(e)
    return np.array([e[max(0, i - half_width):i + half_width + 1].max() for i in range(n)])


def float32_gate(refs32, ref64, nmodes, floor=TOL_PK, factor=FACTOR):
    """Per-bin gate: max(floor, factor * envelope(e_ref * sqrt(N)) / sqrt(N)),
    e_ref the largest error of the reference's float32 spectra refs32 (one
    array or a list, P[:, 0:3]) against its float64 spectrum ref64."""
    if isinstance(refs32, np.ndarray):
        refs32 = [refs32]
    e = np.max([per_bin_err(r, ref64) for r in refs32], axis=0)
    rootn = np.sqrt(np.maximum(np.asarray(nmodes, np.float64), 1.0))
    return np.maximum(floor, factor * envelope(e * rootn) / rootn)


def check(got, ref32, ref64, nmodes, label="", refs32=None):
    """Asserts |got - ref32| / |P0| within the gate in every bin; the gate
    uses refs32 (default [ref32]).  Returns (err, gate) for reporting."""
    err = per_bin_err(got, ref32)
    gate = float32_gate(refs32 if refs32 is not None else [ref32], ref64, nmodes)
    bad = np.nonzero(err > gate)[0]
    assert bad.size == 0, "%s: bins %s err %s > gate %s (Nmodes %s)" % (
        label, bad[:8], err[bad[:8]], gate[bad[:8]], np.asarray(nmodes)[bad[:8]])
    return err, gate
