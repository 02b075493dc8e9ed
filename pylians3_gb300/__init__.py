"""pylians3_gb300: Pylians3's density-field + power-spectrum hot path on GB300.

Drop-in modules (same API as the reference's):
    from pylians3_gb300 import MAS_library as MASL, Pk_library as PKL
    MASL.MA(pos, delta, BoxSize, 'CIC')
    P = PKL.Pk(delta, BoxSize, axis=0, MAS='CIC')
plus ``power_spectrum`` (particles -> spectrum with the grid kept on the
device), ``power_spectra`` (several particle sets, the upload of one
overlapping the computation of the previous) and ``pinned_empty`` (pinned
host buffers for fast transfers).
Every computation runs in libpylgpu.so on a CUDA device (sm_103a).
"""
from . import MAS_library, Pk_library  # noqa: F401
from ._native import Context, PylError, context, pinned_empty  # noqa: F401
from .pipeline import power_spectra, power_spectrum  # noqa: F401

__all__ = ["MAS_library", "Pk_library", "power_spectrum", "power_spectra", "pinned_empty",
           "Context", "PylError", "context"]
