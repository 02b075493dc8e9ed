"""Stand-in for the ``pyfftw`` module, used only to import the reference's
compiled Pk_library here (oracle/build_ref.py) -- test infrastructure.

The reference calls ``pyfftw.empty_aligned`` and ``pyfftw.FFTW(a_in, a_out,
axes, flags, direction, threads)`` (library/Pk_library/Pk_library.pyx:117-245)
and then ``plan(a_in, a_out)``.  pyFFTW/FFTW3 is not installed (pinned
nowhere: setup.py lists an unversioned ``pyfftw``).  This module reproduces
the published conventions of those calls on top of scipy.fft (pocketfft),
computing in the input's precision:
  * forward r2c over ``axes``, unnormalised;
  * backward c2r over ``axes`` normalised by 1/N (pyFFTW's
    ``FFTW.__call__`` defaults to ``normalise_idft=True``).
"""
import numpy as np
import scipy.fft as _sf


def empty_aligned(shape, dtype="float32", n=None):
    return np.empty(shape, dtype=dtype)


class FFTW:
    def __init__(self, a_in, a_out, axes=(0, 1, 2), flags=(),
                 direction="FFTW_FORWARD", threads=1):
        self.axes = tuple(axes)
        self.direction = direction
        self.threads = max(1, int(threads))

    def __call__(self, a_in, a_out):
        if self.direction == "FFTW_FORWARD":
            a_out[...] = _sf.rfftn(a_in, axes=self.axes, workers=self.threads)
        else:
            shape = [a_out.shape[ax] for ax in self.axes]
            a_out[...] = _sf.irfftn(a_in, s=shape, axes=self.axes,
                                    workers=self.threads)
        return a_out
