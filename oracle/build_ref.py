"""Compile the reference's own hot-path sources into oracle/_ref/ (here only).

TEST INFRASTRUCTURE: the compiled reference is used to pin the CPU
restatement (oracle/pyl_oracle.c, oracle/oracle.py) and to generate the
golden vectors under tests/golden/.  Nothing in the product imports it.

The sources are read where they lie in the read-only reference tree:
  library/MAS_library/MAS_library.pyx + MAS_c.c (+ MAS_c.pxd, MAS_c.h)
  library/Pk_library/Pk_library.pyx
with the flags of the reference's setup.py:25-34 (-O3 -ffast-math
-march=native; OpenMP at link time only, as upstream's Linux build ends up,
setup.py:15-23).  Cython writes its generated C into oracle/_ref/gen and the
extension modules land in oracle/_ref/ as top-level ``MAS_library`` and
``Pk_library`` (skipping the package __init__ files, which import the
snapshot readers).  Pk_library imports ``pyfftw``: put oracle/pyfftw_shim on
sys.path before importing it.

Usage:  python oracle/build_ref.py [--ref /root/reference]
"""
import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def build(ref: str) -> None:
    import numpy
    from Cython.Build import cythonize
    from setuptools import Extension
    from setuptools.dist import Distribution

    mas_dir = os.path.join(ref, "library", "MAS_library")
    pk_dir = os.path.join(ref, "library", "Pk_library")
    cflags = ["-O3", "-ffast-math", "-march=native"]
    exts = [
        Extension("MAS_library",
                  [os.path.join(mas_dir, "MAS_library.pyx"),
                   os.path.join(mas_dir, "MAS_c.c")],
                  include_dirs=[numpy.get_include(), mas_dir],
                  extra_compile_args=cflags, extra_link_args=["-fopenmp"],
                  libraries=["m", "gomp"]),
        Extension("Pk_library", [os.path.join(pk_dir, "Pk_library.pyx")],
                  include_dirs=[numpy.get_include()],
                  extra_compile_args=cflags),
    ]
    os.makedirs(OUT, exist_ok=True)
    exts = cythonize(exts, build_dir=os.path.join(OUT, "gen"),
                     include_path=[mas_dir], quiet=True,
                     compiler_directives={"language_level": 3,
                                          "legacy_implicit_noexcept": True})
    dist = Distribution({"name": "pylians_ref_oracle", "ext_modules": exts})
    cmd = dist.get_command_obj("build_ext")
    cmd.build_lib = OUT
    cmd.build_temp = os.path.join(OUT, "tmp")
    cmd.parallel = os.cpu_count()
    cmd.ensure_finalized()
    cmd.run()


def load():
    """Import the compiled reference modules (after build())."""
    for p in (OUT, os.path.join(HERE, "pyfftw_shim")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import MAS_library  # noqa: E402
    import Pk_library  # noqa: E402
    return MAS_library, Pk_library


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    a = ap.parse_args()
    build(a.ref)
    MASL, PKL = load()
    print("built", MASL.__file__, PKL.__file__)
