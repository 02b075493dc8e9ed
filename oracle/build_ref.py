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

The machine that runs the GPU tests and the benchmark has gcc but no Cython
and no reference tree, so build() also stages a compile kit in
oracle/_ref/kit: the two Cython-generated C files and the two C files of the
reference's MAS_c module, as build inputs (oracle/_ref is git-ignored and is
not product source).  build_from_kit() compiles that kit with gcc alone,
with the same flags, into oracle/_ref/ for the machine it runs on.

Usage:  python oracle/build_ref.py [--ref <reference tree>]
        (default: $PYLIANS3_REFERENCE, else /root/reference)
"""
import argparse
import glob
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
KIT = os.path.join(OUT, "kit")
CFLAGS = ["-O3", "-ffast-math", "-march=native"]   # setup.py's extra_compile_args


def default_reference() -> str:
    """Where the reference tree is read (here only)."""
    return os.environ.get("PYLIANS3_REFERENCE", "/root/reference")


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
    stage_kit(mas_dir)


def stage_kit(mas_dir: str) -> None:
    """Copies the generated C and the MAS_c build inputs into oracle/_ref/kit."""
    os.makedirs(KIT, exist_ok=True)
    for name in ("MAS_library", "Pk_library"):
        gen = glob.glob(os.path.join(OUT, "gen", "**", name + ".c"), recursive=True)
        if len(gen) != 1:
            raise RuntimeError("generated %s.c not found under %s" % (name, OUT))
        shutil.copyfile(gen[0], os.path.join(KIT, name + ".c"))
    for name in ("MAS_c.c", "MAS_c.h"):
        shutil.copyfile(os.path.join(mas_dir, name), os.path.join(KIT, name))


def have_kit() -> bool:
    return all(os.path.exists(os.path.join(KIT, f))
               for f in ("MAS_library.c", "Pk_library.c", "MAS_c.c", "MAS_c.h"))


def built() -> bool:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return all(os.path.exists(os.path.join(OUT, n + suffix)) for n in ("MAS_library", "Pk_library"))


def build_from_kit() -> None:
    """Compiles oracle/_ref/kit with gcc (no Cython) into this machine's
    extension modules in oracle/_ref/: MAS_library (MAS_library.c + MAS_c.c,
    OpenMP at link time only, as the reference's Linux build ends up) and
    Pk_library, both with setup.py's flags, in parallel."""
    import numpy
    if not have_kit():
        raise RuntimeError("no reference compile kit in %s" % KIT)
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    inc = ["-I" + sysconfig.get_paths()["include"], "-I" + numpy.get_include(), "-I" + KIT]
    base = ["gcc", "-shared", "-fPIC", "-fno-strict-aliasing", "-DNDEBUG"] + CFLAGS + inc
    jobs = []
    for name, srcs, extra in (
            ("MAS_library", ["MAS_library.c", "MAS_c.c"], ["-fopenmp", "-lm", "-lgomp"]),
            ("Pk_library", ["Pk_library.c"], ["-lm"])):
        tmp = os.path.join(OUT, name + suffix + ".tmp%d" % os.getpid())
        cmd = base + [os.path.join(KIT, f) for f in srcs] + ["-o", tmp] + extra
        jobs.append((subprocess.Popen(cmd, stderr=subprocess.PIPE), tmp,
                     os.path.join(OUT, name + suffix)))
    for proc, tmp, dst in jobs:
        _, err = proc.communicate()
        if proc.returncode:
            raise RuntimeError("gcc failed for %s: %s" % (dst, err.decode()[-2000:]))
        os.replace(tmp, dst)


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
    ap.add_argument("--ref", default=default_reference())
    a = ap.parse_args()
    build(a.ref)
    MASL, PKL = load()
    print("built", MASL.__file__, PKL.__file__)
