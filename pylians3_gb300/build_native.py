"""Build libpylgpu.so in-tree: every CUDA source compiled for sm_103a only.

    python -m pylians3_gb300.build_native        # or __graft_entry__.build()

Translation units are compiled in parallel with nvcc (one -gencode, no
cmake) into pylians3_gb300/_build/ and linked into pylians3_gb300/libpylgpu.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
SO = os.path.join(PKG, "libpylgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: the host-side finalisation evaluates the reference's
# float64 formulas operation by operation (gcc contracts a*b-c into an FMA by
# default on aarch64, which changes e.g. sqrt(kN^2 - k^2) at kN == k).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpylgpu")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "pylgpu.h"))
    return max(os.path.getmtime(h) for h in hs)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    hdr = _headers_mtime()
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        stale = (force or not os.path.exists(obj)
                 or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr))
        jobs.append((src, obj, stale))

    def compile_one(job):
        src, obj, stale = job
        if not stale:
            return ""
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
        if ptxas_v:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        os.replace(obj + ".tmp", obj)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs) or 1)) as ex:
        logs = list(ex.map(compile_one, jobs))
    if verbose:
        for log in logs:
            if log:
                sys.stdout.write(log)
    objs = [o for _, o, _ in jobs]
    if (force or not os.path.exists(SO)
            or os.path.getmtime(SO) < max(os.path.getmtime(o) for o in objs)):
        tmp = SO + ".tmp%d" % os.getpid()
        cmd = [nvcc, *ARCH, "-shared", "-Xlinker", "--no-undefined", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, SO)
    return SO


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="-v" in sys.argv))
