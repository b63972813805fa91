"""Build libsemo_gb300.so (sm_103a) in-tree with nvcc.

Translation units are compiled in parallel, then linked into one shared
library exporting the C-ABI of include/semo_gb300.h.  geometry.cu is built
with --fmad=false so mesh geometry is bit-identical to the reference; the
hot kernels keep FMA contraction.

    python -m semo_mesh_gb300.build
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsemo_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = [
    ("geometry.cu", ["--fmad=false"]),
    ("assemble.cu", []),
    ("momentum.cu", []),
    ("vof.cu", []),
    ("coupled.cu", []),
    ("surftens.cu", []),
    ("amg_setup.cu", []),
    ("cycle.cu", []),
    ("adjoint.cu", []),
    ("noalloc.cu", []),
    ("capi.cpp", []),
    ("foam.cpp", []),
    ("rcm.cpp", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, "semo_internal.h"), os.path.join(CSRC, "face_common.cuh"),
               os.path.join(os.path.dirname(HERE), "include", "semo_gb300.h")]
    procs = []
    objs = []
    for src, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not force and not _stale(o, [s] + headers):
            continue
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O2",
               "-c", s, "-o", o, *extra]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError("nvcc failed for " + ", ".join(failed))
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
