"""In-tree build of the CUDA library (libidrs_gb300.so) for sm_103a.

The translation units are compiled in parallel with nvcc and linked into
idrs-package_gb300/_build/libidrs_gb300.so.  No cmake; rebuilt only when a
source is newer than the library.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libidrs_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
SOURCES = ["matrix.cu", "solvers_real.cu", "solvers_cplx.cu", "solvers_ms_real.cu", "solvers_ms_cplx.cu",
           "adjoint.cu", "recycle.cu", "deflation.cu", "lu.cu", "capi.cu", "setup.cpp", "mm.cpp", "noalloc.cu"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
              "-Xcompiler", "-fPIC", "-I", INCLUDE]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))
    return files


def stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    procs = []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src} ---\n{out.decode(errors='replace')}")
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [obj for _, obj, _ in procs]
    tmp = LIB + ".tmp"
    subprocess.run([nvcc, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
