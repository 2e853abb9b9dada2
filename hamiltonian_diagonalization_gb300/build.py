"""Build libedgb300.so in-tree for sm_103a (GB300) with nvcc.

    python -m hamiltonian_diagonalization_gb300.build        # or build() from Python

Each translation unit is compiled in parallel into _build/, then linked
into hamiltonian_diagonalization_gb300/libedgb300.so.  Host code is compiled
with -ffp-contract=off so that x86-64 and aarch64 hosts compute identical
term tables.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libedgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["ed_terms.cpp", "ed_eigen.cpp", "ed_basis.cu", "ed_build.cu", "ed_spmv.cu", "ed_lanczos.cu",
           "ed_capi.cu", "ed_noalloc.cu", "ed_batched.cu", "ed_mlp.cu", "ed_rotate.cu", "ed_io.cpp", "ed_observables.cu",
           "ed_complex.cu", "ed_subspace.cu", "ed_eigen_dev.cu", "ed_term_hash.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src: str):
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + CSRC]
    if src.endswith(".cu"):
        return ARCH + ["-lineinfo"] + common
    return ["-x", "c++"] + common


def _needs(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "ed_capi.h"))
    nv = nvcc()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            jobs.append([nv] + _flags(s) + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r

    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4) or 1) as ex:
        list(ex.map(run, jobs))
    if jobs or force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
