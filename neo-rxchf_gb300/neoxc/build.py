"""Build libneoxc_gb300.so (sm_103a) in-tree.

Each translation unit in ``csrc/`` is compiled by nvcc in parallel for
``compute_103a/sm_103a`` only, then linked into one shared library (static
CUDA runtime) at ``neoxc/_lib/libneoxc_gb300.so``.  The object files and
the library are git-ignored build artefacts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libneoxc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-O2"]
UNITS = ["abi.cu", "abi_fortran.cu", "abi_io.cu", "k_gam4.cu", "k_gam4f.cu", "k_contract.cu",
         "k_md.cu", "k_gam3.cu", "k_scf.cu", "k_spin.cu", "k_rx.cu", "k_rxscf.cu", "k_probe.cu",
         "k_noalloc.cu"]
HEADERS = ["neoxc_internal.h", "md_math.cuh", "md_math32.cuh", "md_math_body.cuh",
           "boys_table.inc", "g3_fatbra.cuh", "tc_gemm.cuh",
           "narrow.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    include = os.path.join(os.path.dirname(ROOT), "include", "neoxc.h")
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [include]
    objs, jobs = [], []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nv, *ARCH, *FLAGS, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: " + " ".join(j))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        r = subprocess.run([nv, *ARCH, "-shared", "-o", tmp, *objs],
                           capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libneoxc_gb300.so failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
