"""Build libbsagpu.so in-tree (nvcc, sm_103a only, no cmake).

Each translation unit under csrc/ is compiled in parallel, then linked into
bsalib_gb300/libbsagpu.so with the CUDA runtime linked statically, so the library loads
without a CUDA runtime on the loader path.  Run `python -m bsalib_gb300.build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbsagpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code without floating-point contraction: the zone layout's geometry compares rounded
# values (floor of a base / delta ratio, a rotation against pi), so a fused a * b + c where the
# reference rounds twice moves zones (gcc contracts by default where the target has FMA, as on
# aarch64; an x86-64 build of the reference has none)
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbsagpu")
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime() -> float:
    inc = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inc.append(os.path.join(HERE, "..", "include", "bsa_gpu.h"))
    return max(os.path.getmtime(p) for p in inc)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    objs = []

    def one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(one, sources()))
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
