"""Build recipe and binding of the reference's BsaCL kernel run on the host -- TEST
INFRASTRUCTURE ONLY (pins the oracle; see bsacl_ref_driver.c).

`build(ntc, nnl, nm, nn, nfi, nfj, psd_id, plain_loop)` compiles the kernel source where it
lies under the reference tree (BsaCL/src/bsacl.cl with its _base.h) together with
bsacl_shim.h and bsacl_ref_driver.c into oracle/_ref/, one library per problem size (the
kernel takes its sizes as macros).  Only where the reference tree is present (not on the GPU
host).

The kernel as shipped defines _use_optimised_loop_ unconditionally (bsacl.cl:48): its node
loops then visit the triples (k, k, k), (j, j, k), (j, k, j), (k, j, j) and the six orders of
i > j > k, but not (k, k, j), (k, j, k), (j, k, k) for k < j, so it sums n^3 - 3 n (n - 1) / 2
of the n^3 node triples.  plain_loop=True builds the kernel's other branch (the full
triple loop, bsacl.cl:780-865): the recipe writes the source without that one #define line
into a scratch folder, compiles it and deletes it."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_SRC = "/root/reference/BsaCL/src"
WIPWG = 16  # work items per work group (power of two, >= 9 for the kernel's prefetch)


def available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "bsacl.cl")) and os.path.exists(os.path.join(REF_SRC, "_base.h"))


def build(ntc: int, nnl: int, nm: int, nn: int, nfi: int, nfj: int, psd_id: int = 1,
          plain_loop: bool = False) -> str:
    tag = f"tc{ntc}_nl{nnl}_nm{nm}_nn{nn}_f{nfi}x{nfj}_p{psd_id}" + ("_plain" if plain_loop else "")
    so = os.path.join(OUT, f"libbsacl_ref_{tag}.so")
    deps = [os.path.join(HERE, "bsacl_shim.h"), os.path.join(HERE, "bsacl_ref_driver.c")]
    if os.path.exists(so) and all(os.path.getmtime(so) >= os.path.getmtime(d) for d in deps):
        return so
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(REF_SRC, "bsacl.cl")
    tmp = None
    if plain_loop:  # the source without its one optimised-loop #define, in a scratch folder
        with open(src) as fh:
            text = fh.read()
        line = "#define _use_optimised_loop_\n"
        if text.count(line) != 1:
            raise RuntimeError("bsacl.cl: the optimised-loop switch is not where expected")
        tmp = tempfile.TemporaryDirectory()
        src = os.path.join(tmp.name, "bsacl_plain_loop.cl")
        with open(src, "w") as fh:
            fh.write(text.replace(line, "\n"))
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-pthread", "-w", "-ffp-contract=off",
           "-include", os.path.join(HERE, "bsacl_shim.h"),
           f"-DBSACL_CL_SOURCE=\"{src}\"", f"-DBSACL_BASE_DIR={REF_SRC}",
           "-DBSACL_KERNEL_ID=2", "-DBSACL_USE_DOUBLE_PRECISION", f"-DBSACL_WIpWG={WIPWG}",
           f"-DBSACL_WIND_PSD_ID={psd_id}", f"-DNTC__={ntc}", f"-DNNL__={nnl}", f"-DNM_EFF__={nm}",
           f"-DNN__={nn}", "-DNDEGW__=6", f"-DNNOD_CORR__={(nn * nn + nn) // 2}", f"-DNFI__={nfi}",
           f"-DNFJ__={nfj}", "-o", so, os.path.join(HERE, "bsacl_ref_driver.c"), "-lm"]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True)  # the source prints #pragma messages
        if r.returncode:
            raise RuntimeError(f"building the reference kernel failed:\n{r.stderr[-4000:]}")
    finally:
        if tmp is not None:
            tmp.cleanup()
    return so


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class BsaclRef:
    """The reference kernel for one problem size."""

    def __init__(self, ntc, nnl, nm, nn, nfi, nfj, psd_id=1, plain_loop=False):
        self.lib = C.CDLL(build(ntc, nnl, nm, nn, nfi, nfj, psd_id, plain_loop))
        self.lib.bsacl_ref_run.argtypes = [C.c_void_p] * 14
        self.lib.bsacl_ref_run.restype = C.c_int
        self.lib.bsacl_ref_psd.argtypes = [C.c_double] * 4
        self.lib.bsacl_ref_psd.restype = C.c_double
        self.nm = nm

    def psd(self, f, scl, std, ubar):
        return self.lib.bsacl_ref_psd(float(f), float(scl), float(std), float(ubar))

    def m3mr(self, tc, nodes_load, phitc, nod_corr, u, scl, std, winz, Mg, Cg, Kg, fi, fj):
        keep = [np.ascontiguousarray(tc, dtype=np.uint32), np.ascontiguousarray(nodes_load, dtype=np.uint32),
                np.asfortranarray(phitc, dtype=np.float64), np.ascontiguousarray(nod_corr, dtype=np.float64),
                np.ascontiguousarray(u, dtype=np.float64), np.ascontiguousarray(scl, dtype=np.float64),
                np.ascontiguousarray(std, dtype=np.float64), np.ascontiguousarray(winz, dtype=np.int32),
                np.ascontiguousarray(Mg, dtype=np.float64), np.asfortranarray(Cg, dtype=np.float64),
                np.ascontiguousarray(Kg, dtype=np.float64), np.ascontiguousarray(fi, dtype=np.float64),
                np.ascontiguousarray(fj, dtype=np.float64)]
        out = np.zeros(self.nm ** 3)
        rc = self.lib.bsacl_ref_run(*[_p(a) for a in keep], _p(out))
        if rc:
            raise RuntimeError(f"bsacl_ref_run failed ({rc})")
        return out
