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
into a scratch folder, compiles it and deletes it.  exact_literals=True likewise writes the
kernel's two float PSD constants (70.7f, 2.f/3.f) in double precision, so that a comparison
shows what else, if anything, separates the kernel from the oracle.

`BsaclRef.groups` returns the kernel's per-work-group partials (sums over 16 consecutive pairs
of the list, the finest output the kernel has: every work item writes its own pair's value
only into the work group's local reduction array)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference tree: BSALIB_REFERENCE names its root (default: where this build keeps it).
REF_ROOT = os.environ.get("BSALIB_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "BsaCL", "src")
WIPWG = 16  # work items per work group (power of two, >= 9 for the kernel's prefetch)


def available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "bsacl.cl")) and os.path.exists(os.path.join(REF_SRC, "_base.h"))


# The kernel's two PSD constants written as float literals (evalFct, bsacl.cl:104, :118):
# exact_literals=True builds a scratch copy with them written in double precision, which
# isolates their effect (4.3e-8 on the spectra) from everything else the kernel computes.
LITERALS = (("(BSACL_REAL)70.7f", "(BSACL_REAL)70.7", 1), ("2.f/3.f", "((BSACL_REAL)2/(BSACL_REAL)3)", 2))


def build(ntc: int, nnl: int, nm: int, nn: int, nfi: int, nfj: int, psd_id: int = 1,
          plain_loop: bool = False, exact_literals: bool = False) -> str:
    tag = (f"tc{ntc}_nl{nnl}_nm{nm}_nn{nn}_f{nfi}x{nfj}_p{psd_id}" + ("_plain" if plain_loop else "")
           + ("_exact" if exact_literals else ""))
    so = os.path.join(OUT, f"libbsacl_ref_{tag}.so")
    deps = [os.path.join(HERE, "bsacl_shim.h"), os.path.join(HERE, "bsacl_ref_driver.c")]
    if os.path.exists(so) and all(os.path.getmtime(so) >= os.path.getmtime(d) for d in deps):
        return so
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(REF_SRC, "bsacl.cl")
    tmp = None
    if plain_loop or exact_literals:  # an edited copy of the source, in a scratch folder
        with open(src) as fh:
            text = fh.read()
        if plain_loop:  # without its one optimised-loop #define
            line = "#define _use_optimised_loop_\n"
            if text.count(line) != 1:
                raise RuntimeError("bsacl.cl: the optimised-loop switch is not where expected")
            text = text.replace(line, "\n")
        if exact_literals:
            for old, new, count in LITERALS:
                if text.count(old) != count:
                    raise RuntimeError(f"bsacl.cl: the literal {old} is not where expected")
                text = text.replace(old, new)
        tmp = tempfile.TemporaryDirectory()
        src = os.path.join(tmp.name, "bsacl_edited.cl")
        with open(src, "w") as fh:
            fh.write(text)
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

    def __init__(self, ntc, nnl, nm, nn, nfi, nfj, psd_id=1, plain_loop=False, exact_literals=False):
        self.lib = C.CDLL(build(ntc, nnl, nm, nn, nfi, nfj, psd_id, plain_loop, exact_literals))
        for fn in (self.lib.bsacl_ref_run, self.lib.bsacl_ref_groups):
            fn.argtypes = [C.c_void_p] * 14
            fn.restype = C.c_int
        self.nwg = nfi * nfj // WIPWG + 1
        self.lib.bsacl_ref_psd.argtypes = [C.c_double] * 4
        self.lib.bsacl_ref_psd.restype = C.c_double
        self.nm = nm

    def psd(self, f, scl, std, ubar):
        return self.lib.bsacl_ref_psd(float(f), float(scl), float(std), float(ubar))

    def m3mr(self, tc, nodes_load, phitc, nod_corr, u, scl, std, winz, Mg, Cg, Kg, fi, fj):
        return self._call(self.lib.bsacl_ref_run, self.nm ** 3, tc, nodes_load, phitc, nod_corr, u, scl, std, winz,
                          Mg, Cg, Kg, fi, fj)

    def groups(self, tc, nodes_load, phitc, nod_corr, u, scl, std, winz, Mg, Cg, Kg, fi, fj):
        """Per-work-group partials (nwg, nm^3) before the host's weight: group g sums the
        kernel's values of pairs g WIPWG .. g WIPWG + WIPWG - 1 of the list fi x fj (fi fastest)."""
        out = self._call(self.lib.bsacl_ref_groups, self.nwg * self.nm ** 3, tc, nodes_load, phitc, nod_corr, u,
                         scl, std, winz, Mg, Cg, Kg, fi, fj)
        return out.reshape(self.nwg, self.nm ** 3)

    def _call(self, fn, nout, tc, nodes_load, phitc, nod_corr, u, scl, std, winz, Mg, Cg, Kg, fi, fj):
        keep = [np.ascontiguousarray(tc, dtype=np.uint32), np.ascontiguousarray(nodes_load, dtype=np.uint32),
                np.asfortranarray(phitc, dtype=np.float64), np.ascontiguousarray(nod_corr, dtype=np.float64),
                np.ascontiguousarray(u, dtype=np.float64), np.ascontiguousarray(scl, dtype=np.float64),
                np.ascontiguousarray(std, dtype=np.float64), np.ascontiguousarray(winz, dtype=np.int32),
                np.ascontiguousarray(Mg, dtype=np.float64), np.asfortranarray(Cg, dtype=np.float64),
                np.ascontiguousarray(Kg, dtype=np.float64), np.ascontiguousarray(fi, dtype=np.float64),
                np.ascontiguousarray(fj, dtype=np.float64)]
        out = np.zeros(nout)
        rc = fn(*[_p(a) for a in keep], _p(out))
        if rc:
            raise RuntimeError(f"the reference kernel's driver failed ({rc})")
        return out
