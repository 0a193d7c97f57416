"""Python binding of libbsagpu (ctypes over include/bsa_gpu.h).

`BsaSession` mirrors the standalone driver's use of BsaLib (app/bsa.F90:107-117 and its
`setup`, :525-606): it calls bsa_Init, the setters with the Problem's arrays (which the
library borrows -- the session keeps them alive), bsa_setTotDamping and bsa_Run.

The library is the only compute path: there is no CPU fallback.  If libbsagpu.so is
missing, `load()` raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from typing import Dict, Optional

import numpy as np

from .problem import Problem

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbsagpu.so")
HEADER = os.path.join(HERE, "..", "include", "bsa_gpu.h")

BSA_OK = 0
PREC_FP64 = 0
PREC_BF16X3 = 1

_lib = None

# bsa_brm_export_fn: (npts, f1, f2, brm[npts][dim_bisp], user)
EXPORT_FN = C.CFUNCTYPE(None, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                        C.c_void_p)


PLAN_CLS_FORM, PLAN_CLS_E_WIDTH, PLAN_CLS_D_WIDTH, PLAN_MSH_WIDTH, PLAN_CLS_E_SPLIT = 1, 2, 3, 4, 5


def tile_plan(family: int, nm: int, K: int, nf: int = 0) -> int:
    """The tile-plan value the library uses for a case (bsa_gpu_getTilePlan)."""
    v = C.c_int(0)
    check(load().bsa_gpu_getTilePlan(family, nm, K, nf, C.byref(v)), "bsa_gpu_getTilePlan")
    return v.value


class BsaError(RuntimeError):
    """A failed library call; `code` is the BSA_ERR_* status it returned."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


class Zone(C.Structure):
    """bsa_zone: a rectangular Mesher zone (include/bsa_gpu.h)."""
    _fields_ = [("fi0", C.c_double), ("fj0", C.c_double), ("dIi", C.c_double), ("dIj", C.c_double),
                ("dJi", C.c_double), ("dJj", C.c_double), ("ni", C.c_int), ("nj", C.c_int),
                ("Fi", C.c_int), ("Fj", C.c_int), ("sym", C.c_double), ("policy", C.c_int)]


class Triangle(C.Structure):
    """bsa_triangle: a triangular Mesher zone as the pre-mesh dumps it (include/bsa_gpu.h)."""
    _fields_ = [("Ci", C.c_double), ("Cj", C.c_double), ("Ai", C.c_double), ("Aj", C.c_double),
                ("Bi", C.c_double), ("Bj", C.c_double), ("rot", C.c_double), ("sym", C.c_double),
                ("n", C.c_int), ("policy", C.c_int), ("bfm_i", C.c_int), ("bfm_j", C.c_int),
                ("bfm_levels", C.c_int), ("brm_i", C.c_int), ("brm_j", C.c_int), ("seq", C.c_int)]


def triangle_lattice(t: Triangle, visual=False):
    """bsa_gpu_mshTriangLattice (host only): the post-mesh lattice of one triangle as a dict of
    arrays (bfm [nb, 3], brm [nq, 3], qptr, qsrc, qc, exp [ne, 2], eq) and counts."""
    lib = load()
    cnt = np.zeros(6, dtype=np.int64)
    oob = C.c_int(0)
    check(lib.bsa_gpu_mshTriangLattice(C.byref(t), int(visual), _p(cnt), C.byref(oob), None, None, None, None,
                                       None, None, None), "bsa_gpu_mshTriangLattice")
    nb, nq, nnz, ne = (int(x) for x in cnt[:4])
    out = dict(bfm=np.zeros((nb, 3)), brm=np.zeros((nq, 3)), qptr=np.zeros(nq + 1, dtype=np.int32),
               qsrc=np.zeros(max(nnz, 1), dtype=np.int32), qc=np.zeros(max(nnz, 1)), exp=np.zeros((max(ne, 1), 2)),
               eq=np.zeros(max(ne, 1), dtype=np.int32))
    check(lib.bsa_gpu_mshTriangLattice(C.byref(t), int(visual), _p(cnt), C.byref(oob), _p(out["bfm"]),
                                       _p(out["brm"]), _p(out["qptr"]), _p(out["qsrc"]), _p(out["qc"]),
                                       _p(out["exp"]), _p(out["eq"])), "bsa_gpu_mshTriangLattice")
    out["qsrc"], out["qc"], out["exp"], out["eq"] = out["qsrc"][:nnz], out["qc"][:nnz], out["exp"][:ne], out["eq"][:ne]
    out["bfm_post"], out["brm_post"], out["oob"] = int(cnt[4]), int(cnt[5]), bool(oob.value)
    return out


class Stats(C.Structure):
    _fields_ = [("ms_total", C.c_double), ("ms_contraction", C.c_double), ("ms_gemm", C.c_double),
                ("points", C.c_double), ("h2d_bytes", C.c_double), ("d2h_bytes", C.c_double),
                ("kernels", C.c_int), ("precision", C.c_int), ("graphs", C.c_int)]


def header_symbols():
    """Every function name declared in include/bsa_gpu.h."""
    with open(HEADER) as fh:
        txt = fh.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b((?:bsa|bsacl)\w*)\s*\(", txt)))


def load(path: Optional[str] = None):
    """Load libbsagpu.so (build it first with `python -m bsalib_gb300.build`)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise BsaError(f"{p} is missing: build it with `python -m bsalib_gb300.build`")
    lib = C.CDLL(p)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    sig = {
        "bsa_Init": [], "bsa_Finalise": [], "bsa_lastError": None, "bsa_mlp_lastError": None,
        "bsa_setAnalysisType": [i], "bsa_setVersion": [i], "bsa_setScalingConv": [i],
        "bsa_setSpectraComputation": [i, i], "bsa_setSpectraExtension": [i], "bsa_setSpatialSymmetry": [i],
        "bsa_setSpectraSymmetries": [i], "bsa_setTestMode": [i], "bsa_setupClassic": [i, d],
        "bsa_setClassicMode": [i], "bsa_setupMesher": [i, i, d, d, d, i, i],
        "bsa_setWindDirections": [vp, i], "bsa_setWindTurbComps": [vp, i], "bsa_setTotalNOfNodes": [i],
        "bsa_setNumOfNodalDOFs": [i], "bsa_setTotalNumOfDOFs": [i], "bsa_setLoadedNodes": [vp, i],
        "bsa_setLoadedNodalDOFs": [vp, i], "bsa_setNodalCoords": [i, vp], "bsa_setModalInfo": [i, i, vp, vp],
        "bsa_setModalMatrices": [i, vp, vp, vp], "bsa_setTotDamping": [vp, i], "bsa_setPSDType": [i],
        "bsa_setWindVertProf": [i], "bsa_setWindAltDir": [i], "bsa_setAirDensity": [d],
        "bsa_setWZMeanWindVel": [vp, i], "bsa_setWZRefAlt": [vp, i], "bsa_setTurbWindScales": [vp, i],
        "bsa_setTurbWindSDT": [vp, i], "bsa_setNodalVel": [vp, i], "bsa_setNodalWindZones": [vp, i],
        "bsa_setNodalWindAltitudes": [vp, i], "bsa_setSpatialNodalCorr": [vp, C.c_int64],
        "bsa_setWindFCoeffs": [vp, i, i, i], "bsa_getNModesEff": [vp], "bsa_getSpectraDims": [vp, vp],
        "bsa_Run": [vp] * 7, "bsa_computeSkewness": [i, vp, vp, vp],
        "bsa_gpu_setPrecision": [i], "bsa_gpu_setClassicTruncation": [i], "bsa_gpu_setClassicRows": [i, i],
        "bsa_gpu_clsBispectra": [vp, i, vp, vp, vp], "bsa_gpu_mshBispectra": [vp, vp, i, vp, vp],
        "bsa_gpu_clsBispectraAt": [vp, vp, i, vp, vp], "bsa_gpu_setWaitTest": [i],
        "bsa_gpu_setMesherGraphs": [i], "bsa_gpu_setMesherExpansion": [i], "bsa_gpu_setMesherPassBytes": [d], "bsa_gpu_setClassicShard": [i, i], "bsa_enableVisualMode": [], "bsa_setVisualIndexes": [vp, i], "bsa_setBRMExportDefaultMode": [i],
        "bsa_gpu_setTilePlan": [i] * 8, "bsa_gpu_clearTilePlans": [], "bsa_gpu_loadTilePlans": [C.c_char_p],
        "bsa_gpu_getTilePlan": [i, i, i, i, vp],
        "bsa_gpu_mshMoments": [vp, vp, vp, i, vp, vp], "bsa_gpu_getStats": [vp], "bsa_gpu_releaseDeviceCache": [], "bsa_gpu_setClassicForm": [i],
        "bsa_gpu_pointMomentsNoAlloc": [vp, i, i, vp, vp, vp, vp, vp, vp, vp, i, vp, vp, vp, vp, vp, vp],
        "bsa_gpu_mshZones": [vp, i, vp, vp, vp], "bsa_gpu_mshGenerateZones": [vp, i, vp],
        "bsa_setPODTruncationThreshold": [d], "bsa_setPODNOfModesKept": [i],
        "bsa_gpu_mshZonesDiag": [vp, i, vp, vp, vp], "bsa_setBispExportCallback": [EXPORT_FN, vp],
        "bsa_gpu_setClassicSymmetry": [i], "bsa_loadInputFiles": [C.c_char_p],
        "bsa_mlp_create": [i, i, C.c_ulonglong], "bsa_mlp_destroy": [i], "bsa_mlp_num_params": [i],
        "bsa_mlp_get_params": [i, vp, i], "bsa_mlp_set_params": [i, vp], "bsa_mlp_forward": [i, vp, i, vp],
        "bsa_mlp_gradients": [i, vp, vp, vp, i, vp, vp],
        "bsa_mlp_train": [i, vp, vp, vp, i, i, i, C.c_float, C.c_ulonglong, vp],
        "bsa_computeBRdecomp": [vp, vp, vp], "bsa_modalRecombination": [vp] * 11, "bsa_computePeakFactors": [i, vp, vp, d, vp, vp, vp, vp],
        "bsa_gpu_batchAdd": [vp], "bsa_gpu_batchCase": [i, vp, vp], "bsa_gpu_batchRun": [vp] * 5,
        "bsa_gpu_batchClear": [], "bsa_doValidateZoneDeltas": [i], "bsa_setBfmMLR": [i],
        "bsa_setMaxBkgPeakRestriction": [i], "bsa_setPremeshScheme": [i], "bsa_setPremeshMode": [i],
        "bsa_gpu_mshGenerateTriangles": [vp, i, vp], "bsa_gpu_mshTriangles": [vp, i, vp, vp, vp],
        "bsa_gpu_mshTriangLattice": [vp, i, vp, vp, vp, vp, vp, vp, vp, vp, vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        if name in ("bsa_lastError", "bsa_mlp_lastError"):
            fn.restype = C.c_char_p
            fn.argtypes = []
        elif name == "bsa_mlp_num_params":
            fn.restype = C.c_longlong
            fn.argtypes = args
        else:
            fn.restype = C.c_int
            fn.argtypes = args
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def check(rc: int, what: str = ""):
    if rc != BSA_OK:
        msg = load().bsa_lastError().decode(errors="replace")
        raise BsaError(f"{what} failed ({rc}): {msg}", rc)


class BsaSession:
    """One BsaLib run over a Problem (borrowed arrays are kept alive here)."""

    def __init__(self, prob: Problem, precision: int = PREC_FP64, classic_truncation: bool = True):
        self.lib = load()
        self.prob = prob
        self._keep = {}
        self.precision = precision
        self.classic_truncation = classic_truncation
        self._setup()

    def _arr(self, name, a, dt):
        a = np.asfortranarray(np.asarray(a, dtype=dt))
        self._keep[name] = a
        return _p(a)

    def _setup(self):
        L, p, s = self.lib, self.prob, self.prob.settings
        check(L.bsa_Init(), "bsa_Init")
        # settings (app/bsa.F90:560-575)
        if s.suban:
            check(L.bsa_setAnalysisType(s.suban), "bsa_setAnalysisType")
        if s.vers:
            check(L.bsa_setVersion(s.vers), "bsa_setVersion")
        if s.defsc:
            check(L.bsa_setScalingConv(s.defsc), "bsa_setScalingConv")
        check(L.bsa_setSpectraComputation(s.ipsd, s.ibisp), "bsa_setSpectraComputation")
        check(L.bsa_setSpectraExtension(s.onlyd), "bsa_setSpectraExtension")
        check(L.bsa_setSpatialSymmetry(s.bispsym), "bsa_setSpatialSymmetry")
        check(L.bsa_setSpectraSymmetries(s.sym3d), "bsa_setSpectraSymmetries")
        check(L.bsa_setTestMode(s.test), "bsa_setTestMode")
        check(L.bsa_setupClassic(s.nfreqs, float(s.df)), "bsa_setupClassic")
        check(L.bsa_setClassicMode(s.scalar), "bsa_setClassicMode")
        check(L.bsa_setupMesher(s.svd, s.bkgrfmt, s.bkgaext, s.genpaext, s.maxaext, s.fcov, s.dumpmod),
              "bsa_setupMesher")
        check(L.bsa_setWindDirections(self._arr("dirs", s.dirs, np.int32), len(s.dirs)), "dirs")
        check(L.bsa_setWindTurbComps(self._arr("tc", s.tc, np.int32), len(s.tc)), "tc")
        # nodal
        check(L.bsa_setTotalNOfNodes(p.nn), "nn")
        check(L.bsa_setNumOfNodalDOFs(p.nlibs), "nlibs")
        check(L.bsa_setLoadedNodes(self._arr("nl", p.n_load, np.int32), p.nnl), "loaded nodes")
        check(L.bsa_setLoadedNodalDOFs(self._arr("ll", p.libs_load, np.int32), p.nlibsl), "loaded DOFs")
        check(L.bsa_setNodalCoords(p.nn, self._arr("coords", p.coords, np.float64)), "coords")
        # wind
        check(L.bsa_setWindVertProf(p.i_varu), "wind profile")
        check(L.bsa_setPSDType(p.psd_type), "psd type")
        check(L.bsa_setWindAltDir(p.i_vert), "vert dir")
        check(L.bsa_setAirDensity(p.air_dens), "air density")
        check(L.bsa_setWZMeanWindVel(self._arr("ubref", p.UBref, np.float64), p.nz), "UBref")
        check(L.bsa_setWZRefAlt(self._arr("zref", p.Zref, np.float64), p.nz), "Zref")
        check(L.bsa_setTurbWindScales(self._arr("L", p.L, np.float64), p.nz), "L")
        check(L.bsa_setTurbWindSDT(self._arr("sigma", p.sigma, np.float64), p.nz), "sigma")
        check(L.bsa_setNodalVel(self._arr("unod", p.u_node, np.float64), p.nn), "u_node")
        check(L.bsa_setNodalWindZones(self._arr("wz", p.wz_node, np.int32), p.nn), "wz")
        check(L.bsa_setNodalWindAltitudes(self._arr("walt", p.wAlt_node, np.float64), p.nn), "walt")
        check(L.bsa_setSpatialNodalCorr(self._arr("corr", p.nod_corr, np.float64), p.nod_corr.shape[0]), "corr")
        w = p.wfc
        check(L.bsa_setWindFCoeffs(self._arr("wfc", w, np.float64), w.shape[0], w.shape[1], w.shape[2]), "wfc")
        # modal
        check(L.bsa_setModalInfo(p.ndofs, p.nm, self._arr("phi", p.phi, np.float64),
                                 self._arr("natf", p.natf, np.float64)), "modal info")
        check(L.bsa_setModalMatrices(p.nm, self._arr("Mg", p.Mg, np.float64), self._arr("Kg", p.Kg, np.float64),
                                     self._arr("Cg", p.Cg, np.float64)), "modal matrices")
        check(L.bsa_setTotDamping(self._arr("xsi", p.xsi, np.float64), p.nm), "damping")
        check(L.bsa_gpu_setPrecision(self.precision), "precision")
        check(L.bsa_gpu_setClassicTruncation(1 if self.classic_truncation else 0), "truncation")

    def set_precision(self, prec: int):
        self.precision = prec
        check(self.lib.bsa_gpu_setPrecision(prec), "bsa_gpu_setPrecision")

    def set_symmetry(self, on: bool = True):
        """bsa_gpu_setClassicSymmetry: evaluate half of the (symmetric) Classic grid."""
        check(self.lib.bsa_gpu_setClassicSymmetry(1 if on else 0), "bsa_gpu_setClassicSymmetry")

    def set_mesher_controls(self, validate: bool = True, mlr: bool = True, restrict: bool = False):
        """Mesher controls: zone-delta validation, BFM multi-level refinement, background peak
        restricted to the first direction (bsa_doValidateZoneDeltas, bsa_setBfmMLR,
        bsa_setMaxBkgPeakRestriction; the arguments' defaults are the library's)."""
        check(self.lib.bsa_doValidateZoneDeltas(1 if validate else 0), "bsa_doValidateZoneDeltas")
        check(self.lib.bsa_setBfmMLR(1 if mlr else 0), "bsa_setBfmMLR")
        check(self.lib.bsa_setMaxBkgPeakRestriction(1 if restrict else 0), "bsa_setMaxBkgPeakRestriction")

    def use_driver_controls(self):
        """The standalone driver's Mesher controls (app/bsa.F90:544-549): no delta validation,
        no BFM multi-level refinement, background peak from the first direction."""
        self.set_mesher_controls(False, False, True)

    def set_classic_form(self, form: int):
        """1: the E form of the split contraction where it applies (default); 0: D1 / D3 form."""
        check(self.lib.bsa_gpu_setClassicForm(int(form)), "bsa_gpu_setClassicForm")

    def set_shard(self, rank: int, nshards: int):
        """bsa_gpu_setClassicShard: this session evaluates shard `rank` of `nshards`."""
        check(self.lib.bsa_gpu_setClassicShard(int(rank), int(nshards)), "bsa_gpu_setClassicShard")

    def set_rows(self, r_begin: int, r_end: int = -1):
        """Evaluate only Classic grid rows [r_begin, r_end) (f1 index)."""
        check(self.lib.bsa_gpu_setClassicRows(int(r_begin), int(r_end)), "bsa_gpu_setClassicRows")

    def nmodes(self) -> int:
        n = np.zeros(1, dtype=np.int32)
        check(self.lib.bsa_getNModesEff(_p(n)), "bsa_getNModesEff")
        return int(n[0])

    def dims(self):
        """(dim_psd, dim_bisp): nm^2 / nm^3, or nm / nm with the diagonal-only spectra."""
        d = np.zeros(2, dtype=np.int32)
        check(self.lib.bsa_getSpectraDims(_p(d[:1]), _p(d[1:])), "bsa_getSpectraDims")
        return int(d[0]), int(d[1])

    def run(self) -> Dict[str, np.ndarray]:
        """bsa_Run: returns m2mf_cls, m2mr_cls, m2o2mr_cls, m3mf_msh, m3mr_msh, m3mf_cls, m3mr_cls."""
        d2, d3 = self.dims()
        out = {k: np.zeros(d2) for k in ("m2mf_cls", "m2mr_cls", "m2o2mr_cls")}
        out.update({k: np.zeros(d3) for k in ("m3mf_msh", "m3mr_msh", "m3mf_cls", "m3mr_cls")})
        check(self.lib.bsa_Run(_p(out["m2mf_cls"]), _p(out["m2mr_cls"]), _p(out["m2o2mr_cls"]),
                               _p(out["m3mf_msh"]), _p(out["m3mr_msh"]), _p(out["m3mf_cls"]),
                               _p(out["m3mr_cls"])), "bsa_Run")
        return out

    def classic_bispectra(self):
        """Materialised force / response bispectra on the classic grid (f1 fastest)."""
        nm3 = self.dims()[1]
        nf_cap = self.prob.classic_nf() + 8
        nf = np.zeros(1, dtype=np.int32)
        f = np.zeros(nf_cap)
        # query the size first
        s = self.prob.settings
        nfx = self.prob.classic_nf() if s.test else nf_cap * 4
        bf = np.zeros(nfx * nfx * nm3)
        br = np.zeros(nfx * nfx * nm3)
        check(self.lib.bsa_gpu_clsBispectra(_p(f), nf_cap, _p(nf), _p(bf), _p(br)), "bsa_gpu_clsBispectra")
        n = int(nf[0])
        # library layout: (dim_bisp, nf*nf) column-major, point p = i1 + nf*i2
        bf = bf[: n * n * nm3].reshape(n, n, nm3).transpose(1, 0, 2)
        br = br[: n * n * nm3].reshape(n, n, nm3).transpose(1, 0, 2)
        return f[:n].copy(), bf, br

    def classic_points(self, i1, i2):
        """Force / response bispectra (npts, dim_bisp) at Classic grid points (i1[p], i2[p]) in the
        session's precision (bsa_gpu_clsBispectraAt)."""
        i1 = np.ascontiguousarray(i1, dtype=np.int32)
        i2 = np.ascontiguousarray(i2, dtype=np.int32)
        nm3 = self.dims()[1]
        bf = np.zeros((i1.size, nm3))
        br = np.zeros((i1.size, nm3))
        check(self.lib.bsa_gpu_clsBispectraAt(_p(i1), _p(i2), i1.size, _p(bf), _p(br)), "bsa_gpu_clsBispectraAt")
        return bf, br

    def msh_bispectra(self, fi, fj):
        fi = np.ascontiguousarray(fi, dtype=np.float64)
        fj = np.ascontiguousarray(fj, dtype=np.float64)
        nm3 = self.dims()[1]
        bfm = np.zeros((fi.size, nm3))
        brm = np.zeros((fi.size, nm3))
        check(self.lib.bsa_gpu_mshBispectra(_p(fi), _p(fj), fi.size, _p(bfm), _p(brm)), "bsa_gpu_mshBispectra")
        return bfm, brm

    def msh_moments(self, fi, fj, w):
        fi = np.ascontiguousarray(fi, dtype=np.float64)
        fj = np.ascontiguousarray(fj, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        nm3 = self.dims()[1]
        mf, mr = np.zeros(nm3), np.zeros(nm3)
        check(self.lib.bsa_gpu_mshMoments(_p(fi), _p(fj), _p(w), fi.size, _p(mf), _p(mr)), "bsa_gpu_mshMoments")
        return mf, mr

    def msh_zones(self, zones):
        """Third moments (m3mf, m3mr) over a list of Zone structures, and the BFM / BRM
        lattice point counts."""
        arr = (Zone * len(zones))(*zones)
        nm3 = self.dims()[1]
        mf, mr, cnt = np.zeros(nm3), np.zeros(nm3), np.zeros(2)
        check(self.lib.bsa_gpu_mshZones(C.cast(arr, C.c_void_p), len(zones), _p(mf), _p(mr), _p(cnt)),
              "bsa_gpu_mshZones")
        return mf, mr, cnt

    def generate_zones(self):
        """The zone layout of the Mesher analysis."""
        n = C.c_int(0)
        check(self.lib.bsa_gpu_mshGenerateZones(None, 0, C.byref(n)), "bsa_gpu_mshGenerateZones")
        arr = (Zone * n.value)()
        check(self.lib.bsa_gpu_mshGenerateZones(C.cast(arr, C.c_void_p), n.value, C.byref(n)),
              "bsa_gpu_mshGenerateZones")
        return list(arr)

    def generate_triangles(self):
        """The triangles of the Mesher layout (the diagonal-crest scheme lays them)."""
        n = C.c_int(0)
        check(self.lib.bsa_gpu_mshGenerateTriangles(None, 0, C.byref(n)), "bsa_gpu_mshGenerateTriangles")
        arr = (Triangle * max(n.value, 1))()
        check(self.lib.bsa_gpu_mshGenerateTriangles(C.cast(arr, C.c_void_p), n.value, C.byref(n)),
              "bsa_gpu_mshGenerateTriangles")
        return list(arr)[:n.value]

    def msh_triangles(self, tris):
        """Third moments (m3mf, m3mr) over a list of Triangle structures, and the BFM / BRM
        point counts."""
        arr = (Triangle * len(tris))(*tris)
        nm3 = self.dims()[1]
        mf, mr, cnt = np.zeros(nm3), np.zeros(nm3), np.zeros(2)
        check(self.lib.bsa_gpu_mshTriangles(C.cast(arr, C.c_void_p), len(tris), _p(mf), _p(mr), _p(cnt)),
              "bsa_gpu_mshTriangles")
        return mf, mr, cnt

    def set_premesh(self, diag_crest=False, mode_base=False):
        """bsa_setPremeshScheme / bsa_setPremeshMode: each selects its non-default value only."""
        if diag_crest:
            check(self.lib.bsa_setPremeshScheme(1), "bsa_setPremeshScheme")
        if mode_base:
            check(self.lib.bsa_setPremeshMode(0), "bsa_setPremeshMode")

    def stats(self) -> Stats:
        st = Stats()
        check(self.lib.bsa_gpu_getStats(C.byref(st)), "bsa_gpu_getStats")
        return st

    def skewness(self, m2, m3):
        nm = self.nmodes()
        sk = np.zeros(self.dims()[1])
        check(self.lib.bsa_computeSkewness(nm, _p(np.ascontiguousarray(m2)), _p(np.ascontiguousarray(m3)),
                                           _p(sk)), "bsa_computeSkewness")
        return sk

    def modal_recombination(self, m2mr, m3mr, m2o2mr=None):
        """bsa_modalRecombination: nodal m2 / m3 / m2o2 / sk per DOF, diag and CCC branches."""
        nd = self.prob.phi.shape[0]
        keys = ("m2_diag", "m3_diag", "m2o2_diag", "sk_diag", "m2_ccc", "m3_ccc", "m2o2_ccc", "sk_ccc")
        out = {k: np.zeros(nd) for k in keys}
        m2o2 = None if m2o2mr is None else np.ascontiguousarray(m2o2mr, dtype=np.float64)
        check(self.lib.bsa_modalRecombination(_p(np.ascontiguousarray(m2mr, dtype=np.float64)),
                                              _p(np.ascontiguousarray(m3mr, dtype=np.float64)),
                                              None if m2o2 is None else _p(m2o2), *[_p(out[k]) for k in keys]),
              "bsa_modalRecombination")
        if self.dims()[1] == self.nmodes():
            for k in keys[4:]:
                del out[k]
        return out

    def br_decomp(self, m2mf):
        """bsa_computeBRdecomp: (background, resonant) parts of each kept mode's variance."""
        nm = self.nmodes()
        bkg, res = np.zeros(nm), np.zeros(nm)
        check(self.lib.bsa_computeBRdecomp(_p(np.ascontiguousarray(m2mf, dtype=np.float64)), _p(bkg), _p(res)),
              "bsa_computeBRdecomp")
        return bkg, res

    def peak_factors(self, m2, m2o2, obs_time, sk=None):
        """bsa_computePeakFactors: (status, peak_g, peak_ng_pos, peak_ng_neg); status is
        BSA_OK or BSA_SKIPPED (1) where the reference warns and returns."""
        m2 = np.ascontiguousarray(m2, dtype=np.float64)
        g, pos, neg = np.zeros(m2.size), np.zeros(m2.size), np.zeros(m2.size)
        skp = _p(np.ascontiguousarray(sk, dtype=np.float64)) if sk is not None else None
        rc = self.lib.bsa_computePeakFactors(m2.size, _p(m2), _p(np.ascontiguousarray(m2o2, dtype=np.float64)),
                                             float(obs_time), _p(g), skp, _p(pos) if sk is not None else None,
                                             _p(neg) if sk is not None else None)
        if rc < 0:
            check(rc, "bsa_computePeakFactors")
        return rc, g, pos, neg

    def set_export(self, fn):
        """bsa_setBispExportCallback: fn(f1, f2, brm[npts][dim_bisp]) receives the response
        bispectra during run(): the Classic grid in column blocks, the Mesher's BRM lattice one
        zone at a time; None switches the export off."""
        if fn is None:
            self._export = None
            check(self.lib.bsa_setBispExportCallback(C.cast(None, EXPORT_FN), None), "bsa_setBispExportCallback")
            return
        nb = self.dims()[1]

        def tramp(n, f1, f2, brm, user):
            fn(np.ctypeslib.as_array(f1, (n,)).copy(), np.ctypeslib.as_array(f2, (n,)).copy(),
               np.ctypeslib.as_array(brm, (n * nb,)).reshape(n, nb).copy())

        self._export = EXPORT_FN(tramp)  # kept alive with the session
        check(self.lib.bsa_setBispExportCallback(self._export, None), "bsa_setBispExportCallback")

    def set_visual(self, indexes, modal=True):
        """bsa_enableVisualMode + bsa_setVisualIndexes: bsa_Run writes bsaexport_cls.brm (modal,
        Classic), bsaexport_msh.brm / .brn (Mesher) in the working directory."""
        idx = np.ascontiguousarray(indexes, dtype=np.int32)
        self._keep["visual_indexes"] = idx
        check(self.lib.bsa_enableVisualMode(), "bsa_enableVisualMode")
        check(self.lib.bsa_setVisualIndexes(_p(idx), int(bool(modal))), "bsa_setVisualIndexes")

    def set_brm_export_mode(self, mode=1):
        """bsa_setBRMExportDefaultMode: 1 (base) writes the Mesher's bsaexport_msh.brm."""
        check(self.lib.bsa_setBRMExportDefaultMode(int(mode)), "bsa_setBRMExportDefaultMode")

    def msh_zones_diag(self, zones):
        """Split-precision zone integration with each zone's own m3mr(m, m, m):
        (m3mf, m3mr, zdiag[nz][nm])."""
        arr = (Zone * len(zones))(*zones)
        nm3 = self.dims()[1]
        nm = self.nmodes()
        mf, mr, zd = np.zeros(nm3), np.zeros(nm3), np.zeros((len(zones), nm))
        check(self.lib.bsa_gpu_mshZonesDiag(C.cast(arr, C.c_void_p), len(zones), _p(mf), _p(mr), _p(zd)),
              "bsa_gpu_mshZonesDiag")
        return mf, mr, zd

    def close(self):
        self.lib.bsa_Finalise()
        self._keep.clear()


class Sweep:
    """Batched Classic sweep (bsa_gpu_batch*): cases are snapshotted as they are added, then
    every case is evaluated by one split-precision launch per group of cases."""

    def __init__(self):
        self.lib = load()
        check(self.lib.bsa_gpu_batchClear(), "bsa_gpu_batchClear")
        self.nm, self.nf = [], []

    def add_current(self) -> int:
        """Snapshot the library's current inputs as the next case."""
        cid, nm, nf = C.c_int(0), C.c_int(0), C.c_int(0)
        check(self.lib.bsa_gpu_batchAdd(C.byref(cid)), "bsa_gpu_batchAdd")
        check(self.lib.bsa_gpu_batchCase(cid.value, C.byref(nm), C.byref(nf)), "bsa_gpu_batchCase")
        self.nm.append(nm.value)
        self.nf.append(nf.value)
        return cid.value

    def add(self, prob: Problem) -> int:
        """Set up `prob` (bsa_Init and the setters), snapshot it, release the setup."""
        s = BsaSession(prob, precision=PREC_BF16X3)
        try:
            return self.add_current()
        finally:
            s.close()

    def run(self, form: int = 1):
        """Per case: dict(m3mf, m3mr, m2mr, ms); and the sweep's total device ms.  form 1: the
        E form of the contraction for cases of at most 24 kept modes on odd grids (default);
        0: the D1 / D3 form for every case."""
        check(self.lib.bsa_gpu_setClassicForm(int(form)), "bsa_gpu_setClassicForm")
        try:
            return self._run()
        finally:
            check(self.lib.bsa_gpu_setClassicForm(1), "bsa_gpu_setClassicForm")

    def _run(self):
        n3 = sum(n ** 3 for n in self.nm)
        n2 = sum(n ** 2 for n in self.nm)
        mf, mr, m2 = np.zeros(n3), np.zeros(n3), np.zeros(n2)
        lat = np.zeros(len(self.nm))
        tot = C.c_double(0.0)
        check(self.lib.bsa_gpu_batchRun(_p(mf), _p(mr), _p(m2), _p(lat), C.byref(tot)), "bsa_gpu_batchRun")
        out, o3, o2 = [], 0, 0
        for c, n in enumerate(self.nm):
            out.append({"m3mf": mf[o3:o3 + n ** 3], "m3mr": mr[o3:o3 + n ** 3], "m2mr": m2[o2:o2 + n ** 2],
                        "ms": float(lat[c]), "nm": n, "nf": self.nf[c]})
            o3 += n ** 3
            o2 += n ** 2
        return out, float(tot.value)

    def clear(self):
        check(self.lib.bsa_gpu_batchClear(), "bsa_gpu_batchClear")
        self.nm, self.nf = [], []


class Mlp:
    """The zone-refinement proposer network on the device (bsa_mlp_*)."""

    def __init__(self, din: int, width: int = 128, seed: int = 1):
        self.lib = load()
        h = self.lib.bsa_mlp_create(din, width, seed)
        if h < 0:
            raise BsaError(f"bsa_mlp_create failed ({h}): {self.lib.bsa_mlp_lastError().decode()}")
        self.h, self.din, self.width = h, din, width
        self.np = int(self.lib.bsa_mlp_num_params(h))

    def _chk(self, rc, what):
        if rc != BSA_OK:
            raise BsaError(f"{what} failed ({rc}): {self.lib.bsa_mlp_lastError().decode()}")

    def params(self, bf16=False):
        p = np.zeros(self.np, dtype=np.float32)
        self._chk(self.lib.bsa_mlp_get_params(self.h, _p(p), 1 if bf16 else 0), "bsa_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._chk(self.lib.bsa_mlp_set_params(self.h, _p(p)), "bsa_mlp_set_params")

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros(x.shape[0], dtype=np.float32)
        self._chk(self.lib.bsa_mlp_forward(self.h, _p(x), x.shape[0], _p(out)), "bsa_mlp_forward")
        return out

    def gradients(self, x, y, w):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        w = np.ascontiguousarray(w, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(self.np, dtype=np.float32)
        self._chk(self.lib.bsa_mlp_gradients(self.h, _p(x), _p(y), _p(w), x.shape[0], _p(loss), _p(g)),
                  "bsa_mlp_gradients")
        return float(loss[0]), g

    def train(self, x, y, w, epochs=20, batch=512, lr=1e-3, seed=7):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        w = np.ascontiguousarray(w, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        self._chk(self.lib.bsa_mlp_train(self.h, _p(x), _p(y), _p(w), x.shape[0], epochs, batch, float(lr), seed,
                                         _p(loss)), "bsa_mlp_train")
        return float(loss[0])

    def close(self):
        if self.h is not None:
            self.lib.bsa_mlp_destroy(self.h)
            self.h = None
