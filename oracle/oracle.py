"""Python face of the parity oracle -- TEST INFRASTRUCTURE ONLY.

Loads `oracle/liboracle.so` (built from `oracle/bsa_oracle.c` by `build()`), and adds two
independent numpy restatements used to cross-check it on small cases:

* `direct_point`: the BFM at one (f1, f2) point as the plain triple sum over nodes
  (functionsImpl.F90:1494-1538, three terms, no factorisation);
* `pod_point`: the Mesher POD form (getFM_full_tm_scalar_msh_POD_,
  functionsImpl.F90:474-1019) with numpy's symmetric eigensolver in place of LAPACK
  dsyev; with every POD mode kept it must equal the direct form.

Only tests, the smoke check and the benchmark's CPU-baseline leg import this module.

Parity: pinned for the Classic bispectra over frequency pairs and the nodal PSD against the
reference's BsaCL kernel compiled for the host (oracle/bsacl_ref.py,
tests/test_oracle_bsacl_pin.py); the rest through the restatements above.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "bsa_oracle.c")

PI2 = 2.0 * np.pi


def build(force: bool = False) -> str:
    """Compile the oracle (gcc, OpenMP, FP64).  Portable flags only: it is rebuilt on the
    Arm GPU host from the same source."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
               "-o", LIB, SRC, "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        vp = C.c_void_p
        _lib.orc_corr_index.restype = C.c_long
        _lib.orc_corr_index.argtypes = [C.c_int, C.c_int, C.c_int]
        _lib.orc_eval_psd.argtypes = [vp, C.c_int, vp, C.c_int, vp]
        _lib.orc_validate_modes.argtypes = [C.c_int, C.c_int, vp, vp]
        _lib.orc_phitimesc.argtypes = [vp, vp]
        _lib.orc_compute_freqs.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, vp, vp, vp,
                                           C.c_int, vp]
        _lib.orc_cls_vect_bfm.argtypes = [vp, C.c_int, vp, vp, C.c_int, vp, vp, C.c_int]
        _lib.orc_cls_vect_brm.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp]
        _lib.orc_intg_vect.argtypes = [C.c_int, vp, C.c_int, C.c_int, vp, vp, C.c_int, vp, vp]
        _lib.orc_classic_vect.argtypes = [vp, C.c_int, vp] + [vp] * 7 + [C.c_int]
        _lib.orc_cls_scalar_pair.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, vp, vp,
                                             C.c_int, vp, vp, C.c_int, C.c_int]
        _lib.orc_classic_scalar.argtypes = [vp, C.c_int, vp] + [vp] * 5
        _lib.orc_msh_bfm_direct.argtypes = [vp, C.c_double, C.c_double, vp]
        _lib.orc_msh_brm.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, vp]
        _lib.orc_skewness.argtypes = [C.c_int, vp, vp, vp]
        _lib.orc_modal_recomb.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
        _lib.orc_modal_recomb_all.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
        _lib.orc_rect_zone.argtypes = [vp] + [C.c_double] * 6 + [C.c_int] * 4 + [C.c_double, vp, vp]
        _lib.orc_rect_zone_diag.argtypes = _lib.orc_rect_zone.argtypes
        _lib.orc_classic_vect_diag.argtypes = [vp, C.c_int, vp] + [vp] * 7
        _lib.orc_classic_scalar_diag.argtypes = [vp, C.c_int, vp] + [vp] * 5
        _lib.orc_msh_bfm_diag.argtypes = [vp, C.c_double, C.c_double, vp]
        _lib.orc_msh_brm_diag.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, vp]
        _lib.orc_skewness_diag.argtypes = [C.c_int, vp, vp, vp]
        _lib.orc_br_decomp.argtypes = [vp, vp, vp, C.c_int, vp, vp, vp]
        _lib.orc_peak_factors.argtypes = [C.c_int, vp, vp, C.c_double, vp, vp, vp, vp]
    return _lib


class _OrcProblem(C.Structure):
    _fields_ = [
        ("nn", C.c_int), ("nlibs", C.c_int), ("nnl", C.c_int), ("nlibsl", C.c_int),
        ("n_load", C.c_void_p), ("libs_load", C.c_void_p),
        ("psd_type", C.c_int), ("scaling", C.c_int), ("idir", C.c_int), ("ntc", C.c_int),
        ("tc", C.c_void_p), ("nz", C.c_int),
        ("u_mean_ref", C.c_void_p), ("L", C.c_void_p), ("sigma", C.c_void_p),
        ("u_node", C.c_void_p), ("wz_node", C.c_void_p), ("nod_corr", C.c_void_p),
        ("wfc", C.c_void_p), ("ndegw3", C.c_int), ("ndofs", C.c_int), ("nm", C.c_int),
        ("phi", C.c_void_p), ("Mm", C.c_void_p), ("Km", C.c_void_p), ("Cm", C.c_void_p),
        ("nm_eff", C.c_int), ("modes", C.c_void_p), ("phitc", C.c_void_p),
    ]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """Binds one `Problem` to the C oracle (keeps every array alive)."""

    def __init__(self, prob):
        L = lib()
        self.prob = prob
        s = prob.settings
        keep = {}

        def arr(name, a, dt):
            a = np.asfortranarray(np.asarray(a, dtype=dt))
            keep[name] = a
            return _p(a)

        st = _OrcProblem()
        st.nn, st.nlibs, st.nnl, st.nlibsl = prob.nn, prob.nlibs, prob.nnl, prob.nlibsl
        st.n_load = arr("n_load", prob.n_load, np.int32)
        st.libs_load = arr("libs_load", prob.libs_load, np.int32)
        st.psd_type, st.scaling, st.idir = prob.psd_type, s.defsc, int(s.dirs[0])
        st.ntc = len(s.tc)
        st.tc = arr("tc", np.array(s.tc), np.int32)
        st.nz = prob.nz
        st.u_mean_ref = arr("ubref", prob.UBref, np.float64)
        st.L = arr("L", prob.L, np.float64)
        st.sigma = arr("sigma", prob.sigma, np.float64)
        st.u_node = arr("u_node", prob.u_node, np.float64)
        st.wz_node = arr("wz_node", prob.wz_node, np.int32)
        st.nod_corr = arr("nod_corr", prob.nod_corr, np.float64)
        st.wfc = arr("wfc", prob.wfc, np.float64)
        st.ndegw3 = prob.wfc.shape[1]
        st.ndofs, st.nm = prob.ndofs, prob.nm
        st.phi = arr("phi", prob.phi, np.float64)
        st.Mm = arr("Mm", prob.Mg, np.float64)
        st.Km = arr("Km", prob.Kg, np.float64)
        st.Cm = arr("Cm", prob.Cg, np.float64)
        modes = np.zeros(prob.nm, dtype=np.int32)
        nme = L.orc_validate_modes(prob.ndofs, prob.nm, st.phi, _p(modes))
        self.modes = modes[:nme].copy()
        st.nm_eff = nme
        st.modes = arr("modes", self.modes, np.int32)
        phitc = np.zeros((nme, prob.nnl, st.ndegw3), order="F")
        keep["phitc"] = phitc
        st.phitc = _p(phitc)
        self._keep = keep
        self.st = st
        L.orc_phitimesc(C.byref(st), st.phitc)
        self.phitc = phitc
        self.nme = nme

    # -- a1 ------------------------------------------------------------------------------
    def freqs(self, test_mode=None):
        s = self.prob.settings
        tm = s.test if test_mode is None else test_mode
        dfr = float(np.min(self.prob.xsi * self.prob.natf)) / 5.0
        cap = 4 * (s.nfreqs + 8) + 1024 + 2 * int(np.max(self.prob.natf) / max(dfr, 1e-300))
        f = np.zeros(cap)
        dfo = np.zeros(1)
        nf = lib().orc_compute_freqs(s.nfreqs, s.df, s.defsc, tm, self.prob.nm, _p(self.prob.natf),
                                     _p(self.prob.xsi), _p(f), cap, _p(dfo))
        if nf < 0:
            raise ValueError(f"orc_compute_freqs failed ({nf})")
        return f[:nf].copy()

    # -- a2 ------------------------------------------------------------------------------
    def psd(self, f, tc):
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.zeros((f.size, self.prob.nnl), order="F")
        if lib().orc_eval_psd(C.byref(self.st), f.size, _p(f), int(tc), _p(out)):
            raise ValueError("unsupported PSD id")
        return out

    # -- a5..a7 --------------------------------------------------------------------------
    def classic_vect(self, f=None, keep_bisp=True, nthreads=0):
        f = self.freqs() if f is None else np.ascontiguousarray(f, dtype=np.float64)
        nf, nm = f.size, self.nme
        out = {k: np.zeros(nm * nm) for k in ("m2mf", "m2mr", "m2o2mr")}
        out.update({k: np.zeros(nm ** 3) for k in ("m3mf", "m3mr")})
        bf = np.zeros((nf, nf, nm ** 3), order="F") if keep_bisp else None
        br = np.zeros((nf, nf, nm ** 3), order="F") if keep_bisp else None
        rc = lib().orc_classic_vect(C.byref(self.st), nf, _p(f), _p(out["m2mf"]), _p(out["m2mr"]),
                                    _p(out["m2o2mr"]), _p(out["m3mf"]), _p(out["m3mr"]),
                                    _p(bf) if keep_bisp else None, _p(br) if keep_bisp else None,
                                    int(nthreads))
        if rc:
            raise RuntimeError(f"orc_classic_vect failed ({rc})")
        out["f"] = f
        if keep_bisp:
            out["bf"], out["br"] = bf, br
        return out

    def classic_scalar(self, f=None):
        f = self.freqs() if f is None else np.ascontiguousarray(f, dtype=np.float64)
        nm = self.nme
        out = {k: np.zeros(nm * nm) for k in ("m2mf", "m2mr", "m2o2mr")}
        out.update({k: np.zeros(nm ** 3) for k in ("m3mf", "m3mr")})
        rc = lib().orc_classic_scalar(C.byref(self.st), f.size, _p(f), _p(out["m2mf"]), _p(out["m2mr"]),
                                      _p(out["m2o2mr"]), _p(out["m3mf"]), _p(out["m3mr"]))
        if rc:
            raise RuntimeError(f"orc_classic_scalar failed ({rc})")
        return out

    def scalar_pair_slice(self, f, S, Spad, ii, ij, k_lo, k_hi):
        """One pair of the scalar Classic BFM restricted to k-nodes [k_lo, k_hi)
        (the CPU-baseline sample)."""
        nm = self.nme
        psd = np.zeros(nm * nm)
        bisp = np.zeros(nm ** 3)
        lib().orc_cls_scalar_pair(C.byref(self.st), f.size, ii, ij, float(f[ii]), float(f[ij]), _p(S),
                                  _p(Spad), 1, _p(psd), _p(bisp), int(k_lo), int(k_hi))
        return bisp

    def suvw(self, f):
        """Classic nodal PSD table S_uvw(nf, nnl*ntc) (BsaClassicImpl.F90:103-119)."""
        cols = [self.psd(f, tc) for tc in self.prob.settings.tc]
        return np.asfortranarray(np.concatenate(cols, axis=1))

    # -- a9, a11 ---------------------------------------------------------------------------
    def msh_bfm(self, fi, fj):
        out = np.zeros(self.nme ** 3)
        rc = lib().orc_msh_bfm_direct(C.byref(self.st), float(fi), float(fj), _p(out))
        if rc:
            raise RuntimeError(f"orc_msh_bfm_direct failed ({rc})")
        return out

    def msh_brm(self, fi, fj, bfm):
        fi = np.ascontiguousarray(np.atleast_1d(fi), dtype=np.float64)
        fj = np.ascontiguousarray(np.atleast_1d(fj), dtype=np.float64)
        bfm = np.asfortranarray(bfm.reshape(self.nme ** 3, fi.size * fj.size, order="F"))
        out = np.zeros_like(bfm)
        lib().orc_msh_brm(C.byref(self.st), fi.size, _p(fi), fj.size, _p(fj), _p(bfm), _p(out))
        return out

    # -- a12 ------------------------------------------------------------------------------
    def rect_zone(self, fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym=1.0):
        """(m3mf, m3mr) contributions of one rectangular zone."""
        mf, mr = np.zeros(self.nme ** 3), np.zeros(self.nme ** 3)
        rc = lib().orc_rect_zone(C.byref(self.st), fi0, fj0, dIi, dIj, dJi, dJj, int(ni), int(nj), int(Fi),
                                 int(Fj), float(sym), _p(mf), _p(mr))
        if rc:
            raise RuntimeError(f"orc_rect_zone failed ({rc})")
        return mf, mr

    # -- a16: diagonal-only spectra (length-nm tensors) -------------------------------------
    def classic_vect_diag(self, f=None, keep_bisp=True):
        f = self.freqs() if f is None else np.ascontiguousarray(f, dtype=np.float64)
        nf, nm = f.size, self.nme
        out = {k: np.zeros(nm) for k in ("m2mf", "m2mr", "m2o2mr", "m3mf", "m3mr")}
        bf = np.zeros((nf, nf, nm), order="F") if keep_bisp else None
        br = np.zeros((nf, nf, nm), order="F") if keep_bisp else None
        rc = lib().orc_classic_vect_diag(C.byref(self.st), nf, _p(f), _p(out["m2mf"]), _p(out["m2mr"]),
                                         _p(out["m2o2mr"]), _p(out["m3mf"]), _p(out["m3mr"]),
                                         _p(bf) if keep_bisp else None, _p(br) if keep_bisp else None)
        if rc:
            raise RuntimeError(f"orc_classic_vect_diag failed ({rc})")
        out["f"] = f
        if keep_bisp:
            out["bf"], out["br"] = bf, br
        return out

    def classic_scalar_diag(self, f=None):
        f = self.freqs() if f is None else np.ascontiguousarray(f, dtype=np.float64)
        out = {k: np.zeros(self.nme) for k in ("m2mf", "m2mr", "m2o2mr", "m3mf", "m3mr")}
        rc = lib().orc_classic_scalar_diag(C.byref(self.st), f.size, _p(f), _p(out["m2mf"]), _p(out["m2mr"]),
                                           _p(out["m2o2mr"]), _p(out["m3mf"]), _p(out["m3mr"]))
        if rc:
            raise RuntimeError(f"orc_classic_scalar_diag failed ({rc})")
        return out

    def msh_bfm_diag(self, fi, fj):
        out = np.zeros(self.nme)
        rc = lib().orc_msh_bfm_diag(C.byref(self.st), float(fi), float(fj), _p(out))
        if rc:
            raise RuntimeError(f"orc_msh_bfm_diag failed ({rc})")
        return out

    def msh_brm_diag(self, fi, fj, bfm):
        fi = np.ascontiguousarray(np.atleast_1d(fi), dtype=np.float64)
        fj = np.ascontiguousarray(np.atleast_1d(fj), dtype=np.float64)
        bfm = np.asfortranarray(bfm.reshape(self.nme, fi.size * fj.size, order="F"))
        out = np.zeros_like(bfm)
        lib().orc_msh_brm_diag(C.byref(self.st), fi.size, _p(fi), fj.size, _p(fj), _p(bfm), _p(out))
        return out

    def rect_zone_diag(self, fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym=1.0):
        mf, mr = np.zeros(self.nme), np.zeros(self.nme)
        rc = lib().orc_rect_zone_diag(C.byref(self.st), fi0, fj0, dIi, dIj, dJi, dJj, int(ni), int(nj), int(Fi),
                                      int(Fj), float(sym), _p(mf), _p(mr))
        if rc:
            raise RuntimeError(f"orc_rect_zone_diag failed ({rc})")
        return mf, mr

    def skewness_diag(self, m2, m3):
        sk = np.zeros(self.nme)
        lib().orc_skewness_diag(self.nme, _p(np.ascontiguousarray(m2)), _p(np.ascontiguousarray(m3)), _p(sk))
        return sk

    # -- second-order post-processing -----------------------------------------------------
    def br_decomp(self, m2mf):
        bkg, res = np.zeros(self.nme), np.zeros(self.nme)
        diag = int(self.prob.settings.onlyd)
        rc = lib().orc_br_decomp(C.byref(self.st), _p(np.ascontiguousarray(self.prob.natf, dtype=np.float64)),
                                 _p(np.ascontiguousarray(self.prob.xsi, dtype=np.float64)), diag,
                                 _p(np.ascontiguousarray(m2mf, dtype=np.float64)), _p(bkg), _p(res))
        if rc:
            raise RuntimeError(f"orc_br_decomp failed ({rc})")
        return bkg, res

    def peak_factors(self, m2, m2o2, obs_time, sk=None):
        """(status, peak_g, peak_ng_pos, peak_ng_neg); status 1 / 2 where the reference skips."""
        m2 = np.ascontiguousarray(m2, dtype=np.float64)
        n = m2.size
        g, pos, neg = np.zeros(n), np.zeros(n), np.zeros(n)
        skp = _p(np.ascontiguousarray(sk, dtype=np.float64)) if sk is not None else None
        rc = lib().orc_peak_factors(n, _p(m2), _p(np.ascontiguousarray(m2o2, dtype=np.float64)), float(obs_time),
                                    skp, _p(g), _p(pos), _p(neg))
        return rc, g, pos, neg

    # -- a15 ------------------------------------------------------------------------------
    def skewness(self, m2, m3):
        sk = np.zeros(self.nme ** 3)
        lib().orc_skewness(self.nme, _p(np.ascontiguousarray(m2)), _p(np.ascontiguousarray(m3)), _p(sk))
        return sk

    def modal_recomb(self, m2mr, m3mr):
        phi = np.asfortranarray(self.prob.phi[:, self.modes - 1])
        nd = phi.shape[0]
        m2, m3, sk = np.zeros(nd), np.zeros(nd), np.zeros(nd)
        lib().orc_modal_recomb(nd, phi.shape[1], _p(phi), _p(np.ascontiguousarray(m2mr)),
                               _p(np.ascontiguousarray(m3mr)), _p(m2), _p(m3), _p(sk))
        return m2, m3, sk

    def modal_recomb_all(self, m2mr, m3mr, m2o2mr=None):
        """modalRecombination, both branches (app/bsa.F90:935-1053): dict of m2 / m3 / m2o2 / sk,
        diag and ccc, per DOF of the modal matrix."""
        phi = np.asfortranarray(self.prob.phi[:, self.modes - 1])
        nd = phi.shape[0]
        is_diag = int(np.size(m3mr) == phi.shape[1])
        out, sk = np.zeros(6 * nd), np.zeros(2 * nd)
        lib().orc_modal_recomb_all(nd, phi.shape[1], is_diag, _p(phi), _p(np.ascontiguousarray(m2mr)),
                                   _p(np.ascontiguousarray(m3mr)),
                                   None if m2o2mr is None else _p(np.ascontiguousarray(m2o2mr)), _p(out), _p(sk))
        out = out.reshape(6, nd)
        res = {"m2_diag": out[0], "m3_diag": out[1], "m2o2_diag": out[2], "sk_diag": sk[:nd]}
        if not is_diag:
            res.update({"m2_ccc": out[3], "m3_ccc": out[4], "m2o2_ccc": out[5], "sk_ccc": sk[nd:]})
        return res

    # -- independent numpy restatements -----------------------------------------------------
    def coherence_matrix(self, tc):
        """Dense NNL x NNL coherence base for component tc (getFullNodalPSD's c_ij)."""
        p = self.prob
        nl = p.n_load.astype(np.int64)
        a = np.minimum.outer(nl, nl)
        b = np.maximum.outer(nl, nl)
        idx = (a - 1) * p.nn + b - (a * a - a) // 2
        return p.nod_corr[idx - 1, tc - 1]

    def cross_psd(self, f, tc):
        """S_ij(f) = c_ij^|f| sqrt(S_i S_j) (functionsImpl.F90:1450-1477)."""
        s = self.psd(np.array([f]), tc)[0]
        c = self.coherence_matrix(tc)
        with np.errstate(divide="ignore"):
            return np.power(c, abs(f)) * np.sqrt(np.outer(s, s))

    def direct_point(self, f1, f2, s12=None):
        """B_F^{mno}(f1, f2) by the plain triple sum (numpy einsum); m fastest.
        s12 overrides S(f1+f2) per tc (e.g. zeros for the Classic truncation)."""
        nm = self.nme
        out = np.zeros((nm, nm, nm))
        for it, tc in enumerate(self.prob.settings.tc):
            l = self.phitc[:, :, tc - 1]          # (nm, nnl)
            q = self.phitc[:, :, tc + 2]
            S1 = self.cross_psd(f1, tc)
            S2 = self.cross_psd(f2, tc)
            S3 = self.cross_psd(f1 + f2, tc) if s12 is None else s12[it]
            # term1: q_m(i) l_n(j) l_o(k) S_ij(f1) S_ik(f2)
            t1 = np.einsum("mi,nj,ok,ij,ik->mno", q, l, l, S1, S2, optimize=True)
            # term2: l_m(i) q_n(j) l_o(k) S_ij(f1+f2) S_jk(f2)
            t2 = np.einsum("mi,nj,ok,ij,jk->mno", l, q, l, S3, S2, optimize=True)
            # term3: l_m(i) l_n(j) q_o(k) S_jk(f1) S_ik(f1+f2)
            t3 = np.einsum("mi,nj,ok,jk,ik->mno", l, l, q, S1, S3, optimize=True)
            out += 2.0 * (t1 + t2 + t3)
        return out.reshape(-1, order="F")

    def pod_point(self, f1, f2, trunc_lim=0.0, nmodes=0):
        """Mesher POD form (getFM_full_tm_scalar_msh_POD_, functionsImpl.F90:474-1019; numpy
        eigh, ascending like dsyev).  trunc_lim: bsa_setPODTruncationThreshold's value / 100
        (the count then follows pod_count, :203-230); nmodes: bsa_setPODNOfModesKept, used
        when no threshold is set (:795-815).  Both zero: every POD mode."""
        nm = self.nme
        nnl = self.prob.nnl
        do_trunc = trunc_lim > 0.0 and trunc_lim != 1.0          # BsaLibImpl.F90:479-481
        nfix = nmodes if 0 < nmodes < nnl else 0                  # :482-486

        def top(D, V):
            n = pod_count(D, trunc_lim) if do_trunc else (nfix if nfix else len(D))
            k = len(D) - n
            return D[k:], V[:, k:]

        out = np.zeros((nm, nm, nm))
        for tc in self.prob.settings.tc:
            l = self.phitc[:, :, tc - 1]
            q = self.phitc[:, :, tc + 2]
            D1, V1 = top(*np.linalg.eigh(self.cross_psd(f1, tc)))
            D2, V2 = top(*np.linalg.eigh(self.cross_psd(f2, tc)))
            D3, V3 = top(*np.linalg.eigh(self.cross_psd(f1 + f2, tc)))
            for p in range(V1.shape[1]):
                ep, Dp = V1[:, p], D1[p]
                tm1 = l @ ep
                for qq in range(V2.shape[1]):     # 5-2-2
                    eq, Tq = V2[:, qq], D2[qq]
                    tm2 = q @ (ep * eq)
                    tm3 = l @ eq
                    out += 2 * np.einsum("m,n,o->mno", tm2, tm1, tm3) * Dp * Tq
                for qq in range(V3.shape[1]):     # 2-2-5
                    eq, Tq = V3[:, qq], D3[qq]
                    tm2 = l @ eq
                    tm3 = q @ (ep * eq)
                    out += 2 * np.einsum("m,n,o->mno", tm2, tm1, tm3) * Dp * Tq
            for p in range(V3.shape[1]):          # 2-5-2
                ep, Dp = V3[:, p], D3[p]
                tm1 = l @ ep
                for qq in range(V2.shape[1]):
                    eq, Tq = V2[:, qq], D2[qq]
                    tm2 = l @ eq
                    tm3 = q @ (ep * eq)
                    out += 2 * np.einsum("m,n,o->mno", tm1, tm3, tm2) * Dp * Tq
        return out.reshape(-1, order="F")

    def frf(self, w):
        """H_m(w) for the kept modes (FP64)."""
        m = self.modes - 1
        r = -(w * w * self.prob.Mg[m]) + self.prob.Kg[m]
        ip = self.prob.Cg[m, m] * w
        h = r * r + ip * ip
        return r / h - 1j * (ip / h)

    def brm_factor(self, f1, f2):
        """Re[H_m(w1) H_n(w2) conj(H_o(w1+w2))], m fastest."""
        w1, w2 = PI2 * f1, PI2 * f2
        h1, h2, h3 = self.frf(w1), self.frf(w2), self.frf(w1 + w2)
        return np.real(np.einsum("m,n,o->mno", h1, h2, np.conj(h3))).reshape(-1, order="F")


def pod_count(eig, rlim):
    """getNPODModesByThreshold_ (functionsImpl.F90:203-230) as the reference builds it by
    default (dsyev, ascending eigenvalues eig(1) <= ... <= eig(n)): the count starts at 2 and
    walks DOWN while eig(count) >= rlim * eig(n), then subtracts one.  With ascending
    eigenvalues that inspects the two smallest ones, so the result is 1 when eig(2) is below
    the limit (the usual case: one POD mode kept) and 0 when eig(2) reaches it but eig(1) does
    not.  Where eig(1) reaches it too the reference reads eig(0), outside the array; that case
    is taken as 0 modes here."""
    eig = np.asarray(eig, dtype=np.float64)
    if not np.any(eig != eig[-1]):
        return 1
    limval = rlim * eig[-1]
    n = 2
    while n >= 1 and eig[n - 1] >= limval:
        n -= 1
    return max(n - 1, 0)


def classic_weights(nf, df, scaling=1):
    """Classic m3 integration weights of intgSpectraVect_ (BsaClassicImpl.F90:596-632)."""
    d = df * (PI2 if scaling == 1 else 1.0)
    w = np.full((nf, nf), d * d)
    w[0, :] *= 0.5; w[-1, :] *= 0.5; w[:, 0] *= 0.5; w[:, -1] *= 0.5
    for i, j in ((0, 0), (0, nf - 1), (nf - 1, 0), (nf - 1, nf - 1)):
        w[i, j] = -0.5 * d * d
    return w
