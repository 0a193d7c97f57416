"""Problem description for the BFM hot path, and BsaLib's two input files.

`Problem` holds exactly what BsaLib's standalone driver reads from `bsa.extdata`
(app/bsa.F90:696-871) and `bsa.bsadata` (app/bsa.F90:877-930), in the reference's
Fortran (column-major) layouts, so that a problem built here can be written to those
files and a user's existing files can be read back unchanged.

Synthetic workloads (seeded) are built by `cantilever_tower` (the 30-node tower, 4 modes,
129x129 grid) and `tall_building` (400 nodes, u and w components, 24 modes, 1025x1025
grid).  There is no dataset: every array is generated here from the stated formulas.
"""
from __future__ import annotations

import dataclasses
import io
import os
import struct
from typing import Optional

import numpy as np

F64 = np.float64
I32 = np.int32


def _f(a, shape=None):
    a = np.asarray(a, dtype=F64)
    if shape is not None:
        a = a.reshape(shape, order="F")
    return np.asfortranarray(a)


def _i(a, shape=None):
    a = np.asarray(a, dtype=I32)
    if shape is not None:
        a = a.reshape(shape, order="F")
    return np.asfortranarray(a)


@dataclasses.dataclass
class Settings:
    """bsa.bsadata sections GENERAL / CLASSIC / MESHER / DIRECTIONS / TURBULENCE."""

    suban: int = 1          # 1 classic, 2 mesher, 3 both
    vers: int = 2
    defsc: int = 1          # 1 circular-frequency convention, 2 frequency convention
    ipsd: int = 1
    ibisp: int = 1
    onlyd: int = 0
    bispsym: int = 0
    sym3d: int = 0
    test: int = 1
    scalar: int = 0         # 0 vectorised classic, 1 scalar classic
    nfreqs: int = 65
    df: float = 0.03125
    svd: int = 0
    bkgrfmt: int = 20
    bkgaext: float = 2.0
    genpaext: float = 2.0
    maxaext: float = 2.0
    fcov: int = 1
    dumpmod: int = 0
    dirs: tuple = (1,)
    tc: tuple = (1,)


@dataclasses.dataclass
class Problem:
    """Everything `bsa.extdata` carries (app/bsa.F90:696-871), Fortran layouts."""

    nn: int
    nlibs: int
    n_load: np.ndarray          # (nnl,) 1-based
    libs_load: np.ndarray       # (nlibsl,) 1-based
    coords: np.ndarray          # (3, nn)
    i_varu: int
    psd_type: int
    i_vert: int
    ndegw: int                  # wfc has ndegw+3 coefficient columns
    air_dens: float
    rotW2G: np.ndarray          # (3, 3)
    Zref: np.ndarray            # (nz,)
    UBref: np.ndarray           # (nz,)
    L: np.ndarray               # (3, 3, nz)
    sigma: np.ndarray           # (3, nz)
    corrC: np.ndarray           # (3, 3, nz)
    corrEx: np.ndarray          # (3, 3, nz)
    lims: np.ndarray            # (nz+1,)
    rotW2G_z: np.ndarray        # (3, 3, nz)
    incang: np.ndarray          # (nz,)
    wz_node: np.ndarray         # (nn,) 1-based
    wAlt_node: np.ndarray       # (nn,)
    u_node: np.ndarray          # (nn,)
    nod_corr: np.ndarray        # ((nn*nn+nn)/2, 3)
    wfc: np.ndarray             # (nlibsl, ndegw+3, nnl)
    ndofs: int
    nm: int
    natf: np.ndarray            # (nm,)
    phi: np.ndarray             # (ndofs, nm)
    Mg: np.ndarray              # (nm,)
    Kg: np.ndarray              # (nm,)
    Cg: np.ndarray              # (nm, nm)
    xsi: np.ndarray             # (nm,)
    settings: Settings = dataclasses.field(default_factory=Settings)

    @property
    def nnl(self) -> int:
        return int(self.n_load.size)

    @property
    def nlibsl(self) -> int:
        return int(self.libs_load.size)

    @property
    def nz(self) -> int:
        return int(self.Zref.size)

    @property
    def ntc(self) -> int:
        return len(self.settings.tc)

    def classic_nf(self) -> int:
        """Grid size of the classic analysis in test mode (computeFreqsVect_)."""
        n1 = self.settings.nfreqs - 1
        if self.settings.defsc == 1:
            return 2 * n1 + 1
        return n1 + (n1 % 2) + 1


# ----------------------------------------------------------------------------------------
# bsa.extdata (Fortran unformatted stream: raw little-endian int32 / real64, column-major)
# ----------------------------------------------------------------------------------------

def write_extdata(p: Problem, path: str) -> None:
    """Write `bsa.extdata` in the order app/bsa.F90:696-871 reads it
    (and generateBSAInputFiles_, src/bsa/BsaLibImpl.F90:2119-2152, writes it)."""
    b = io.BytesIO()

    def wi(*vals):
        for v in vals:
            b.write(struct.pack("<i", int(v)))

    def wd(v):
        b.write(struct.pack("<d", float(v)))

    def wa(a, dt):
        b.write(np.asarray(a, dtype=dt).ravel(order="F").astype("<" + np.dtype(dt).str[1:]).tobytes())

    wi(p.nn, p.nlibs, p.nnl, p.nlibsl)
    wa(p.n_load, I32)
    wa(p.libs_load, I32)
    wa(p.coords, F64)
    wi(p.i_varu, p.psd_type, p.i_vert, p.ndegw)
    wd(p.air_dens)
    wa(p.rotW2G, F64)
    wi(p.nz)
    for a in (p.Zref, p.UBref, p.L, p.sigma, p.corrC, p.corrEx, p.lims, p.rotW2G_z, p.incang):
        wa(a, F64)
    wa(p.wz_node, I32)
    for a in (p.wAlt_node, p.u_node, p.nod_corr, p.wfc):
        wa(a, F64)
    wi(p.ndofs, p.nm)
    for a in (p.natf, p.phi, p.Mg, p.Kg, p.Cg, p.xsi):
        wa(a, F64)
    with open(path, "wb") as fh:
        fh.write(b.getvalue())


def read_extdata(path: str, settings: Optional[Settings] = None) -> Problem:
    """Read `bsa.extdata` (stream form) exactly as app/bsa.F90:696-871 does."""
    with open(path, "rb") as fh:
        buf = fh.read()
    pos = [0]

    def ri(n=1):
        v = np.frombuffer(buf, dtype="<i4", count=n, offset=pos[0]).astype(I32)
        pos[0] += 4 * n
        return v

    def rd(n=1):
        v = np.frombuffer(buf, dtype="<f8", count=n, offset=pos[0]).astype(F64)
        pos[0] += 8 * n
        return v

    nn, nlibs, nnl, nlibsl = (int(x) for x in ri(4))
    n_load = ri(nnl)
    libs_load = ri(nlibsl)
    coords = _f(rd(3 * nn), (3, nn))
    i_varu, psd_type, i_vert, ndegw = (int(x) for x in ri(4))
    air = float(rd(1)[0])
    rot = _f(rd(9), (3, 3))
    nz = int(ri(1)[0])
    Zref = rd(nz)
    UBref = rd(nz)
    L = _f(rd(9 * nz), (3, 3, nz))
    sigma = _f(rd(3 * nz), (3, nz))
    corrC = _f(rd(9 * nz), (3, 3, nz))
    corrEx = _f(rd(9 * nz), (3, 3, nz))
    lims = rd(nz + 1)
    rotz = _f(rd(9 * nz), (3, 3, nz))
    incang = rd(nz)
    wz = ri(nn)
    walt = rd(nn)
    unod = rd(nn)
    ncorr = (nn * nn + nn) // 2
    corr = _f(rd(3 * ncorr), (ncorr, 3))
    wfc = _f(rd(nlibsl * (ndegw + 3) * nnl), (nlibsl, ndegw + 3, nnl))
    ndofs, nm = (int(x) for x in ri(2))
    natf = rd(nm)
    phi = _f(rd(ndofs * nm), (ndofs, nm))
    Mg = rd(nm)
    Kg = rd(nm)
    Cg = _f(rd(nm * nm), (nm, nm))
    xsi = rd(nm)
    if pos[0] != len(buf):
        raise ValueError(f"bsa.extdata: {len(buf) - pos[0]} trailing bytes")
    return Problem(nn, nlibs, _i(n_load), _i(libs_load), coords, i_varu, psd_type, i_vert, ndegw,
                   air, rot, _f(Zref), _f(UBref), L, sigma, corrC, corrEx, _f(lims), rotz,
                   _f(incang), _i(wz), _f(walt), _f(unod), corr, wfc, ndofs, nm, _f(natf), phi,
                   _f(Mg), _f(Kg), Cg, _f(xsi), settings or Settings())


def write_bsadata(s: Settings, path: str) -> None:
    """Write `bsa.bsadata` with the section layout of src/bsa/BsaLibImpl.F90:2072-2112."""
    lines = ["-GENERAL:"]
    lines += [f"{v:4d}" for v in (s.suban, s.vers, s.defsc, s.ipsd, s.ibisp, s.onlyd, s.bispsym, s.sym3d, s.test)]
    lines += ["-CLASSIC:", f"{s.scalar:4d}", f"{s.nfreqs:4d}", repr(float(s.df))]
    lines += ["-MESHER:", f"{s.svd:4d}", f"{s.bkgrfmt:4d}", repr(float(s.bkgaext)), repr(float(s.genpaext)),
              repr(float(s.maxaext)), f"{s.fcov:4d}", f"{s.dumpmod:4d}"]
    lines += ["-DIRECTIONS:", f"{len(s.dirs):4d}"] + [f"{d:4d}" for d in s.dirs]
    lines += ["-TURBULENCE:", f"{len(s.tc):4d}"] + [f"{t:4d}" for t in s.tc]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_bsadata(path: str) -> Settings:
    """Read `bsa.bsadata` in the order of getBsaData (app/bsa.F90:877-930)."""
    with open(path) as fh:
        rows = [ln.strip() for ln in fh]
    it = iter(rows)

    def label():
        v = next(it)
        if not v.startswith("-"):
            raise ValueError(f"bsa.bsadata: expected a section label, got {v!r}")

    def rint():
        return int(next(it).split()[0])

    def rflt():
        return float(next(it).split()[0].replace("d", "e").replace("D", "e"))

    s = Settings()
    label()
    s.suban, s.vers, s.defsc, s.ipsd, s.ibisp, s.onlyd, s.bispsym, s.sym3d, s.test = (rint() for _ in range(9))
    label()
    s.scalar = rint(); s.nfreqs = rint(); s.df = rflt()
    label()
    s.svd = rint(); s.bkgrfmt = rint(); s.bkgaext = rflt(); s.genpaext = rflt(); s.maxaext = rflt()
    s.fcov = rint(); s.dumpmod = rint()
    label()
    nd = rint(); s.dirs = tuple(rint() for _ in range(nd))
    label()
    nt = rint(); s.tc = tuple(rint() for _ in range(nt))
    return s


def read_inputs(dirname: str) -> Problem:
    """Load `bsa.extdata` + `bsa.bsadata` from a directory (the standalone driver's inputs)."""
    s = read_bsadata(os.path.join(dirname, "bsa.bsadata"))
    return read_extdata(os.path.join(dirname, "bsa.extdata"), s)


def write_inputs(p: Problem, dirname: str) -> None:
    os.makedirs(dirname, exist_ok=True)
    write_extdata(p, os.path.join(dirname, "bsa.extdata"))
    write_bsadata(p.settings, os.path.join(dirname, "bsa.bsadata"))


# ----------------------------------------------------------------------------------------
# Synthetic structures
# ----------------------------------------------------------------------------------------

def packed_coherence(z: np.ndarray, U: np.ndarray, C: float) -> np.ndarray:
    """Davenport coherence base c_ij = exp(-C |z_i - z_j| / Ubar_ij), packed upper
    triangle in the order of util_getCorrVectIndex (src/utils/utility.F90:60-71)."""
    nn = z.size
    i, j = np.triu_indices(nn)  # row-major upper triangle: (0,0..nn-1), (1,1..nn-1), ...
    return np.exp(-C * np.abs(z[i] - z[j]) / (0.5 * (U[i] + U[j])))


def _unit_max(phi: np.ndarray) -> np.ndarray:
    """Normalise each column to max|phi| == 1 exactly (BsaLib keeps only such modes)."""
    phi = phi / np.max(np.abs(phi), axis=0, keepdims=True)
    return phi


def _assemble(z, U, sig_u, sig_v, sig_w, Lu, Lv, Lw, phi, natf, xsi, lin, quad, coh_C,
              psd_type, settings, rho=1.22, Uref=None) -> Problem:
    nn = z.size
    nm = natf.size
    coords = np.zeros((3, nn)); coords[2] = z
    nz = nn  # one wind zone per node: sigma and L may vary along the height
    L = np.zeros((3, 3, nz))
    L[0, 0, :] = Lu; L[1, 0, :] = Lv; L[2, 0, :] = Lw
    L[:, 1:, :] = L[:, :1, :]
    sigma = np.zeros((3, nz)); sigma[0] = sig_u; sigma[1] = sig_v; sigma[2] = sig_w
    ncorr = (nn * nn + nn) // 2
    corr = np.empty((ncorr, 3))
    for c in range(3):
        corr[:, c] = packed_coherence(z, U, coh_C[c])
    wfc = np.zeros((1, 6, nn))
    wfc[0, 0:3, :] = lin
    wfc[0, 3:6, :] = quad
    w = 2 * np.pi * natf
    return Problem(
        nn=nn, nlibs=1, n_load=_i(np.arange(1, nn + 1)), libs_load=_i([1]), coords=_f(coords),
        i_varu=1, psd_type=psd_type, i_vert=3, ndegw=3, air_dens=rho, rotW2G=_f(np.eye(3)),
        Zref=_f(z.copy()), UBref=_f(U.copy() if Uref is None else Uref), L=_f(L), sigma=_f(sigma),
        corrC=_f(np.zeros((3, 3, nz))), corrEx=_f(np.zeros((3, 3, nz))),
        lims=_f(np.concatenate([[0.0], z])), rotW2G_z=_f(np.tile(np.eye(3)[:, :, None], (1, 1, nz))),
        incang=_f(np.zeros(nz)), wz_node=_i(np.arange(1, nn + 1)), wAlt_node=_f(z.copy()),
        u_node=_f(U.copy()), nod_corr=_f(corr), wfc=_f(wfc), ndofs=nn, nm=nm, natf=_f(natf),
        phi=_f(phi), Mg=_f(np.ones(nm)), Kg=_f(w * w), Cg=_f(np.diag(2 * xsi * w)), xsi=_f(xsi),
        settings=settings)


def cantilever_tower(nfreqs: int = 65, df: float = 0.03125, nodes: int = 30) -> Problem:
    """Cantilever tower, H = 100 m, along-wind DOF per node, 4 modes
    phi_k = sin((2k-1) pi z / 2H), f = [0.3, 1.1, 2.4, 4.0] Hz, 1 % damping, unit modal
    mass; U(z) = 30 (z/10)^0.16, I_u = 0.15, von Karman (L = 100 m), Davenport coherence
    exp(-10 |f| |dz| / Ubar), quasi-steady drag 0.5 rho CdA (U+u)^2 (rho 1.22, CdA 2).
    nfreqs = 65, df = 1/32 gives the 129 x 129 grid on [-2, 2] Hz."""
    H = 100.0
    z = np.arange(1, nodes + 1) * (H / nodes)
    U = 30.0 * (z / 10.0) ** 0.16
    natf = np.array([0.3, 1.1, 2.4, 4.0])
    k = np.arange(1, 5)
    phi = _unit_max(np.sin((2 * k[None, :] - 1) * np.pi * z[:, None] / (2 * H)))
    xsi = np.full(4, 0.01)
    rho, CdA = 1.22, 2.0
    lin = np.zeros((3, nodes)); lin[0] = rho * CdA * U
    quad = np.zeros((3, nodes)); quad[0] = 0.5 * rho * CdA
    s = Settings(suban=1, nfreqs=nfreqs, df=df, tc=(1,), test=1)
    return _assemble(z, U, 0.15 * U, 0.1 * U, 0.08 * U, 100.0, 100.0, 100.0, phi, natf, xsi, lin,
                     quad, (10.0, 10.0, 10.0), 1, s, rho=rho)


def tall_building(nodes: int = 400, modes: int = 24, nfreqs: int = 513, df: float = 1.0 / 128,
                  seed: int = 2024) -> Problem:
    """Tall building, 400 nodes over 300 m, u and w turbulence (I_u 0.15, I_w 0.08,
    L_u 150 m, L_w 50 m), 24 modes log-spaced over 0.15-3 Hz, damping U(1 %, 2 %),
    shapes = seeded sums of 6 sines normalised to unit max, U(z) = 35 (z/10)^0.2,
    von Karman spectra, Davenport coherence (C = 10).  Drag coefficients as the tower;
    the w component acts through lin_w = 0.5 rho CdA U and quad_w = 0.125 rho CdA.
    nfreqs = 513, df = 1/128 gives the 1025 x 1025 grid on [-4, 4] Hz."""
    rng = np.random.default_rng(seed)
    H = 300.0
    z = np.arange(1, nodes + 1) * (H / nodes)
    U = 35.0 * (z / 10.0) ** 0.2
    natf = np.geomspace(0.15, 3.0, modes)
    xsi = rng.uniform(0.01, 0.02, modes)
    a = rng.uniform(-1.0, 1.0, (6, modes))
    b = rng.uniform(0.25, 6.0, (6, modes))
    c = rng.uniform(0.0, np.pi, (6, modes))
    zz = z[:, None, None] / H
    phi = _unit_max(np.sum(a[None] * np.sin(b[None] * np.pi * zz + c[None]), axis=1))
    rho, CdA = 1.22, 2.0
    lin = np.zeros((3, nodes)); lin[0] = rho * CdA * U; lin[2] = 0.5 * rho * CdA * U
    quad = np.zeros((3, nodes)); quad[0] = 0.5 * rho * CdA; quad[2] = 0.125 * rho * CdA
    s = Settings(suban=1, nfreqs=nfreqs, df=df, tc=(1, 3), test=1)
    return _assemble(z, U, 0.15 * U, 0.10 * U, 0.08 * U, 150.0, 100.0, 50.0, phi, natf, xsi, lin,
                     quad, (10.0, 10.0, 10.0), 1, s, rho=rho)


def bridge_deck(nodes: int = 1200, modes: int = 60, seed: int = 77, span: float = 1200.0) -> Problem:
    """Long-span bridge deck: `nodes` loaded nodes along `span` m, u and w turbulence
    (I_u 0.10, I_w 0.05, L_u 100 m, L_w 40 m), uniform U = 40 m/s, `modes` modes closely
    spaced over 0.08-1.5 Hz (log spacing with a seeded +-2 % jitter), 0.5 % damping, shapes
    sin(n pi x / span + phase) with seeded integer wave numbers, von Karman spectra,
    Davenport coherence C = 8 on the separation along the deck (stored as the nodes' third
    coordinate; only separations enter).  Mesher analysis (analysis type 2)."""
    rng = np.random.default_rng(seed)
    x = np.arange(1, nodes + 1) * (span / nodes)
    U = np.full(nodes, 40.0)
    natf = np.sort(np.geomspace(0.08, 1.5, modes) * (1.0 + rng.uniform(-0.02, 0.02, modes)))
    xsi = np.full(modes, 0.005)
    nwave = rng.integers(1, 16, modes)
    phase = rng.uniform(0.0, 0.5 * np.pi, modes)
    phi = _unit_max(np.sin(nwave[None, :] * np.pi * x[:, None] / span + phase[None, :]))
    rho, CdA = 1.22, 4.0
    lin = np.zeros((3, nodes)); lin[0] = rho * CdA * U; lin[2] = 0.5 * rho * CdA * U
    quad = np.zeros((3, nodes)); quad[0] = 0.5 * rho * CdA; quad[2] = 0.125 * rho * CdA
    s = Settings(suban=2, nfreqs=65, df=1.5 / 32, tc=(1, 3), test=1)
    return _assemble(x, U, 0.10 * U, 0.07 * U, 0.05 * U, 100.0, 60.0, 40.0, phi, natf, xsi, lin,
                     quad, (8.0, 8.0, 8.0), 1, s, rho=rho)


def random_structure(seed: int, nodes=(30, 600), modes=(4, 40), nfreq_grid=(129, 513),
                     U_mean: Optional[float] = None) -> Problem:
    """A seeded random cantilever (parametric sweeps): nodes uniform in `nodes`, modes
    uniform in `modes`, natural frequencies log-uniform in 0.05-5 Hz, damping 0.3-3 %,
    U 15-50 m/s, I_u 0.08-0.2, Davenport-Uliege spectra."""
    rng = np.random.default_rng(seed)
    nn = int(rng.integers(nodes[0], nodes[1] + 1))
    nm = int(rng.integers(modes[0], modes[1] + 1))
    H = float(rng.uniform(50.0, 400.0))
    z = np.arange(1, nn + 1) * (H / nn)
    Ub = float(rng.uniform(15.0, 50.0)) if U_mean is None else float(U_mean)
    U = Ub * (z / 10.0) ** 0.16
    Iu = float(rng.uniform(0.08, 0.2))
    natf = np.sort(np.exp(rng.uniform(np.log(0.05), np.log(5.0), nm)))
    xsi = rng.uniform(0.003, 0.03, nm)
    a = rng.uniform(-1.0, 1.0, (6, nm))
    b = rng.uniform(0.25, 6.0, (6, nm))
    c = rng.uniform(0.0, np.pi, (6, nm))
    phi = _unit_max(np.sum(a[None] * np.sin(b[None] * np.pi * (z[:, None, None] / H) + c[None]), axis=1))
    rho, CdA = 1.22, 2.0
    lin = np.zeros((3, nn)); lin[0] = rho * CdA * U
    quad = np.zeros((3, nn)); quad[0] = 0.5 * rho * CdA
    nf = int(rng.integers(nfreq_grid[0] // 2, nfreq_grid[1] // 2 + 1)) * 2 + 1
    fmax = 1.25 * natf.max()
    s = Settings(suban=1, nfreqs=(nf - 1) // 2 + 1, df=fmax / ((nf - 1) // 2), tc=(1,), test=1)
    return _assemble(z, U, Iu * U, 0.75 * Iu * U, 0.5 * Iu * U, 120.0, 80.0, 40.0, phi, natf, xsi,
                     lin, quad, (8.0, 8.0, 8.0), 5, s, rho=rho)


def synthetic_zones(prob: Problem, nzones: int = 50000, seed: int = 0, brm_min: int = 8, brm_max: int = 256):
    """A seeded zone list for the batched Mesher workload: about `nzones` axis-aligned zones of
    uneven size tiling [-F, F]^2 (F = 1.25 max natural frequency of the kept modes), refined
    around the resonance ridges f1 = +-f_m, f2 = +-f_m and f1 + f2 = +-f_m (bands of +-8 xi_m f_m)
    and coarse in the background.  A quadtree: starting from 16 x 16 cells, the largest cell that
    crosses a ridge band is split into four until the leaf count reaches `nzones`.  Each leaf is a
    zone with a BFM lattice of 2-5 points per side (seeded) and a BRM lattice of brm_min ..
    brm_max points per side in proportion to the cell's size (the smallest cells brm_min).
    Returns bsalib_gb300.api.Zone records (spatial symmetry 1, policy 0)."""
    import heapq

    from .api import Zone
    rng = np.random.default_rng(seed)
    keep = np.nonzero(np.max(np.abs(prob.phi), axis=0) == 1.0)[0]
    fm = np.asarray(prob.natf, dtype=float)[keep]
    bw = 8.0 * np.asarray(prob.xsi, dtype=float)[keep] * fm
    F = 1.25 * float(fm.max())

    def crosses(x0, x1, y0, y1):
        for c, b in zip(fm, bw):
            for v in (c, -c):
                if x0 <= v + b and x1 >= v - b:
                    return True
                if y0 <= v + b and y1 >= v - b:
                    return True
                if x0 + y0 <= v + b and x1 + y1 >= v - b:
                    return True
        return False

    n0 = 16
    h0 = 2.0 * F / n0
    leaves = []   # (x0, y0, size)
    heap = []     # (-size, x0, y0) of cells crossing a band
    for i in range(n0):
        for j in range(n0):
            x0, y0 = -F + i * h0, -F + j * h0
            if crosses(x0, x0 + h0, y0, y0 + h0):
                heapq.heappush(heap, (-h0, x0, y0))
            else:
                leaves.append((x0, y0, h0))
    while heap and len(leaves) + len(heap) < nzones:
        nh, x0, y0 = heapq.heappop(heap)
        h = -nh / 2.0
        for dx in (0.0, h):
            for dy in (0.0, h):
                a, b = x0 + dx, y0 + dy
                if crosses(a, a + h, b, b + h):
                    heapq.heappush(heap, (-h, a, b))
                else:
                    leaves.append((a, b, h))
    leaves += [(x0, y0, -nh) for nh, x0, y0 in heap]
    hmin = min(h for _, _, h in leaves)
    hmax = max(h for _, _, h in leaves)
    span = max(np.log(hmax / hmin), 1e-12)
    zones = []
    for (x0, y0, h) in sorted(leaves):
        ni, nj = int(rng.integers(2, 6)), int(rng.integers(2, 6))
        # BRM points per side from brm_min (smallest cells) to brm_max (largest), geometric in size
        side = brm_min * (brm_max / brm_min) ** (np.log(h / hmin) / span)
        Fi = max(1, int(np.floor((side - 1) / (ni - 1))))
        Fj = max(1, int(np.floor((side - 1) / (nj - 1))))
        Fi = max(Fi, -(-(brm_min - 1) // (ni - 1)))
        Fj = max(Fj, -(-(brm_min - 1) // (nj - 1)))
        zones.append(Zone(x0, y0, h / (ni - 1), 0.0, 0.0, h / (nj - 1), ni, nj, Fi, Fj, 1.0, 0))
    return zones
