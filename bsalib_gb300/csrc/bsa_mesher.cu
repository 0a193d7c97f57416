// bsa_mesher.cu -- the Mesher analysis: the zone layout (bsa_premesh.cu), then all zones
// evaluated in one batched device pass (the FP64 contraction over every zone's BFM lattice
// points, with the bilinear BRM neighbourhood and the trapezoid zone weights in its epilogue).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {

// Zone integration in the precision selected by bsa_gpu_setPrecision: the split-precision
// path evaluates the axis-aligned zones on the tensor cores (bsa_msh_mixed.cu); the
// diagonal-only spectra and the FP64 setting use the FP64 point kernel.
int Engine::run_zones(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts) {
    if (precision == BSA_PREC_BF16X3 && !set.onlyd) return run_zones_mixed(zones, m3mf, m3mr, npts);
    return run_zones_fp64(zones, m3mf, m3mr, npts);
}

// Every zone's BFM lattice points in one point list; m3mf weights are the trapezoid
// weights of the BFM lattice, the BRM lattice is handled in the kernel epilogue.
int Engine::run_zones_fp64(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts) {
    size_t n = 0;
    double nbrm = 0.0;
    for (const ZoneDev &z : zones) {
        if (z.ni < 2 || z.nj < 2 || z.Fi < 1 || z.Fj < 1)
            return fail(BSA_ERR_ARG, "zone lattice needs ni, nj >= 2 and Fi, Fj >= 1");
        n += (size_t)z.ni * z.nj;
        nbrm += (double)((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1);
    }
    if (n == 0) return fail(BSA_ERR_ARG, "empty zone list");
    if (n > (size_t)0x7fffffff) return fail(BSA_ERR_ARG, "too many zone points");
    std::vector<double> f1(n), f2(n), w(n);
    std::vector<int> zid(n), zi(n), zj(n);
    size_t p = 0;
    for (size_t k = 0; k < zones.size(); ++k) {
        const ZoneDev &z = zones[k];
        for (int i = 0; i < z.ni; ++i)
            for (int j = 0; j < z.nj; ++j, ++p) {
                f1[p] = z.fi0 + i * z.dIi + j * z.dJi;
                f2[p] = z.fj0 + i * z.dIj + j * z.dJj;
                const double ti = (i == 0 || i == z.ni - 1) ? 0.5 : 1.0, tj = (j == 0 || j == z.nj - 1) ? 0.5 : 1.0;
                w[p] = z.sym * z.wI * z.wJ * ti * tj;
                zid[p] = (int)k;
                zi[p] = i;
                zj[p] = j;
            }
    }
    int rc = run_points(f1.data(), f2.data(), w.data(), 0.0, (long long)n, m3mf, m3mr, nullptr, nullptr, &zones,
                        zid.data(), zi.data(), zj.data());
    if (rc) return rc;
    last_points = nbrm;
    if (npts) {
        npts[0] = (double)n;
        npts[1] = nbrm;
    }
    return BSA_OK;
}

ZoneDev zone_from_abi(const bsa_zone &z) {
    ZoneDev d;
    d.fi0 = z.fi0; d.fj0 = z.fj0; d.dIi = z.dIi; d.dIj = z.dIj; d.dJi = z.dJi; d.dJj = z.dJj;
    d.ni = z.ni; d.nj = z.nj; d.Fi = z.Fi; d.Fj = z.Fj; d.sym = z.sym;
    d.wI = std::sqrt(z.dIi * z.dIi + z.dIj * z.dIj) * kPi2;
    d.wJ = std::sqrt(z.dJi * z.dJi + z.dJj * z.dJj) * kPi2;
    return d;
}

// Triangular zones: each triangle's post-mesh lattice traced on the host (bsa_triang.cu), then
// every BFM point of every triangle in one FP64 point pass, each with the BRM points it feeds
// and their coefficients (integration weight times interpolation share) listed for the epilogue.
int Engine::run_triangles(const std::vector<TriDump> &tris, double *m3mf, double *m3mr, double *npts) {
    std::vector<double> f1, f2, w, cq;
    std::vector<long long> cptr(1, 0);
    double nbrm = 0.0;
    TriLattice L;
    for (const TriDump &t : tris) {
        const char *err = nullptr;
        int rc = triangle_lattice(t, visual, L, &err);
        if (rc) return fail(rc, "%s", err ? err : "triangle lattice");
        const size_t nb = L.bf1.size();
        std::vector<long long> ptr(nb + 1, 0);
        for (size_t r = 0; r < L.q1.size(); ++r)
            if (L.qw[r] != 0.0)
                for (int k = L.qptr[r]; k < L.qptr[r + 1]; ++k) ++ptr[(size_t)L.qsrc[k] + 1];
        for (size_t b = 0; b < nb; ++b) ptr[b + 1] += ptr[b];
        const size_t e0 = cq.size() / 3;
        cq.resize(3 * (e0 + (size_t)ptr[nb]));
        std::vector<long long> fill(ptr.begin(), ptr.end() - 1);
        for (size_t r = 0; r < L.q1.size(); ++r) {
            if (L.qw[r] == 0.0) continue;
            for (int k = L.qptr[r]; k < L.qptr[r + 1]; ++k) {
                const size_t e = e0 + (size_t)fill[(size_t)L.qsrc[k]]++;
                cq[3 * e] = L.q1[r];
                cq[3 * e + 1] = L.q2[r];
                cq[3 * e + 2] = t.sym * L.qw[r] * L.qc[k];
            }
        }
        for (size_t b = 0; b < nb; ++b) {
            f1.push_back(L.bf1[b]);
            f2.push_back(L.bf2[b]);
            w.push_back(t.sym * L.bw[b]);
            cptr.push_back((long long)e0 + ptr[b + 1]);
        }
        nbrm += (double)L.q1.size();
    }
    const long long n = (long long)f1.size();
    if (n == 0) return fail(BSA_ERR_ARG, "empty triangle list");
    if (n > 0x7fffffffLL) return fail(BSA_ERR_ARG, "too many triangle points");
    int rc = run_points(f1.data(), f2.data(), w.data(), 0.0, n, m3mf, m3mr, nullptr, nullptr, nullptr, nullptr,
                        nullptr, nullptr, cptr.data(), cq.data());
    if (rc) return rc;
    last_points = nbrm;
    if (npts) {
        npts[0] = (double)n;
        npts[1] = nbrm;
    }
    return BSA_OK;
}

int Engine::run_mesher(double *m3mf, double *m3mr) {
    std::vector<ZoneDev> zones;
    std::vector<int> pol, order;
    std::vector<TriDump> tris;
    std::vector<unsigned char> swapped;
    int rc = mesher_zones(zones, pol, &tris, &order, &swapped);
    if (rc) return rc;
    const long long nm3 = dim_bisp();
    std::vector<double> mf(nm3, 0.0), mr(nm3, 0.0);
    if ((rc = run_zones(zones, mf.data(), mr.data(), nullptr))) return rc;
    if (!tris.empty()) {
        // the triangles' pass after the rectangles', its counters added to theirs
        const int k0 = kernels, g0 = graph_launches;
        const double h0 = h2d, d0 = d2h, p0 = last_points, ms0 = last_ms, mg0 = last_ms_gemm,
                     mc0 = last_ms_contraction;
        std::vector<double> tf(nm3), tr(nm3);
        if ((rc = run_triangles(tris, tf.data(), tr.data(), nullptr))) return rc;
        for (long long x = 0; x < nm3; ++x) {
            mf[x] += tf[x];
            mr[x] += tr[x];
        }
        kernels += k0;
        graph_launches += g0;
        h2d += h0;
        d2h += d0;
        last_points += p0;
        last_ms += (float)ms0;
        last_ms_gemm += mg0;
        last_ms_contraction += mc0;
    }
    if (m3mf) std::memcpy(m3mf, mf.data(), sizeof(double) * nm3);
    if (m3mr) std::memcpy(m3mr, mr.data(), sizeof(double) * nm3);
    if (!(export_fn || brm_file_wanted(false))) return BSA_OK;
    const double pts = last_points;
    const float ms = last_ms;
    rc = zones_export(zones, tris, order, swapped);
    last_points = pts;
    last_ms = ms;
    return rc;
}

// The Mesher's response-bispectrum export (the post-mesh interpolation hands every BRM
// lattice point of a zone to write_brm_fptr_, zones/_shared_poly2d.fi:1040-1210; the callback
// is set by bsa_setBispExportCallback, BsaLibImpl.F90:1809-1816).  Per zone: the force
// bispectra at its BFM lattice from the FP64 point path, then at every BRM lattice point the
// bilinear interpolation of the BFM values at the corners of its cell (the weights the zone
// integration uses) times Re[H_m(w1) H_n(w2) conj H_o(w1 + w2)] at the point.  One callback
// per zone, points i fastest then j, brm laid out [npts][dim_bisp].
int Engine::zones_export(const std::vector<ZoneDev> &zones, const std::vector<TriDump> &tris,
                         const std::vector<int> &order, const std::vector<unsigned char> &swapped) {
    const long long nb = dim_bisp();
    const int nm = nme;
    const bool diag = set.onlyd != 0;
    std::vector<double> bfm, brm, f1, f2, pi, pj, mf(nb), mr(nb), H(6 * (size_t)nm);
    // Re[H_m(w1) H_n(w2) conj H_o(w1 + w2)] * b at (v1, v2) for every combination x
    auto brm_at = [&](double v1, double v2, const double *b, double *out) {
        for (int m = 0; m < nm; ++m) {
            frf_eval(hM[m], hK[m], hC[m], v1 * kPi2, H[2 * m], H[2 * m + 1]);
            frf_eval(hM[m], hK[m], hC[m], v2 * kPi2, H[2 * nm + 2 * m], H[2 * nm + 2 * m + 1]);
            frf_eval(hM[m], hK[m], hC[m], (v1 + v2) * kPi2, H[4 * nm + 2 * m], H[4 * nm + 2 * m + 1]);
        }
        for (long long x = 0; x < nb; ++x) {
            const int m = diag ? (int)x : (int)(x % nm);
            const int nn = diag ? (int)x : (int)((x / nm) % nm);
            const int o = diag ? (int)x : (int)(x / ((long long)nm * nm));
            const double h2r = H[2 * nm + 2 * nn], h2i = H[2 * nm + 2 * nn + 1];
            const double h3r = H[4 * nm + 2 * o], h3i = H[4 * nm + 2 * o + 1];
            const double cr = h2r * h3r + h2i * h3i, ci = h2i * h3r - h2r * h3i;  // H_n conj H_o
            out[x] = (H[2 * m] * cr - H[2 * m + 1] * ci) * b[x];
        }
    };
    std::vector<int> seq = order;
    if (seq.empty())
        for (size_t k = 0; k < zones.size(); ++k) seq.push_back((int)k);
    int rc0 = brm_file_open(false, (int)seq.size());
    if (rc0) return rc0;
    long long total = 0;
    TriLattice L;
    for (int item : seq) {
        if (item < 0) {
            // a triangle: the BFM at its BFM points, the BRM at its BRM points from the
            // interpolated BFM, written in the routine's order with its written coordinates
            const TriDump &t = tris[(size_t)(-item - 1)];
            const char *err = nullptr;
            int rc = triangle_lattice(t, visual, L, &err);
            if (rc) {
                brm_file_close(-1);
                return fail(rc, "%s", err ? err : "triangle lattice");
            }
            const size_t np = L.bf1.size(), nq = L.q1.size(), ne = L.e1.size();
            if ((np + nq + ne) * (size_t)nb > ((size_t)1 << 31)) {
                brm_file_close(-1);
                return fail(BSA_ERR_ARG, "zone export block too large");
            }
            bfm.resize(np * nb);
            if ((rc = run_points(L.bf1.data(), L.bf2.data(), nullptr, 0.0, (long long)np, mf.data(), mr.data(),
                                 bfm.data(), nullptr))) {
                brm_file_close(-1);
                return rc;
            }
            std::vector<double> qv(nq * nb), bi((size_t)nb);
            for (size_t r = 0; r < nq; ++r) {
                std::fill(bi.begin(), bi.end(), 0.0);
                for (int k = L.qptr[r]; k < L.qptr[r + 1]; ++k) {
                    const double *src = bfm.data() + (size_t)L.qsrc[k] * nb;
                    for (long long x = 0; x < nb; ++x) bi[x] += L.qc[k] * src[x];
                }
                brm_at(L.q1[r], L.q2[r], bi.data(), qv.data() + r * nb);
            }
            brm.assign(ne * nb, 0.0);
            for (size_t e = 0; e < ne; ++e)
                if (L.eq[e] >= 0) std::memcpy(brm.data() + e * nb, qv.data() + (size_t)L.eq[e] * nb, sizeof(double) * nb);
            if ((rc = brm_file_zone(2, L.nI, L.nJ)) ||
                (rc = emit_brm((int)ne, L.e1.data(), L.e2.data(), brm.data()))) {
                brm_file_close(-1);
                return rc;
            }
            total += (long long)ne;
            continue;
        }
        const ZoneDev &z = zones[(size_t)item];
        const bool sw = (size_t)item < swapped.size() && swapped[(size_t)item];
        if (z.ni < 2 || z.nj < 2 || z.Fi < 1 || z.Fj < 1)
            return fail(BSA_ERR_ARG, "zone lattice needs ni, nj >= 2 and Fi, Fj >= 1");
        const int n = z.ni * z.nj;
        pi.resize(n);
        pj.resize(n);
        for (int i = 0; i < z.ni; ++i)
            for (int j = 0; j < z.nj; ++j) {
                pi[(size_t)i * z.nj + j] = z.fi0 + i * z.dIi + j * z.dJi;
                pj[(size_t)i * z.nj + j] = z.fj0 + i * z.dIj + j * z.dJj;
            }
        bfm.resize((size_t)n * nb);
        int rc = run_points(pi.data(), pj.data(), nullptr, 0.0, n, mf.data(), mr.data(), bfm.data(), nullptr, nullptr,
                            nullptr, nullptr, nullptr);
        if (rc) return rc;
        const int NI = (z.ni - 1) * z.Fi + 1, NJ = (z.nj - 1) * z.Fj + 1;
        const size_t nq = (size_t)NI * NJ;
        if (nq * (size_t)nb > ((size_t)1 << 31)) return fail(BSA_ERR_ARG, "zone export block too large");
        brm.resize(nq * nb);
        f1.resize(nq);
        f2.resize(nq);
        for (int qj = 0; qj < NJ; ++qj)
            for (int qi = 0; qi < NI; ++qi) {
                const size_t q = (size_t)qj * NI + qi;
                const double a = (double)qi / z.Fi, b = (double)qj / z.Fj;
                const double v1 = z.fi0 + a * z.dIi + b * z.dJi, v2 = z.fj0 + a * z.dIj + b * z.dJj;
                f1[q] = sw ? v2 : v1;  // written with the walk's coordinate exchange undone
                f2[q] = sw ? v1 : v2;
                // cell corners and their bilinear weights (one corner on a lattice line)
                const int i0 = qi / z.Fi, j0 = qj / z.Fj;
                const double li = (double)(qi % z.Fi) / z.Fi, lj = (double)(qj % z.Fj) / z.Fj;
                const int i1 = li > 0.0 ? i0 + 1 : i0, j1 = lj > 0.0 ? j0 + 1 : j0;
                const double *B00 = bfm.data() + ((size_t)i0 * z.nj + j0) * nb;
                const double *B10 = bfm.data() + ((size_t)i1 * z.nj + j0) * nb;
                const double *B01 = bfm.data() + ((size_t)i0 * z.nj + j1) * nb;
                const double *B11 = bfm.data() + ((size_t)i1 * z.nj + j1) * nb;
                const double c00 = (1.0 - li) * (1.0 - lj), c10 = li * (1.0 - lj), c01 = (1.0 - li) * lj, c11 = li * lj;
                double *out = brm.data() + q * nb;
                for (long long x = 0; x < nb; ++x) out[x] = c00 * B00[x] + c10 * B10[x] + c01 * B01[x] + c11 * B11[x];
                brm_at(v1, v2, out, out);
            }
        if ((rc = brm_file_zone(1, NI, NJ)) || (rc = emit_brm((int)nq, f1.data(), f2.data(), brm.data()))) {
            brm_file_close(-1);
            return rc;
        }
        total += (long long)nq;
    }
    if ((rc0 = brm_file_close(total))) return rc0;
    return BSA_OK;
}

}  // namespace bsa

using bsa::eng;

extern "C" {

int bsa_gpu_mshZones(const bsa_zone *zones, int nz, double *m3mf, double *m3mr, double *npts) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    if (!zones || nz <= 0) return E.fail(BSA_ERR_ARG, "empty zone list");
    std::vector<bsa::ZoneDev> zd(nz);
    for (int k = 0; k < nz; ++k) zd[k] = bsa::zone_from_abi(zones[k]);
    return E.run_zones(zd, m3mf, m3mr, npts);
}

namespace {
bsa::TriDump tri_from_abi(const bsa_triangle &t) {
    bsa::TriDump d;
    d.Ci = t.Ci; d.Cj = t.Cj; d.Ai = t.Ai; d.Aj = t.Aj; d.Bi = t.Bi; d.Bj = t.Bj; d.rot = t.rot; d.sym = t.sym;
    d.n = t.n; d.pol = t.policy; d.bfi = t.bfm_i; d.bfj = t.bfm_j; d.nlevs = t.bfm_levels; d.bri = t.brm_i;
    d.brj = t.brm_j;
    return d;
}
bool tri_ok(const bsa_triangle &t) {
    return t.n >= 2 && t.bfm_i >= 1 && t.bfm_j >= 1 && t.bfm_levels >= 0 && t.bfm_levels <= 8 && t.brm_i >= 1 &&
           t.brm_j >= 1 && t.bfm_i <= 64 && t.bfm_j <= 64 && t.brm_i <= 64 && t.brm_j <= 64;
}
}  // namespace

int bsa_gpu_mshGenerateTriangles(bsa_triangle *tris, int cap, int *nt) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    std::vector<bsa::ZoneDev> zd;
    std::vector<int> pol, order;
    std::vector<bsa::TriDump> td;
    int rc = E.mesher_zones(zd, pol, &td, &order);
    if (rc) return rc;
    if (nt) *nt = (int)td.size();
    for (size_t s = 0; s < order.size(); ++s) {
        if (order[s] >= 0) continue;
        const int k = -order[s] - 1;
        if (k >= cap || !tris) continue;
        const bsa::TriDump &d = td[(size_t)k];
        bsa_triangle &t = tris[k];
        t.Ci = d.Ci; t.Cj = d.Cj; t.Ai = d.Ai; t.Aj = d.Aj; t.Bi = d.Bi; t.Bj = d.Bj; t.rot = d.rot; t.sym = d.sym;
        t.n = d.n; t.policy = d.pol; t.bfm_i = d.bfi; t.bfm_j = d.bfj; t.bfm_levels = d.nlevs; t.brm_i = d.bri;
        t.brm_j = d.brj; t.seq = (int)s;
    }
    return BSA_OK;
}

int bsa_gpu_mshTriangles(const bsa_triangle *tris, int nt, double *m3mf, double *m3mr, double *npts) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    if (!tris || nt <= 0) return E.fail(BSA_ERR_ARG, "empty triangle list");
    std::vector<bsa::TriDump> td((size_t)nt);
    for (int k = 0; k < nt; ++k) {
        if (!tri_ok(tris[k])) return E.fail(BSA_ERR_ARG, "triangle %d: invalid refinements or policy factors", k);
        td[(size_t)k] = tri_from_abi(tris[k]);
    }
    return E.run_triangles(td, m3mf, m3mr, npts);
}

int bsa_gpu_mshTriangLattice(const bsa_triangle *t, int visual, long long *counts, int *oob, double *bfm,
                             double *brm, int *qptr, int *qsrc, double *qc, double *exp, int *eq) {
    bsa::Engine &E = eng();
    if (!t || !counts) return E.fail(BSA_ERR_ARG, "null triangle or counts");
    if (!tri_ok(*t)) return E.fail(BSA_ERR_ARG, "invalid refinements or policy factors");
    bsa::TriLattice L;
    const char *err = nullptr;
    int rc = bsa::triangle_lattice(tri_from_abi(*t), visual != 0, L, &err);
    if (rc) return E.fail(rc, "%s", err ? err : "triangle lattice");
    const size_t nb = L.bf1.size(), nq = L.q1.size(), nnz = L.qsrc.size(), ne = L.e1.size();
    counts[0] = (long long)nb; counts[1] = (long long)nq; counts[2] = (long long)nnz; counts[3] = (long long)ne;
    counts[4] = L.bfm_post; counts[5] = L.brm_post;
    if (oob) *oob = L.oob ? 1 : 0;
    for (size_t k = 0; bfm && k < nb; ++k) {
        bfm[3 * k] = L.bf1[k]; bfm[3 * k + 1] = L.bf2[k]; bfm[3 * k + 2] = L.bw[k];
    }
    for (size_t k = 0; brm && k < nq; ++k) {
        brm[3 * k] = L.q1[k]; brm[3 * k + 1] = L.q2[k]; brm[3 * k + 2] = L.qw[k];
    }
    if (qptr) std::memcpy(qptr, L.qptr.data(), sizeof(int) * (nq + 1));
    if (qsrc && nnz) std::memcpy(qsrc, L.qsrc.data(), sizeof(int) * nnz);
    if (qc && nnz) std::memcpy(qc, L.qc.data(), sizeof(double) * nnz);
    for (size_t k = 0; exp && k < ne; ++k) {
        exp[2 * k] = L.e1[k]; exp[2 * k + 1] = L.e2[k];
    }
    if (eq && ne) std::memcpy(eq, L.eq.data(), sizeof(int) * ne);
    return BSA_OK;
}

int bsa_gpu_mshGenerateZones(bsa_zone *zones, int cap, int *nz) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    std::vector<bsa::ZoneDev> zd;
    std::vector<int> pol;
    std::vector<bsa::TriDump> td;  // returned by bsa_gpu_mshGenerateTriangles
    int rc = E.mesher_zones(zd, pol, &td);
    if (rc) return rc;
    if (nz) *nz = (int)zd.size();
    for (int k = 0; k < (int)zd.size() && k < cap && zones; ++k) {
        const bsa::ZoneDev &d = zd[k];
        bsa_zone &z = zones[k];
        z.fi0 = d.fi0; z.fj0 = d.fj0; z.dIi = d.dIi; z.dIj = d.dIj; z.dJi = d.dJi; z.dJj = d.dJj;
        z.ni = d.ni; z.nj = d.nj; z.Fi = d.Fi; z.Fj = d.Fj; z.sym = d.sym; z.policy = pol[k];
    }
    return BSA_OK;
}

}  // extern "C"
