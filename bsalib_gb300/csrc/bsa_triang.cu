// bsa_triang.cu -- triangular Mesher zones: the post-mesh lattice of a dumped triangle as the
// device integrates it.
//
// The reference interpolates a triangle's BFM onto its BRM lattice in interpolateTZ_HTPC_v3
// (src/bsa/meshing/zones/_shared_poly2d.fi:470-2166, triangle branches): the BFM at the
// pre-mesh lattice (compute_TZ_iso_, :40-454: C..A along the J side, then lines parallel to CA of
// one point less each, the B point last), evaluated again at the policy's BFM refinement points,
// is interpolated linearly along J, along I between consecutive lines and, past the lattice's
// diagonal, from an interpolant along the hypotenuse; the BRM is formed at every BRM point and
// summed with the routine's influence weights into m3mr, the BFM with its own into m3mf.
//
// Every interpolated value is a linear combination of BFM point values, so the walk is run here
// once per zone on symbolic values (the BFM point ids and coefficients each value combines) and
// yields the zone's BFM points with their m3mf weights, its BRM points with their m3mr weights
// and, per BRM point, the BFM points it interpolates.  The device then evaluates each BFM point
// once (the FP64 point kernel) and folds the BRM factors of the points it feeds into its
// epilogue: m3mr = sum_b B_F(b) * sum_q w_q c_qb Re[H(w1_q) H(w2_q) conj H(w1_q + w2_q)].
//
// The walk follows the routine's control flow and its brm(:, slot) work array slot by slot,
// quirks included (they are listed with the design notes): the exchanged start point for rot in
// [pi/2, pi) and [3 pi/2, 2 pi) with unexchanged steps, the dfJ_bfm_lv0_ start of the diagonal
// interpolant on refinement lines, the pre-mesh line's interpolated lines walking the full BRM
// line length nj (past the hypotenuse, from the interpolants the work array still holds), whose
// slots run past the routine's nPtsPost -- those slots are kept here as storage of their own.
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {

namespace {

constexpr double kMachPrec = 1e-12;  // MACHINE_PRECISION (_CONSTANTS.F90:196)
const double kPI = 4.0 * std::atan(1.0);
const double kPId2 = kPI / 2.0, kPIt3d2 = kPI * (3.0 / 2.0), kPIt2c = kPI * 2.0;

// A value of the walk: sum of c[k] * BFM(id[k]).
constexpr int kLinMax = 24;
struct Lin {
    int n = 0;
    int id[kLinMax];
    double c[kLinMax];
};

struct Fail {
    const char *msg;
};

Lin lin_pt(int id) {
    Lin v;
    v.n = 1;
    v.id[0] = id;
    v.c[0] = 1.0;
    return v;
}

void lin_add(Lin &r, int id, double c) {
    for (int k = 0; k < r.n; ++k)
        if (r.id[k] == id) {
            r.c[k] += c;
            return;
        }
    if (r.n == kLinMax) throw Fail{"triangle interpolant with too many terms"};
    r.id[r.n] = id;
    r.c[r.n] = c;
    ++r.n;
}

// (x a + y b) / d
Lin lin_comb(const Lin &x, double a, const Lin &y, double b, double d) {
    Lin r;
    for (int k = 0; k < x.n; ++k) lin_add(r, x.id[k], x.c[k] * a / d);
    for (int k = 0; k < y.n; ++k) lin_add(r, y.id[k], y.c[k] * b / d);
    return r;
}

// getRotatedUnaryDF with both optional outputs (MTriangZoneImpl.F90:209-261)
void rotated_unary_df(double rot, double &vi, double &vj, double &ci, double &cj) {
    if (rot <= kPId2) {
        vi = std::sin(rot);
        vj = std::cos(rot);
    } else if (rot <= kPI) {
        const double a = rot - kPId2;
        vi = std::cos(a);
        vj = -std::sin(a);
    } else if (rot <= kPIt3d2) {
        const double a = rot - kPI;
        vi = -std::sin(a);
        vj = -std::cos(a);
    } else {
        const double a = rot - kPIt3d2;
        vi = -std::cos(a);
        vj = std::sin(a);
    }
    if (std::fabs(vi) < kMachPrec) vi = 0.0;
    if (std::fabs(vj) < kMachPrec) vj = 0.0;
    ci = vj;
    cj = -vi;
    if (std::fabs(ci) < kMachPrec) ci = 0.0;
    if (std::fabs(cj) < kMachPrec) cj = 0.0;
}

bool tri_swaps(double rot) { return (rot >= kPId2 && rot < kPI) || (rot >= kPIt3d2 && rot < kPIt2c); }

double pdist(double ai, double aj, double bi, double bj) {
    const double dx = std::fabs(ai - bi), dy = std::fabs(aj - bj);
    return std::sqrt(dx * dx + dy * dy);
}

// getTriangZoneEquivNPts: int((ni nj + ni) / 2.0 in single precision)
long long equiv_npts(long long ni, long long nj) { return (long long)((float)(ni * nj + ni) / 2.0f); }

// The walk's state and its outputs.
struct Walk {
    TriLattice &L;
    bool sw;
    std::unordered_map<long long, int> slot;  // brm(:, k) -> BRM point (absent: zero)
    Walk(TriLattice &l, bool s) : L(l), sw(s) {}

    int new_bfm(double fi, double fj) {
        L.bf1.push_back(fi);
        L.bf2.push_back(fj);
        L.bw.push_back(0.0);
        return (int)L.bf1.size() - 1;
    }
    void put(long long k, double fi, double fj, const Lin &v) {  // getBRM_msh(brm(:, k), fi, fj, v)
        const int r = (int)L.q1.size();
        L.q1.push_back(fi);
        L.q2.push_back(fj);
        L.qw.push_back(0.0);
        for (int t = 0; t < v.n; ++t) {
            L.qsrc.push_back(v.id[t]);
            L.qc.push_back(v.c[t]);
        }
        L.qptr.push_back((int)L.qsrc.size());
        slot[k] = r;
    }
    void add_brm(long long k, double w) {  // intg += brm(:, k) * w
        auto it = slot.find(k);
        if (it != slot.end()) L.qw[it->second] += w;
    }
    void add_bfm(const Lin &v, double w) {  // intg_bfm += v * w
        for (int t = 0; t < v.n; ++t) L.bw[v.id[t]] += v.c[t] * w;
    }
    void out(double fi, double fj, long long k) {  // write_brm_fptr_(fi_ptr, fj_ptr, brm(:, k))
        auto it = slot.find(k);
        L.e1.push_back(sw ? fj : fi);
        L.e2.push_back(sw ? fi : fj);
        L.eq.push_back(it == slot.end() ? -1 : it->second);
    }
};

}  // namespace

// compute_TZ_iso_ (lattice, dump order) and interpolateTZ_HTPC_v3 (symbolic) of one triangle.
int triangle_lattice(const TriDump &t, bool visual, TriLattice &L, const char **err) {
    const int bfi = t.bfi, bfj = t.bfj, bri = t.bri, brj = t.brj, nlevs = t.nlevs;
    L = TriLattice();
    L.qptr.push_back(0);
    try {
        if (t.n < 2) throw Fail{"triangle with fewer than 2 lattice points per side"};
        const bool sw = tri_swaps(t.rot);
        Walk W(L, sw);
        // ---- pre-mesh lattice (the dumped BFM, ids 0 .. n(n+1)/2 - 1)
        {
            const int n = t.n, Np_m1 = n - 1;
            int Nj_m1 = Np_m1;
            const double df = pdist(t.Ci, t.Cj, t.Ai, t.Aj) / Np_m1;
            double dJi, dJj, dIi, dIj;
            rotated_unary_df(t.rot, dJi, dJj, dIi, dIj);
            dJi *= df; dJj *= df; dIi *= df; dIj *= df;
            double bi = sw ? t.Cj : t.Ci, bj = sw ? t.Ci : t.Cj;
            double fi = bi, fj = bj;
            W.new_bfm(fi, fj);
            for (int j = 2; j <= Nj_m1; ++j) {
                fi += dJi; fj += dJj;
                W.new_bfm(fi, fj);
            }
            fi += dJi; fj += dJj;
            W.new_bfm(fi, fj);
            for (int i = 2; i <= Np_m1; ++i) {
                --Nj_m1;
                bi += dIi; bj += dIj;
                fi = bi; fj = bj;
                W.new_bfm(fi, fj);
                for (int j = 2; j <= Nj_m1; ++j) {
                    fi += dJi; fj += dJj;
                    W.new_bfm(fi, fj);
                }
                fi += dJi; fj += dJj;
                W.new_bfm(fi, fj);
            }
            bi += dIi; bj += dIj;
            W.new_bfm(bi, bj);
        }
        // ---- post-mesh
        int nsi = 1, nsj = 1;
        if (!visual)
            for (int l = 0; l < nlevs; ++l) {
                nsi *= bfi;
                nsj *= bfj;
            }
        const int F = bri > brj ? bri : brj;
        int njOld = t.n - 1;
        const double df_cst = pdist(t.Ci, t.Cj, t.Ai, t.Aj) / njOld;
        double dJi0, dJj0, dIi0, dIj0;
        rotated_unary_df(t.rot, dJi0, dJj0, dIi0, dIj0);
        dIi0 *= df_cst; dIj0 *= df_cst; dJi0 *= df_cst; dJj0 *= df_cst;
        const double dfI0 = df_cst, dfJ0 = df_cst;
        const int npr_i = nsi - 1, npr_j = nsj - 1;
        const double dIi_r = dIi0 / nsi, dIj_r = dIj0 / nsi, dJi_r = dJi0 / nsj, dJj_r = dJj0 / nsj;
        const double dIi_b = dIi_r / F, dIj_b = dIj_r / F, dJi_b = dJi_r / F, dJj_b = dJj_r / F;
        const double dfI_r = dfI0 / nsi, dfI_b = dfI_r / F, dfJ_r = dfJ0 / nsj, dfJ_b = dfJ_r / F;
        double dw = dfI_r * kPIt2c;
        const double ctr_bfm = dw * dw, brd_bfm = ctr_bfm / 2.0, vtx_bfm = brd_bfm / 2.0;
        dw = dfI_b * kPIt2c;
        const double ctr = dw * dw, brd = ctr / 2.0, vtx = brd / 2.0;
        const double vtx_t = vtx / 2, vtx_t_bfm = vtx_bfm / 2;
        const long long ni_lv = t.n - 1, nj_lv = t.n - 1;
        njOld = (int)nj_lv;
        const long long ni = ni_lv * (nsi * F) + 1, nj = nj_lv * (nsj * F) + 1;
        const long long ni_r = ni_lv * nsi + 1, nj_r = nj_lv * nsj + 1;
        if (ni * nj > ((long long)1 << 31)) throw Fail{"triangle BRM lattice too large"};
        long long njNew_picurr = nj, njNew_piprev = 0;
        const int nipI = F - 1, nipJ = nipI;
        const double df_diag_old = std::sqrt(dfI0 * dfI0 + dfJ0 * dfJ0);
        const double df_diag_ref = df_diag_old / nsi, df_diag_b = df_diag_ref / F;
        const long long nPtsPost = equiv_npts(ni, nj);
        L.nI = (int)ni;
        L.nJ = (int)nj;
        std::vector<Lin> left((size_t)nj + 1), right((size_t)nj + 1), itp((size_t)nj + 1);
        const long long right_n = nj - nipJ - 1;
        bool oob = false;
        auto chk = [&](long long k, long long n) {
            if (k < 1 || k > n) oob = true;
        };
        double fbI = sw ? t.Cj : t.Ci, gbI = sw ? t.Ci : t.Cj;
        long long i_brm = 1;
        double fi = fbI, fj = gbI, fbJ = fi, gbJ = fj;
        Lin tail = lin_pt(0), head;
        W.add_bfm(tail, vtx_bfm);
        left[1] = tail;
        W.put(1, fi, fj, left[1]);
        W.out(fi, fj, 1);
        W.add_brm(1, vtx);
        // J side, C to A
        for (int pJhead = 2; pJhead <= t.n; ++pJhead) {
            for (int r = 0; r < npr_j; ++r) {
                fbJ += dJi_r; gbJ += dJj_r;
                head = lin_pt(W.new_bfm(fbJ, gbJ));
                W.add_bfm(head, brd_bfm);
                double dh = dfJ_r, dt = 0.0;
                for (int p = 0; p < nipJ; ++p) {
                    fi += dJi_b; fj += dJj_b; dt += dfJ_b; dh -= dfJ_b;
                    ++i_brm;
                    chk(i_brm, nj);
                    left[i_brm] = lin_comb(head, dt, tail, dh, dfJ_r);
                    W.put(i_brm, fi, fj, left[i_brm]);
                    W.out(fi, fj, i_brm);
                    W.add_brm(i_brm, brd);
                }
                fi += dJi_b; fj += dJj_b;
                ++i_brm;
                chk(i_brm, nj);
                left[i_brm] = head;
                W.put(i_brm, fi, fj, left[i_brm]);
                W.out(fi, fj, i_brm);
                W.add_brm(i_brm, brd);
                tail = head;
            }
            head = lin_pt(pJhead - 1);
            W.add_bfm(head, brd_bfm);
            double dh = dfJ_r, dt = 0.0;
            for (int p = 0; p < nipJ; ++p) {
                fi += dJi_b; fj += dJj_b; dt += dfJ_b; dh -= dfJ_b;
                ++i_brm;
                chk(i_brm, nj);
                left[i_brm] = lin_comb(head, dt, tail, dh, dfJ_r);
                W.put(i_brm, fi, fj, left[i_brm]);
                W.out(fi, fj, i_brm);
                W.add_brm(i_brm, brd);
            }
            fi += dJi_b; fj += dJj_b;
            ++i_brm;
            chk(i_brm, nj);
            left[i_brm] = head;
            W.put(i_brm, fi, fj, left[i_brm]);
            W.out(fi, fj, i_brm);
            W.add_brm(i_brm, brd);
            tail = head;
            fbJ = fi; gbJ = fj;
        }
        W.add_brm(i_brm, -vtx_t);
        W.add_bfm(tail, -vtx_t_bfm);
        int i_bfm_old = t.n;  // 1-based position in the dumped BFM
        // one J-side walk of a new line (refinement or pre-mesh): bfm(head) at the step ahead,
        // the interpolated BRM points between tail and head, then head itself
        auto walk_j = [&](long long &i_brm_shift, long long &ij, const Lin &hd, double wq) {
            double dh = dfJ_r, dt = 0.0;
            for (int p = 0; p < nipJ; ++p) {
                fi += dJi_b; fj += dJj_b; dt += dfJ_b; dh -= dfJ_b;
                ++ij;
                chk(ij, right_n);
                right[ij] = lin_comb(hd, dt, tail, dh, dfJ_r);
                ++i_brm_shift;
                W.put(i_brm_shift, fi, fj, right[ij]);
                W.add_brm(i_brm_shift, wq);
            }
            fi += dJi_b; fj += dJj_b;
            ++ij;
            chk(ij, right_n);
            right[ij] = hd;
            ++i_brm_shift;
            W.put(i_brm_shift, fi, fj, right[ij]);
            W.add_brm(i_brm_shift, ctr);
            tail = hd;
        };
        // the nipI interpolated lines between the previous line (left) and the new one (right)
        auto interp_lines = [&](bool full_nj, double dfJ_start) {
            int njtmp = nipJ;
            double dfJ_oldtmp = dfJ_start, dIcurr = dfI_r, dIprev = 0.0;
            for (int pIprev = 1; pIprev <= nipI; ++pIprev) {
                dIprev += dfI_b;
                dIcurr -= dfI_b;
                for (long long k = 1; k <= njNew_picurr; ++k) itp[k] = lin_comb(left[k], dIcurr, right[k], dIprev, dfI_r);
                fi = fbI + dIi_b * pIprev;
                fj = gbI + dIj_b * pIprev;
                ++i_brm;
                W.put(i_brm, fi, fj, itp[1]);
                W.out(fi, fj, i_brm);
                W.add_brm(i_brm, brd);
                const long long last = full_nj ? nj : njNew_picurr;
                for (long long pJ = 2; pJ <= last; ++pJ) {
                    fi += dJi_b; fj += dJj_b;
                    ++i_brm;
                    W.put(i_brm, fi, fj, itp[pJ]);
                    W.out(fi, fj, i_brm);
                    W.add_brm(i_brm, ctr);
                }
                const Lin hd = lin_comb(left[njNew_piprev], df_diag_b * pIprev, right[njNew_picurr],
                                        df_diag_b * (nipI + 1 - pIprev), df_diag_ref);
                --njtmp;
                dfJ_oldtmp -= dfJ_b;
                double dh = dfJ_oldtmp, dt = 0.0;
                long long ipos = njNew_picurr;
                for (int p = 0; p < njtmp; ++p) {
                    fi += dJi_b; fj += dJj_b; dt += dfJ_b; dh -= dfJ_b;
                    ++ipos;
                    chk(ipos, nj);
                    itp[ipos] = lin_comb(hd, dt, itp[njNew_picurr], dh, dfJ_oldtmp);
                    ++i_brm;
                    W.put(i_brm, fi, fj, itp[ipos]);
                    W.out(fi, fj, i_brm);
                    W.add_brm(i_brm, ctr);
                }
                fi += dJi_b; fj += dJj_b;
                ++i_brm;
                W.put(i_brm, fi, fj, hd);
                W.out(fi, fj, i_brm);
                W.add_brm(i_brm, vtx_t);
            }
        };
        auto shift_start = [&]() {
            long long s = i_brm, tmp = njNew_picurr;
            for (int p = 0; p < nipI; ++p) {
                --tmp;
                s += tmp;
            }
            return s;
        };
        for (int pIcurr = 2; pIcurr <= t.n; ++pIcurr) {
            for (int rI = 1; rI <= npr_i; ++rI) {  // BFM refinement lines before the pre-mesh line
                long long i_brm_shift = shift_start();
                long long i_brm_write = i_brm_shift;
                fbJ = fbI + dIi_r; gbJ = gbI + dIj_r;
                fi = fbJ; fj = gbJ;
                tail = lin_pt(W.new_bfm(fi, fj));
                W.add_bfm(tail, brd_bfm);
                right[1] = tail;
                ++i_brm_shift;
                W.put(i_brm_shift, fi, fj, right[1]);
                W.add_brm(i_brm_shift, brd);
                long long ij = 1;
                for (int pJhead = 2; pJhead <= njOld; ++pJhead) {
                    for (int r = 0; r < npr_j; ++r) {
                        fbJ += dJi_r; gbJ += dJj_r;
                        const Lin hd = lin_pt(W.new_bfm(fbJ, gbJ));
                        W.add_bfm(hd, ctr_bfm);
                        walk_j(i_brm_shift, ij, hd, ctr);
                    }
                    fbJ += dJi_r; gbJ += dJj_r;
                    const Lin hd = lin_pt(W.new_bfm(fbJ, gbJ));
                    W.add_bfm(hd, vtx_bfm);
                    walk_j(i_brm_shift, ij, hd, ctr);
                }
                for (int r = 1; r <= npr_j - (rI - 1); ++r) {
                    fbJ += dJi_r; gbJ += dJj_r;
                    const Lin hd = lin_pt(W.new_bfm(fbJ, gbJ));
                    W.add_bfm(hd, ctr_bfm);
                    walk_j(i_brm_shift, ij, hd, ctr);
                }
                njNew_piprev = njNew_picurr;
                njNew_picurr = ij;
                W.add_brm(i_brm_shift, -brd);
                W.add_bfm(tail, -brd_bfm);
                interp_lines(false, dfJ0);
                fbI += dIi_r; gbI += dIj_r;
                fi = fbI; fj = gbI;
                for (long long k = 0; k < nj; ++k) {
                    ++i_brm_write;
                    W.out(fi, fj, i_brm_write);
                    fi += dJi_b; fj += dJj_b;
                }
                for (long long k = 1; k <= njNew_picurr; ++k) left[k] = right[k];
                i_brm = i_brm_shift;
            }
            // the pre-mesh line
            long long i_brm_shift = shift_start();
            long long i_brm_write = i_brm_shift;
            fbJ = fbI + dIi_r; gbJ = gbI + dIj_r;
            fi = fbJ; fj = gbJ;
            ++i_bfm_old;
            tail = lin_pt(i_bfm_old - 1);
            W.add_bfm(tail, brd_bfm);
            right[1] = tail;
            ++i_brm_shift;
            W.put(i_brm_shift, fi, fj, right[1]);
            W.add_brm(i_brm_shift, brd);
            long long ij = 1;
            for (int pJhead = 2; pJhead <= njOld; ++pJhead) {
                for (int r = 0; r < npr_j; ++r) {
                    fbJ += dJi_r; gbJ += dJj_r;
                    const Lin hd = lin_pt(W.new_bfm(fbJ, gbJ));
                    W.add_bfm(hd, ctr_bfm);
                    walk_j(i_brm_shift, ij, hd, ctr);
                }
                fi = fbJ; fj = gbJ;
                fbJ += dJi_r; gbJ += dJj_r;
                ++i_bfm_old;
                const Lin hd = lin_pt(i_bfm_old - 1);
                W.add_bfm(hd, ctr_bfm);
                walk_j(i_brm_shift, ij, hd, ctr);
            }
            W.add_brm(i_brm_shift, -brd);
            W.add_bfm(tail, -brd_bfm);
            njNew_piprev = njNew_picurr;
            njNew_picurr = ij;
            interp_lines(true, dfJ_r);
            i_brm = i_brm_shift;
            fbI += dIi_r; gbI += dIj_r;
            fi = fbI; fj = gbI;
            for (long long k = 0; k < njNew_picurr; ++k) {
                ++i_brm_write;
                W.out(fi, fj, i_brm_write);
                fi += dJi_b; fj += dJj_b;
            }
            --njOld;
            for (long long k = 1; k <= njNew_picurr; ++k) left[k] = right[k];
        }
        W.add_brm(i_brm, -vtx_t);
        W.add_bfm(tail, -vtx_t_bfm);
        for (auto &kv : W.slot)
            if (kv.first < 1 || kv.first > nPtsPost) oob = true;
        L.bfm_post = equiv_npts(ni_r, nj_r);
        L.brm_post = nPtsPost;
        L.oob = oob;
    } catch (const Fail &f) {
        if (err) *err = f.msg;
        return BSA_ERR_ARG;
    }
    return BSA_OK;
}

}  // namespace bsa
