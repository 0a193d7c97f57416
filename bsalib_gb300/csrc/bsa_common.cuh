// bsa_common.cuh -- device-side data layout shared by the BFM kernels of libbsagpu.
//
// Layout in HBM (all FP64 unless stated):
//   k index           k = itc * nnl + i   (turbulent component major, loaded node minor)
//   L[k][m], Q[k][m]  modal projections of the linear / quadratic force coefficients,
//                     L = PHItimesC(:, :, tc), Q = PHItimesC(:, :, tc+3)
//                     (setPhitimesCLocalInstance_, src/bsa/BsaLibImpl.F90:611-671)
//   logc[itc][i][j]   log of the nodal coherence base c_ij for component tc
//   S[f][itc][i]      nodal turbulence PSD (evalPSD_, src/wind/WindPSDImpl.F90:123-144)
//   A[f][k][m]        A(f) = S(f) L with S_ij(f) = c_ij^|f| sqrt(S_i S_j): the per-frequency
//                     factor of the BFM contraction (every term of functionsImpl.F90:1494-1538
//                     is a product of two such factors and one row of Q)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bsa {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kPi2 = 2.0 * kPi;
constexpr double kPi4 = 4.0 * kPi;

// Per (component, loaded node) parameters of the nodal PSD models.
struct PsdNode {
    double U;      // nodal mean wind speed u_node(n)
    double sigma;  // sigmaUVW_wz_(tc, wz)
    double Ls;     // turbulence length scale used by the model
    double Uref;   // u_mean_ref_wz_(wz) (Davenport-Greisch)
};

// How the contraction kernel enumerates its (f1, f2) points.
enum PointMode : int {
    kPointsGrid = 0,   // classic grid: p -> (i1 = p % nf, i2 = p / nf)
    kPointsList = 1,   // explicit lists of A-table rows and weights
};

// A rectangular Mesher zone on the device: BFM lattice point (i, j), 0 <= i < ni,
// 0 <= j < nj, sits at (f1, f2) = (fi0, fj0) + i (dIi, dIj) + j (dJi, dJj).  The response
// bispectrum is integrated on the BRM lattice refined by (Fi, Fj), with the force
// bispectrum interpolated bilinearly between BFM points and the trapezoid weights of the
// zone integration (_shared_poly2d.fi:470-2166): vertex 1/4, border 1/2, centre 1, times
// the lattice cell area (wI / Fi) (wJ / Fj), times the spatial-symmetry factor sym.
struct ZoneDev {
    double fi0, fj0, dIi, dIj, dJi, dJj;
    double wI, wJ;   // BFM lattice steps in rad/s (|dI| 2 pi, |dJ| 2 pi)
    double sym;
    int ni, nj, Fi, Fj;
};

enum WeightMode : int {
    kWeightClassicVect = 0,  // intgSpectraVect_ edge weights (BsaClassicImpl.F90:596-632)
    kWeightUniform = 1,      // one weight for every point (scalar classic, BsaCL)
    kWeightList = 2,         // per point
};

struct PointSrc {
    int mode;
    int nf;                 // grid size (kPointsGrid)
    int n_pad;              // (nf - 1) / 2, centre offset of the padded S(f1+f2) copy
    int trunc;              // 1: S(f1+f2) beyond the grid reads zero
    int sum_base;           // A-table row of the analytic sum table (s = i1 + i2)
    int r0, nr;             // grid rows (f1 index) of this run: i1 in [r0, r0 + nr)
    long long pbase;        // kPointsGrid: point p of the launch is grid point pbase + p
    int sym_rows;           // kPointsGrid, central symmetry: rows i1 < sym_rows weigh twice
    int wmode;
    double wval;            // uniform weight, or d^2 for the classic edge weights
    const double *fgrid;    // grid frequencies (kPointsGrid)
    const int *ix, *iy, *iz; // A rows of f1, f2, f1+f2 (kPointsList; iz < 0: zero)
    const double *w;        // weights (kWeightList)
    const double *f1, *f2;  // point frequencies (kPointsList)
    const ZoneDev *zones;   // optional (kPointsList): BRM neighbourhood of each point
    const int *zid, *zi, *zj; // zone and lattice coordinates of each point
    // optional (kPointsList), listed BRM points: point p feeds entries [cptr[p], cptr[p + 1]) of
    // cq, each (f1, f2, coefficient) of a BRM point, the coefficient its integration weight
    // times the share of this BFM point in its interpolated BFM
    const long long *cptr;
    const double *cq;
};

struct FrfPar {
    const double *M, *K, *C;  // kept modes: generalised mass, stiffness, damping C(m,m)
};

__host__ __device__ inline void frf_eval(double M, double K, double C, double w, double &hr,
                                         double &hi) {
    // H(w) = 1 / (K - w^2 M + i w C)  (functionsImpl.F90:1031-1115)
    const double r = -(w * w * M) + K;
    const double ip = C * w;
    const double h = r * r + ip * ip;
    hr = r / h;
    hi = -ip / h;
}

// Point p of a point source: A/S-table rows of f1, f2, f1+f2 (iz < 0: the sum reads zero),
// integration weight and the two frequencies.
__device__ __forceinline__ void get_point(const PointSrc &ps, long long p, int &ix, int &iy, int &iz,
                                          double &w, double &f1, double &f2) {
    if (ps.mode == kPointsGrid) {
        const int nf = ps.nf;
        const long long q = p + ps.pbase;
        const int i1 = ps.r0 + (int)(q % ps.nr), i2 = (int)(q / ps.nr);
        ix = i1;
        iy = i2;
        const int s = i1 + i2;
        if (ps.trunc) {
            const int c = s - ps.n_pad;
            iz = (c >= 0 && c < nf) ? c : -1;
        } else {
            iz = ps.sum_base + s;
        }
        f1 = ps.fgrid[i1];
        f2 = ps.fgrid[i2];
        if (ps.wmode == kWeightClassicVect) {
            const bool b1 = (i1 == 0 || i1 == nf - 1), b2 = (i2 == 0 || i2 == nf - 1);
            w = ps.wval * ((b1 && b2) ? -0.5 : ((b1 || b2) ? 0.5 : 1.0));
        } else {
            w = ps.wval;
        }
        if (i1 < ps.sym_rows) w *= 2.0;  // the mirror point (nf-1-i1, nf-1-i2) is not evaluated
    } else {
        ix = ps.ix[p];
        iy = ps.iy[p];
        iz = ps.iz[p];
        f1 = ps.f1[p];
        f2 = ps.f2[p];
        w = (ps.wmode == kWeightList) ? ps.w[p] : ps.wval;
    }
}

// Two FP32 lanes in one 64-bit register.  The paired FP32 instructions of sm_100 and later
// (fma.rn.f32x2, mul.rn.f32x2) run both lanes from one issue slot, each lane rounded as the
// scalar fma.rn / mul.rn would round it.
using f2x = unsigned long long;
__device__ __forceinline__ f2x pk2(float lo, float hi) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 up2(f2x v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

}  // namespace bsa
