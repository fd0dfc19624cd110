// plain_flux.cu -- FP64 parity form of the momentum right-hand side and the
// low-storage RK update.  Compiled with -fmad=false: every multiply and add
// is rounded separately, in the operation order of the reference, so the
// results agree with a plain FP64 build of the Fortran bit for bit.
//
//   tstle4_kon   src/flow/tstle4_mod.F90:139-265
//   tstle4_diff  src/flow/tstle4_mod.F90:268-458 (no LES: qc = st*0)
//   tstle4_gradp src/flow/tstle4_mod.F90:461-529
//   rkstep       src/core/rungekutta_mod.F90:315-333
//
// GB300 note: FP64 issues at a small fraction of the FP32 rate on this part,
// so this kernel is FP64-compute bound (~430 flop per cell, incl. divides);
// it is the reference-order baseline, the mixed form is the fast path.
#include "internal.h"

namespace mg {
MG_PLAIN_BEGIN
namespace {

struct GridPtrs {
    int kk, jj, ii;
    const double *dx, *dy, *dz, *ddx, *ddy, *ddz, *rdx, *rdy, *rdz, *rddx, *rddy, *rddz;
    const double *wx, *wy, *wz;   // ddx**(-cwb), ddy**(-cwb), ddz**(-cwb)
};

struct Spacing {
    const double *dx, *dy, *dz, *ddx, *ddy, *ddz, *rdx, *rdy, *rdz, *rddx, *rddy, *rddz;
    const double *wx, *wy, *wz;
};

// The Werner-Wengle constants (wernerwengle_mod.F90:13-28) and the face
// codes of one grid, for swcle3d on NOS (code 5) faces.
struct Wall {
    double rho, gmol, cpo4, cpo5, cpo6, cpo8;
    int bc[6];
    bool any;
    // G equal to one value g0 on every point tstle4_diff reads: each face
    // mean pair hm(g0, g0) + hm(g0, g0) is the same number h2
    bool guni;
    double h2;
};

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))
#define A(a, k, j, i) a[IX(k, j, i)]

__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }
// harmonic face mean of tstle4_diff: g*g'/MAX(g+g', gmol)
__device__ __forceinline__ double hm(double a, double b, double gmol) {
    return a * b / dmax(a + b, gmol);
}

// tauwin (wernerwengle_mod.F90:64-87) over rho and dds, swcle3d_one
// (tstle4_mod.F90:1832-1844); ddsb = dds**(-cwb) comes from the host.
__device__ double swcle3d_one(const Wall& q, double dds, double ddsb, double u) {
    const double vz = copysign(1.0, u);
    const double uquern = fabs(u);
    double tauwin;
    if (uquern >= q.cpo6 / dds)
        tauwin = vz * q.rho * pow(ddsb * (q.cpo4 * uquern + q.cpo5 / dds), q.cpo8);
    else
        tauwin = vz * 2.0 * q.gmol * uquern / dds;
    return tauwin / q.rho / dds;
}

// swcle3d (tstle4_mod.F90:1756-1829) at one point, per component in the
// reference's face order (front, back, right, left, bottom, top); each face
// acts on the layer next to the wall over its rows 2..n-1.
__device__ double wall_u(double x, int k, int j, int i, const GridPtrs& s, const Wall& q, double u) {
    if (!q.any) return x;
    const bool ik = i >= 2 && i <= s.ii - 1 && k >= 2 && k <= s.kk - 1;
    const bool ij = i >= 2 && i <= s.ii - 1 && j >= 2 && j <= s.jj - 1;
    if (q.bc[2] == 5 && j == 3 && ik) x = x - swcle3d_one(q, s.ddy[j], s.wy[j], u);
    if (q.bc[3] == 5 && j == s.jj - 2 && ik) x = x - swcle3d_one(q, s.ddy[j], s.wy[j], u);
    if (q.bc[4] == 5 && k == 3 && ij) x = x - swcle3d_one(q, s.ddz[k], s.wz[k], u);
    if (q.bc[5] == 5 && k == s.kk - 2 && ij) x = x - swcle3d_one(q, s.ddz[k], s.wz[k], u);
    return x;
}
__device__ double wall_v(double x, int k, int j, int i, const GridPtrs& s, const Wall& q, double v) {
    if (!q.any) return x;
    const bool jk = j >= 2 && j <= s.jj - 1 && k >= 2 && k <= s.kk - 1;
    const bool ij = i >= 2 && i <= s.ii - 1 && j >= 2 && j <= s.jj - 1;
    if (q.bc[0] == 5 && i == 3 && jk) x = x - swcle3d_one(q, s.ddx[i], s.wx[i], v);
    if (q.bc[1] == 5 && i == s.ii - 2 && jk) x = x - swcle3d_one(q, s.ddx[i], s.wx[i], v);
    if (q.bc[4] == 5 && k == 3 && ij) x = x - swcle3d_one(q, s.ddz[k], s.wz[k], v);
    if (q.bc[5] == 5 && k == s.kk - 2 && ij) x = x - swcle3d_one(q, s.ddz[k], s.wz[k], v);
    return x;
}
__device__ double wall_w(double x, int k, int j, int i, const GridPtrs& s, const Wall& q, double w) {
    if (!q.any) return x;
    const bool jk = j >= 2 && j <= s.jj - 1 && k >= 2 && k <= s.kk - 1;
    const bool ik = i >= 2 && i <= s.ii - 1 && k >= 2 && k <= s.kk - 1;
    if (q.bc[0] == 5 && i == 3 && jk) x = x - swcle3d_one(q, s.ddx[i], s.wx[i], w);
    if (q.bc[1] == 5 && i == s.ii - 2 && jk) x = x - swcle3d_one(q, s.ddx[i], s.wx[i], w);
    if (q.bc[2] == 5 && j == 3 && ik) x = x - swcle3d_one(q, s.ddy[j], s.wy[j], w);
    if (q.bc[3] == 5 && j == s.jj - 2 && ik) x = x - swcle3d_one(q, s.ddy[j], s.wy[j], w);
    return x;
}

// One output point of tstle4 for the U component (kon, swcle3d, diff, gradp).
__device__ double uo_point(int k, int j, int i, int kk, int jj, const double* u, const double* v,
                           const double* w, const double* ut, const double* vt, const double* wt,
                           const double* p, const double* gg, const GridPtrs& s, const Wall& wl,
                           double gmol, double rho, double iles, double gpx) {
    const double *dx = s.dx, *dy = s.dy, *ddx = s.ddx, *ddy = s.ddy, *ddz = s.ddz;
    const double *rdx = s.rdx, *rdy = s.rdy, *rdz = s.rdz, *rddx = s.rddx, *rddy = s.rddy,
                 *rddz = s.rddz;
    double uo;
    {
        double ax = ddy[j] * ddz[k], ay = dx[i] * ddz[k], az = dx[i] * ddy[j];
        double fe = ax * (A(ut, k, j, i) + (A(ut, k, j, i + 1) - A(ut, k, j, i)) * 0.5 * dx[i] / ddx[i + 1]);
        double fw = ax * (A(ut, k, j, i - 1) + (A(ut, k, j, i) - A(ut, k, j, i - 1)) * 0.5 * dx[i - 1] / ddx[i]);
        double fn = ay * (A(vt, k, j, i) + A(vt, k, j, i + 1)) * 0.5;
        double fs = ay * (A(vt, k, j - 1, i) + A(vt, k, j - 1, i + 1)) * 0.5;
        double ft = az * (A(wt, k, j, i) + A(wt, k, j, i + 1)) * 0.5;
        double fb = az * (A(wt, k - 1, j, i) + A(wt, k - 1, j, i + 1)) * 0.5;
        double qe = 0.5 * fe * (A(u, k, j, i) + A(u, k, j, i + 1));
        double qw = 0.5 * fw * (A(u, k, j, i - 1) + A(u, k, j, i));
        double qn = 0.5 * fn * (A(u, k, j, i) + A(u, k, j + 1, i));
        double qs = 0.5 * fs * (A(u, k, j - 1, i) + A(u, k, j, i));
        double qt = 0.5 * ft * (A(u, k, j, i) + A(u, k + 1, j, i));
        double qb = 0.5 * fb * (A(u, k - 1, j, i) + A(u, k, j, i));
        uo = -(qe - qw + qn - qs + qt - qb) * rdx[i] * rddy[j] * rddz[k];
    }
    uo = wall_u(uo, k, j, i, s, wl, A(u, k, j, i));
    {
        double ax = ddy[j] * ddz[k], ay = dx[i] * ddz[k], az = dx[i] * ddy[j];
        double ge = A(gg, k, j, i + 1);
        double gw = A(gg, k, j, i);
        double gn = wl.guni ? wl.h2 : hm(A(gg, k, j, i), A(gg, k, j + 1, i), gmol) + hm(A(gg, k, j, i + 1), A(gg, k, j + 1, i + 1), gmol);
        double gs = wl.guni ? wl.h2 : hm(A(gg, k, j - 1, i), A(gg, k, j, i), gmol) + hm(A(gg, k, j - 1, i + 1), A(gg, k, j, i + 1), gmol);
        double gt = wl.guni ? wl.h2 : hm(A(gg, k, j, i), A(gg, k + 1, j, i), gmol) + hm(A(gg, k, j, i + 1), A(gg, k + 1, j, i + 1), gmol);
        double gb = wl.guni ? wl.h2 : hm(A(gg, k - 1, j, i), A(gg, k, j, i), gmol) + hm(A(gg, k - 1, j, i + 1), A(gg, k, j, i + 1), gmol);
        double qe = -ge * ax * rddx[i + 1] * (A(u, k, j, i + 1) - A(u, k, j, i));
        double qw = -gw * ax * rddx[i] * (A(u, k, j, i) - A(u, k, j, i - 1));
        double qn = -gn * ay * rdy[j] * (A(u, k, j + 1, i) - A(u, k, j, i));
        double qs = -gs * ay * rdy[j - 1] * (A(u, k, j, i) - A(u, k, j - 1, i));
        double qt = -gt * az * rdz[k] * (A(u, k + 1, j, i) - A(u, k, j, i));
        double qb = -gb * az * rdz[k - 1] * (A(u, k, j, i) - A(u, k - 1, j, i));
        double st = ((ge * (A(u, k, j, i + 1) - A(u, k, j, i)) * rddx[i + 1]) -
                     (gw * (A(u, k, j, i) - A(u, k, j, i - 1)) * rddx[i])) * ax +
                    ((gn * (A(v, k, j, i + 1) - A(v, k, j, i))) -
                     (gs * (A(v, k, j - 1, i + 1) - A(v, k, j - 1, i)))) * ddz[k] +
                    ((gt * (A(w, k, j, i + 1) - A(w, k, j, i))) -
                     (gb * (A(w, k - 1, j, i + 1) - A(w, k - 1, j, i)))) * ddy[j];
        double qc = st * iles;   // the LES cross term (iles = 0 without LES model)
        double fak = 1.0 / rho * rddy[j] * rdx[i] * rddz[k];
        uo = uo - fak * (qe - qw + qn - qs + qt - qb - qc);
    }
    uo = uo - 1.0 / (rho * dx[i]) * (A(p, k, j, i + 1) - A(p, k, j, i) + gpx * dx[i]);
    return uo;
}

__device__ double vo_point(int k, int j, int i, int kk, int jj, const double* u, const double* v,
                           const double* w, const double* ut, const double* vt, const double* wt,
                           const double* p, const double* gg, const GridPtrs& s, const Wall& wl,
                           double gmol, double rho, double iles, double gpy) {
    const double *dy = s.dy, *ddx = s.ddx, *ddy = s.ddy, *ddz = s.ddz;
    const double *rdx = s.rdx, *rdy = s.rdy, *rdz = s.rdz, *rddx = s.rddx, *rddy = s.rddy,
                 *rddz = s.rddz;
    double vo;
    {
        double ax = dy[j] * ddz[k], ay = ddx[i] * ddz[k], az = ddx[i] * dy[j];
        double fe = ax * (A(ut, k, j, i) + A(ut, k, j + 1, i)) * 0.5;
        double fw = ax * (A(ut, k, j, i - 1) + A(ut, k, j + 1, i - 1)) * 0.5;
        double fn = ay * (A(vt, k, j, i) + (A(vt, k, j + 1, i) - A(vt, k, j, i)) * 0.5 * dy[j] / ddy[j + 1]);
        double fs = ay * (A(vt, k, j - 1, i) + (A(vt, k, j, i) - A(vt, k, j - 1, i)) * 0.5 * dy[j - 1] / ddy[j]);
        double ft = az * (A(wt, k, j, i) + A(wt, k, j + 1, i)) * 0.5;
        double fb = az * (A(wt, k - 1, j, i) + A(wt, k - 1, j + 1, i)) * 0.5;
        double qe = 0.5 * fe * (A(v, k, j, i) + A(v, k, j, i + 1));
        double qw = 0.5 * fw * (A(v, k, j, i - 1) + A(v, k, j, i));
        double qn = 0.5 * fn * (A(v, k, j, i) + A(v, k, j + 1, i));
        double qs = 0.5 * fs * (A(v, k, j - 1, i) + A(v, k, j, i));
        double qt = 0.5 * ft * (A(v, k, j, i) + A(v, k + 1, j, i));
        double qb = 0.5 * fb * (A(v, k - 1, j, i) + A(v, k, j, i));
        vo = -(qe - qw + qn - qs + qt - qb) * rddx[i] * rdy[j] * rddz[k];
    }
    vo = wall_v(vo, k, j, i, s, wl, A(v, k, j, i));
    {
        double ax = dy[j] * ddz[k], ay = ddx[i] * ddz[k], az = ddx[i] * dy[j];
        double ge = wl.guni ? wl.h2 : hm(A(gg, k, j, i), A(gg, k, j, i + 1), gmol) + hm(A(gg, k, j + 1, i), A(gg, k, j + 1, i + 1), gmol);
        double gw = wl.guni ? wl.h2 : hm(A(gg, k, j, i - 1), A(gg, k, j, i), gmol) + hm(A(gg, k, j + 1, i - 1), A(gg, k, j + 1, i), gmol);
        double gn = A(gg, k, j + 1, i);
        double gs = A(gg, k, j, i);
        double gt = wl.guni ? wl.h2 : hm(A(gg, k, j, i), A(gg, k + 1, j, i), gmol) + hm(A(gg, k, j + 1, i), A(gg, k + 1, j + 1, i), gmol);
        double gb = wl.guni ? wl.h2 : hm(A(gg, k - 1, j, i), A(gg, k, j, i), gmol) + hm(A(gg, k - 1, j + 1, i), A(gg, k, j + 1, i), gmol);
        double qe = -ge * ax * rdx[i] * (A(v, k, j, i + 1) - A(v, k, j, i));
        double qw = -gw * ax * rdx[i - 1] * (A(v, k, j, i) - A(v, k, j, i - 1));
        double qn = -gn * ay * rddy[j + 1] * (A(v, k, j + 1, i) - A(v, k, j, i));
        double qs = -gs * ay * rddy[j] * (A(v, k, j, i) - A(v, k, j - 1, i));
        double qt = -gt * az * rdz[k] * (A(v, k + 1, j, i) - A(v, k, j, i));
        double qb = -gb * az * rdz[k - 1] * (A(v, k, j, i) - A(v, k - 1, j, i));
        double st = ((ge * (A(u, k, j + 1, i) - A(u, k, j, i))) -
                     (gw * (A(u, k, j + 1, i - 1) - A(u, k, j, i - 1)))) * ddz[k] +
                    ((gn * (A(v, k, j + 1, i) - A(v, k, j, i)) * rddy[j + 1]) -
                     (gs * (A(v, k, j, i) - A(v, k, j - 1, i)) * rddy[j])) * ay +
                    ((gt * (A(w, k, j + 1, i) - A(w, k, j, i))) -
                     (gb * (A(w, k - 1, j + 1, i) - A(w, k - 1, j, i)))) * ddx[i];
        double qc = st * iles;
        double fak = 1.0 / rho * rddx[i] * rdy[j] * rddz[k];
        vo = vo - fak * (qe - qw + qn - qs + qt - qb - qc);
    }
    vo = vo - 1.0 / (rho * dy[j]) * (A(p, k, j + 1, i) - A(p, k, j, i) + gpy * dy[j]);
    return vo;
}

__device__ double wo_point(int k, int j, int i, int kk, int jj, const double* u, const double* v,
                           const double* w, const double* ut, const double* vt, const double* wt,
                           const double* p, const double* gg, const GridPtrs& s, const Wall& wl,
                           double gmol, double rho, double iles, double gpz) {
    const double *dz = s.dz, *ddx = s.ddx, *ddy = s.ddy, *ddz = s.ddz;
    const double *rdx = s.rdx, *rdy = s.rdy, *rdz = s.rdz, *rddx = s.rddx, *rddy = s.rddy,
                 *rddz = s.rddz;
    double wo;
    {
        double ax = ddy[j] * dz[k], ay = ddx[i] * dz[k], az = ddx[i] * ddy[j];
        double fe = ax * (A(ut, k, j, i) + A(ut, k + 1, j, i)) * 0.5;
        double fw = ax * (A(ut, k, j, i - 1) + A(ut, k + 1, j, i - 1)) * 0.5;
        double fn = ay * (A(vt, k, j, i) + A(vt, k + 1, j, i)) * 0.5;
        double fs = ay * (A(vt, k, j - 1, i) + A(vt, k + 1, j - 1, i)) * 0.5;
        double ft = az * (A(wt, k, j, i) + (A(wt, k + 1, j, i) - A(wt, k, j, i)) * 0.5 * dz[k] / ddz[k + 1]);
        double fb = az * (A(wt, k - 1, j, i) + (A(wt, k, j, i) - A(wt, k - 1, j, i)) * 0.5 * dz[k - 1] / ddz[k]);
        double qe = 0.5 * fe * (A(w, k, j, i) + A(w, k, j, i + 1));
        double qw = 0.5 * fw * (A(w, k, j, i - 1) + A(w, k, j, i));
        double qn = 0.5 * fn * (A(w, k, j, i) + A(w, k, j + 1, i));
        double qs = 0.5 * fs * (A(w, k, j - 1, i) + A(w, k, j, i));
        double qt = 0.5 * ft * (A(w, k, j, i) + A(w, k + 1, j, i));
        double qb = 0.5 * fb * (A(w, k - 1, j, i) + A(w, k, j, i));
        wo = -(qe - qw + qn - qs + qt - qb) * rddx[i] * rddy[j] * rdz[k];
    }
    wo = wall_w(wo, k, j, i, s, wl, A(w, k, j, i));
    {
        double ax = ddy[j] * dz[k], ay = ddx[i] * dz[k], az = ddx[i] * ddy[j];
        double ge = wl.guni ? wl.h2 : hm(A(gg, k, j, i), A(gg, k, j, i + 1), gmol) + hm(A(gg, k + 1, j, i), A(gg, k + 1, j, i + 1), gmol);
        double gw = wl.guni ? wl.h2 : hm(A(gg, k, j, i - 1), A(gg, k, j, i), gmol) + hm(A(gg, k + 1, j, i - 1), A(gg, k + 1, j, i), gmol);
        double gn = wl.guni ? wl.h2 : hm(A(gg, k, j, i), A(gg, k, j + 1, i), gmol) + hm(A(gg, k + 1, j, i), A(gg, k + 1, j + 1, i), gmol);
        double gs = wl.guni ? wl.h2 : hm(A(gg, k, j - 1, i), A(gg, k, j, i), gmol) + hm(A(gg, k + 1, j - 1, i), A(gg, k + 1, j, i), gmol);
        double gt = A(gg, k + 1, j, i);
        double gb = A(gg, k, j, i);
        double qe = -ge * ax * rdx[i] * (A(w, k, j, i + 1) - A(w, k, j, i));
        double qw = -gw * ax * rdx[i - 1] * (A(w, k, j, i) - A(w, k, j, i - 1));
        double qn = -gn * ay * rdy[j] * (A(w, k, j + 1, i) - A(w, k, j, i));
        double qs = -gs * ay * rdy[j - 1] * (A(w, k, j, i) - A(w, k, j - 1, i));
        double qt = -gt * az * rddz[k + 1] * (A(w, k + 1, j, i) - A(w, k, j, i));
        double qb = -gb * az * rddz[k] * (A(w, k, j, i) - A(w, k - 1, j, i));
        double st = ((ge * (A(u, k + 1, j, i) - A(u, k, j, i))) -
                     (gw * (A(u, k + 1, j, i - 1) - A(u, k, j, i - 1)))) * ddy[j] +
                    ((gn * (A(v, k + 1, j, i) - A(v, k, j, i))) -
                     (gs * (A(v, k + 1, j - 1, i) - A(v, k, j - 1, i)))) * ddx[i] +
                    ((gt * (A(w, k + 1, j, i) - A(w, k, j, i)) * rddz[k + 1]) -
                     (gb * (A(w, k, j, i) - A(w, k - 1, j, i)) * rddz[k])) * az;
        double qc = st * iles;
        double fak = 1.0 / rho * rddx[i] * rddy[j] * rdz[k];
        wo = wo - fak * (qe - qw + qn - qs + qt - qb - qc);
    }
    wo = wo - 1.0 / (rho * dz[k]) * (A(p, k + 1, j, i) - A(p, k, j, i) + gpz * dz[k]);
    return wo;
}

// tstle4 over the full box of every grid: points outside the reference's
// loop ranges get 0, as tstle4 zeroes uo, vo, wo before its loops.
__global__ void __launch_bounds__(256) k_tstle4(const DevGrid* __restrict__ grids, Spacing sp,
                                                double* __restrict__ uo, double* __restrict__ vo,
                                                double* __restrict__ wo, const double* __restrict__ U,
                                                const double* __restrict__ V, const double* __restrict__ W,
                                                const double* __restrict__ UT, const double* __restrict__ VT,
                                                const double* __restrict__ WT,
                                                const double* __restrict__ P, const double* __restrict__ Gf,
                                                Wall wl, double iles, double gx, double gy, double gz,
                                                const double* __restrict__ FX, const double* __restrict__ FY,
                                                const double* __restrict__ FZ, const double* __restrict__ GU) {
    const int gi = blockIdx.y;
    const DevGrid G = grids[gi];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int npts = kk * jj * ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npts) return;
    const int k = t % kk + 1;
    const int j = (t / kk) % jj + 1;
    const int i = t / (kk * jj) + 1;
    if (GU) {
        wl.guni = GU[2 * gi] != 0.0;
        wl.h2 = GU[2 * gi + 1];
    }
    GridPtrs s;
    s.kk = kk; s.jj = jj; s.ii = ii;
    s.dx = sp.dx + G.ipx - 1; s.dy = sp.dy + G.ipy - 1; s.dz = sp.dz + G.ipz - 1;
    s.ddx = sp.ddx + G.ipx - 1; s.ddy = sp.ddy + G.ipy - 1; s.ddz = sp.ddz + G.ipz - 1;
    s.rdx = sp.rdx + G.ipx - 1; s.rdy = sp.rdy + G.ipy - 1; s.rdz = sp.rdz + G.ipz - 1;
    s.rddx = sp.rddx + G.ipx - 1; s.rddy = sp.rddy + G.ipy - 1; s.rddz = sp.rddz + G.ipz - 1;
    s.wx = sp.wx + G.ipx - 1; s.wy = sp.wy + G.ipy - 1; s.wz = sp.wz + G.ipz - 1;
    const long long o = G.ip3;
    const double *u = U + o, *v = V + o, *w = W + o, *p = P + o, *g = Gf + o;
    const double *ut = UT + o, *vt = VT + o, *wt = WT + o;
    const int nfro = G.bc[0], nbac = G.bc[1], nrgt = G.bc[2], nlft = G.bc[3], nbot = G.bc[4],
              ntop = G.bc[5];
    const int nbu = (nbac == 7 || nbac == 3) ? 1 : 0;
    const int nlv = (nlft == 7 || nlft == 3) ? 1 : 0;
    const int ntw = (ntop == 7 || ntop == 3) ? 1 : 0;
    const int nfu = nfro == 3 ? 1 : 0, nrv = nrgt == 3 ? 1 : 0, nbw = nbot == 3 ? 1 : 0;
    const double gfl = (double)G.gradpflag;
    const bool jin = j >= 3 && j <= jj - 2, kin = k >= 3 && k <= kk - 2, iin = i >= 3 && i <= ii - 2;
    for (int f = 0; f < 6; ++f) wl.bc[f] = G.bc[f];
    wl.any = nfro == 5 || nbac == 5 || nrgt == 5 || nlft == 5 || nbot == 5 || ntop == 5;
    const double gmol = wl.gmol, rho = wl.rho;
    // outside the flux ranges uo, vo, wo are zero apart from swcle3d's rows
    double ru, rv, rw;
    // the steady body force FX, FY, FZ (when set) follows gradp
    if (i >= 3 - nfu && i <= ii - 3 + nbu && jin && kin) {
        ru = uo_point(k, j, i, kk, jj, u, v, w, ut, vt, wt, p, g, s, wl, gmol, rho, iles, gx * gfl);
        if (FX) ru = ru + FX[o + t];
    } else {
        ru = wall_u(0.0, k, j, i, s, wl, u[t]);
    }
    if (iin && j >= 3 - nrv && j <= jj - 3 + nlv && kin) {
        rv = vo_point(k, j, i, kk, jj, u, v, w, ut, vt, wt, p, g, s, wl, gmol, rho, iles, gy * gfl);
        if (FY) rv = rv + FY[o + t];
    } else {
        rv = wall_v(0.0, k, j, i, s, wl, v[t]);
    }
    if (iin && jin && k >= 3 - nbw && k <= kk - 3 + ntw) {
        rw = wo_point(k, j, i, kk, jj, u, v, w, ut, vt, wt, p, g, s, wl, gmol, rho, iles, gz * gfl);
        if (FZ) rw = rw + FZ[o + t];
    } else {
        rw = wall_w(0.0, k, j, i, s, wl, w[t]);
    }
    uo[o + t] = ru;
    vo[o + t] = rv;
    wo[o + t] = rw;
}

// rkstep: dp = frhs*dp + rhs; p = p + dtfu*dp over the whole flat array.
__global__ void k_rkstep(double* __restrict__ p, double* __restrict__ dp,
                         const double* __restrict__ rhs, double frhs, double dtfu, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; t < n; t += stride) {
        double d = frhs * dp[t] + rhs[t];
        dp[t] = d;
        p[t] = p[t] + dtfu * d;
    }
}

}  // namespace

static Spacing spacing(Ctx* c) {
    Spacing s;
    s.dx = c->L("DX"); s.dy = c->L("DY"); s.dz = c->L("DZ");
    s.ddx = c->L("DDX"); s.ddy = c->L("DDY"); s.ddz = c->L("DDZ");
    s.rdx = c->L("RDX"); s.rdy = c->L("RDY"); s.rdz = c->L("RDZ");
    s.rddx = c->L("RDDX"); s.rddy = c->L("RDDY"); s.rddz = c->L("RDDZ");
    s.wx = c->L("WWX"); s.wy = c->L("WWY"); s.wz = c->L("WWZ");
    return s;
}

// Per grid {1, h2} when G holds one value g0 on the box 2..n-1 in every
// direction (all points of G that tstle4_diff reads), else {0, 0}; h2 is
// hm(g0, g0) + hm(g0, g0) by the same operations, so the shortcut keeps the
// bits.  Without an LES model G is gmol there on grids without walls.
__global__ void k_g_uniform(const DevGrid* __restrict__ grids, const double* __restrict__ Gf, double gmol,
                            double* __restrict__ out) {
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int nk = kk - 2, nj = jj - 2, ni = ii - 2;
    const double* g = Gf + G.ip3;
    const double g0 = A(g, 2, 2, 2);
    int bad = 0;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 2, j = (t / nk) % nj + 2, i = t / (nk * nj) + 2;
        bad |= !(A(g, k, j, i) == g0);
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        const double h = hm(g0, g0, gmol);
        out[2 * blockIdx.x] = bad ? 0.0 : 1.0;
        out[2 * blockIdx.x + 1] = bad ? 0.0 : h + h;
    }
}

// Per grid {1, h2} where G is one value on the box 2..n-1 (see k_g_uniform)
// into the context's d_guni.
int launch_g_uniform(Ctx* c) {
    k_g_uniform<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, c->F("G"), c->prm.gmol, c->d_guni);
    MG_LAUNCHED(c);
    return 0;
}

static int max_points(Ctx* c) {
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    return m;
}

int launch_tstle4(Ctx* c, double* uo, double* vo, double* wo, const double* u, const double* v,
                  const double* w, const double* ut, const double* vt, const double* wt,
                  const double* p, const double* g) {
    ProfScope ps_(c, "tstle4");
    dim3 grid((max_points(c) + 255) / 256, c->ngrid);
    k_g_uniform<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, g, c->prm.gmol, c->d_guni);
    MG_LAUNCHED(c);
    // wernerwengle_mod.F90:13-28 init_wernerwengle
    Wall wl = {};
    const double gmol = c->prm.gmol, rho = c->prm.rho, cwa = 8.3, cwb = 1.0 / 7.0;
    const double cpo1 = 1.0 - cwb, cpo2 = 1.0 + cwb;
    wl.rho = rho;
    wl.gmol = gmol;
    wl.cpo4 = cpo2 / cwa * std::pow(gmol / rho, cwb);
    wl.cpo5 = 0.5 * cpo1 * std::pow(cwa, cpo2 / cpo1) * std::pow(gmol / rho, cpo2);
    wl.cpo6 = 0.5 * gmol / rho * std::pow(cwa, 2.0 / cpo1);
    wl.cpo8 = 2.0 / cpo2;
    k_tstle4<<<grid, 256, 0, c->stream>>>(c->d_grids, spacing(c), uo, vo, wo, u, v, w, ut, vt, wt, p, g,
                                          wl, c->ilesmodel ? 1.0 : 0.0, c->prm.gradp[0], c->prm.gradp[1],
                                          c->prm.gradp[2],
                                          c->bodyforce ? c->F("FBX") : nullptr,
                                          c->bodyforce ? c->F("FBY") : nullptr,
                                          c->bodyforce ? c->F("FBZ") : nullptr, c->d_guni);
    MG_LAUNCHED(c);
    // tstle4_mod.F90:114: tstle4_par after kon, diff and gradp (PAR faces)
    return launch_tstle4_par(c, uo, vo, wo, u, v, w, ut, vt, wt);
}

int launch_rkstep(Ctx* c, double* p, double* dp, const double* rhs, double frhs, double dtfu) {
    ProfScope ps_(c, "rkstep");
    long long n = c->idim3d;
    int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_rkstep<<<blocks, 256, 0, c->stream>>>(p, dp, rhs, frhs, dtfu, n);
    MG_LAUNCHED(c);
    return 0;
}

MG_PLAIN_END
}  // namespace mg
