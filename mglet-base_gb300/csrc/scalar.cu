// scalar.cu -- transport of passive scalars (src/scalar/
// timeintegrate_scalar_mod.F90:17-545, plain FP64 form, no IB): per scalar
// and RK stage the face fluxes of tstsca4 (central convection, diffusion
// with the LES diffusivity and the turbulent Prandtl number of
// scacore_mod.F90:232-262, upwind at PAR faces), the parent's fluxes on PAR
// faces split by open area (bound_scalar_mod.F90:103-123 and twins), the
// flux balance with a constant source, the RK update, the restriction of T
// to the coarser levels and the corner connect.  One thread per point; the
// thread of a point computes its three face fluxes, so the PAR correction
// of a face follows its central flux as in the reference's loop order.
// Built without FMA contraction (bit-exact with the CPU restatement; the
// Kays/Crawford fit takes CUDA's exp).

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "internal.h"

namespace mg {
namespace {

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

struct ScaArgs {
    const DevGrid* grids;
    const double *t, *u, *v, *w, *g, *bt;
    double *qtu, *qtv, *qtw;
    const double *ddx, *ddy, *ddz, *rdx, *rdy, *rdz;
    double gmol, rho, prmol, prturb;
    int kayscrawford, les;
};

__device__ __forceinline__ double prt(const ScaArgs& A, double gtgmol) {
    if (A.kayscrawford == 0) return A.prturb;
    if (gtgmol > 0.0)
        return (double)0.5882f + (double)0.228f * gtgmol -
               (double)0.0441f * (gtgmol * gtgmol) * (1.0 - exp((double)(-5.165f) / gtgmol));
    return A.prmol;
}

__device__ __forceinline__ double gsca(const ScaArgs& A, double g0, double g1) {
    const double gscamol = A.gmol / A.rho / A.prmol;
    if (!A.les) return gscamol;
    const double gtgmolp = (g0 - A.gmol) / A.gmol, gtgmoln = (g1 - A.gmol) / A.gmol;
    const double gs = gscamol + (g1 + g0 - 2.0 * A.gmol) / A.rho / (prt(A, gtgmoln) + prt(A, gtgmolp));
    return gscamol < gs ? gs : gscamol;
}

__global__ void k_tstsca4(ScaArgs A) {
    const DevGrid G = A.grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int tt = blockIdx.x * blockDim.x + threadIdx.x;
    if (tt >= kk * jj * ii) return;
    const int k = tt % kk + 1, j = (tt / kk) % jj + 1, i = tt / (kk * jj) + 1;
    const long long o = G.ip3;
    const double *t = A.t + o, *u = A.u + o, *v = A.v + o, *w = A.w + o, *g = A.g + o, *bt = A.bt + o;
    const double *ddx = A.ddx + G.ipx - 1, *ddy = A.ddy + G.ipy - 1, *ddz = A.ddz + G.ipz - 1;
    const double *rdx = A.rdx + G.ipx - 1, *rdy = A.rdy + G.ipy - 1, *rdz = A.rdz + G.ipz - 1;
    const int nfro = G.bc[0], nbac = G.bc[1], nrgt = G.bc[2], nlft = G.bc[3], nbot = G.bc[4], ntop = G.bc[5];
    const int nfu = nfro == 7, nbu = nbac == 7, nrv = nrgt == 7, nlv = nlft == 7, nbw = nbot == 7, ntw = ntop == 7;
    const bool iin = i >= 3 && i <= ii - 2, jin = j >= 3 && j <= jj - 2, kin = k >= 3 && k <= kk - 2;
    const long long c = IX(k, j, i);
    double qu = 0.0, qv = 0.0, qw = 0.0;
    if (i >= 3 - nfu && i <= ii - 3 + nbu && jin && kin) {
        const double gs = gsca(A, g[c], g[IX(k, j, i + 1)]);
        const double adv = (ddy[j] * ddz[k]) * u[c] * 0.5 * (t[c] + t[IX(k, j, i + 1)]);
        const double area = bt[c] * bt[IX(k, j, i + 1)] * (ddy[j] * ddz[k]);
        const double diff = -gs * rdx[i] * (t[IX(k, j, i + 1)] - t[c]) * area;
        qu = adv + diff;
        if (nfro == 8 && i == 3)
            qu = qu + (ddy[j] * ddz[k]) * (u[c] - fabs(u[c])) * 0.5 * 0.5 * (-t[c] + t[IX(k, j, i + 1)]);
        if (nbac == 8 && i == ii - 3)
            qu = qu + (ddy[j] * ddz[k]) * (u[c] + fabs(u[c])) * 0.5 * 0.5 * (t[c] - t[IX(k, j, i + 1)]);
    }
    if (iin && j >= 3 - nrv && j <= jj - 3 + nlv && kin) {
        const double gs = gsca(A, g[c], g[IX(k, j + 1, i)]);
        const double adv = (ddx[i] * ddz[k]) * v[c] * 0.5 * (t[c] + t[IX(k, j + 1, i)]);
        const double area = bt[c] * bt[IX(k, j + 1, i)] * (ddx[i] * ddz[k]);
        const double diff = -gs * rdy[j] * (t[IX(k, j + 1, i)] - t[c]) * area;
        qv = adv + diff;
        if (nrgt == 8 && j == 3)
            qv = qv + (ddx[i] * ddz[k]) * (v[c] - fabs(v[c])) * 0.5 * 0.5 * (-t[c] + t[IX(k, j + 1, i)]);
        if (nlft == 8 && j == jj - 3)
            qv = qv + (ddx[i] * ddz[k]) * (v[c] + fabs(v[c])) * 0.5 * 0.5 * (t[c] - t[IX(k, j + 1, i)]);
    }
    if (iin && jin && k >= 3 - nbw && k <= kk - 3 + ntw) {
        const double gs = gsca(A, g[c], g[IX(k + 1, j, i)]);
        const double adv = (ddx[i] * ddy[j]) * w[c] * 0.5 * (t[c] + t[IX(k + 1, j, i)]);
        const double area = bt[c] * bt[IX(k + 1, j, i)] * (ddx[i] * ddy[j]);
        const double diff = -gs * rdz[k] * (t[IX(k + 1, j, i)] - t[c]) * area;
        qw = adv + diff;
        if (nbot == 8 && k == 3)
            qw = qw + (ddx[i] * ddy[j]) * (w[c] - fabs(w[c])) * 0.5 * 0.5 * (-t[c] + t[IX(k + 1, j, i)]);
        if (ntop == 8 && k == kk - 3)
            qw = qw + (ddx[i] * ddy[j]) * (w[c] + fabs(w[c])) * 0.5 * 0.5 * (t[c] - t[IX(k + 1, j, i)]);
    }
    A.qtu[o + c] = qu;
    A.qtv[o + c] = qv;
    A.qtw[o + c] = qw;
}

// the PAR flux of face f (1..6) of the grids of ilevel: one thread per 2x2
// block of fine faces
__global__ void k_scaflux_par(const DevGrid* __restrict__ grids, const BFace* __restrict__ bface, int f,
                              int ilevel, double* Q, const double* __restrict__ buf, const double* __restrict__ BT) {
    const DevGrid G = grids[blockIdx.y];
    if (G.level != ilevel || G.bc[f - 1] != MGLET_BC_PAR) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int d = (f - 1) / 2;
    const int na = d == 0 ? jj : ii, nq = d == 2 ? jj : kk;
    const int nba = (na - 4) / 2, nbq = (nq - 4) / 2;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nba * nbq) return;
    const int a = 3 + 2 * (b / nbq), q = 3 + 2 * (b % nbq);
    const int n = d == 0 ? ii : (d == 1 ? jj : kk);
    const int p3 = f % 2 == 1 ? 3 : n - 2, ps = f % 2 == 1 ? 2 : n - 2;
    auto at = [&](int p, int aa, int qq) -> long long {
        if (d == 0) return IX(qq, aa, p);
        if (d == 1) return IX(qq, p, aa);
        return IX(p, qq, aa);
    };
    const double* bt = BT + G.ip3;
    double* qf = Q + G.ip3;
    const double a1 = bt[at(p3, a, q)], a2 = bt[at(p3, a, q + 1)];
    const double a3 = bt[at(p3, a + 1, q)], a4 = bt[at(p3, a + 1, q + 1)];
    const double tot = a1 + a2 + a3 + a4;
    const double qtot = buf[bface[6 * blockIdx.y + f - 1].off + (q - 1) + (long long)(a - 1) * nq];
    qf[at(ps, a, q)] = (tot == 0.0 ? 0.0 : a1 / tot) * qtot;
    qf[at(ps, a, q + 1)] = (tot == 0.0 ? 0.0 : a2 / tot) * qtot;
    qf[at(ps, a + 1, q)] = (tot == 0.0 ? 0.0 : a3 / tot) * qtot;
    qf[at(ps, a + 1, q + 1)] = (tot == 0.0 ? 0.0 : a4 / tot) * qtot;
}

struct WallArgs {
    const DevGrid* grids;
    const BFace* bface;
    const int *kind, *type;      // [ngrid*6], [ngrid*6*9]
    const double *t, *u, *v, *w, *tb;
    double *qtu, *qtv, *qtw;
    const double *dx, *dy, *dz, *ddx, *ddy, *ddz;
    double gmol, rho, prmol;
    // wernerwengle_mod.F90:13-28
    double cwa, cwb, cpo4, cpo5, cpo6, cpo8;
    int f, ilevel, l, les;
};

// wernerwengle_mod.F90:92-122 qwallfix (CUDA's pow)
__device__ double qwallfix(const WallArgs& A, double tbound, double tfluid, double uquer, double dds) {
    const double cpo1 = 1.0 - A.cwb, cpo2 = 1.0 + A.cwb;
    const double uquern = fabs(uquer);
    if (uquern >= A.cpo6 / dds) {
        const double ddsb = pow(dds, -A.cwb);
        const double tauwin = A.rho * pow(ddsb * (A.cpo4 * uquern + A.cpo5 / dds), A.cpo8);
        const double sm = A.gmol / sqrt(tauwin * A.rho) * pow(A.cwa, 1.0 / (1.0 - A.cwb));
        const double fsm = 1.0 / (dds * dds) *
                           (0.5 * (sm * sm) * A.prmol + pow(sqrt(tauwin * A.rho) / A.gmol, -cpo1) * A.cwa / cpo2 *
                                                            (pow(dds, cpo2) - pow(sm, cpo2)));
        return A.gmol / A.rho * (tbound - tfluid) / dds / fsm;
    }
    return A.gmol / A.rho / A.prmol * (tbound - tfluid) * 2.0 / dds;
}

// bound_scalar_mod.F90:124-210 and twins: the SWA / SIO flux of face A.f
// of scalar A.l on the grids of A.ilevel, one thread per plane point
__global__ void k_scaflux_walls(WallArgs A) {
    const DevGrid G = A.grids[blockIdx.y];
    if (G.level != A.ilevel) return;
    const int f = A.f;
    const int kind = A.kind[6 * blockIdx.y + f - 1];
    if (kind == 0) return;
    const int type = A.type[(6 * blockIdx.y + f - 1) * 9 + A.l];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int d = (f - 1) / 2;
    const double dir = f % 2 == 1 ? -1.0 : 1.0;
    const int n = d == 0 ? ii : (d == 1 ? jj : kk);
    const int p2 = f % 2 == 1 ? 2 : n - 2, p3 = f % 2 == 1 ? 3 : n - 2;
    const int na = d == 0 ? jj : ii, nq = d == 2 ? jj : kk;
    const int q0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (q0 >= na * nq) return;
    const int a = q0 / nq + 1, qq = q0 % nq + 1;
    const bool les_wall = kind == 1 && type == 0 && A.les;
    if (les_wall && (a < 2 || qq < 2)) return;
    const long long o = G.ip3;
    const double *dd0 = A.ddx + G.ipx - 1, *dd1 = A.ddy + G.ipy - 1, *dd2 = A.ddz + G.ipz - 1;
    const double* dxs = d == 0 ? A.dx + G.ipx - 1 : (d == 1 ? A.dy + G.ipy - 1 : A.dz + G.ipz - 1);
    const double* A1 = d == 0 ? dd1 : dd0;
    const double* A2 = d == 2 ? dd1 : dd2;
    auto at = [&](int p) -> long long {
        if (d == 0) return IX(qq, a, p);
        if (d == 1) return IX(qq, p, a);
        return IX(p, qq, a);
    };
    const double *t = A.t + o, *u = A.u + o, *v = A.v + o, *w = A.w + o;
    const double tbv = A.tb[A.bface[6 * blockIdx.y + f - 1].off + (qq - 1) + (long long)(a - 1) * nq];
    const double tin = t[at(p3)];
    double r;
    if (type == 1) {
        const double area = A1[a] * A2[qq];
        r = -dir * tbv * area;
    } else if (kind == 1 && !A.les) {
        const double gamma2dx = 2.0 * A.gmol / A.rho / A.prmol / dxs[p2];
        const double diff = gamma2dx * (tbv - tin);
        r = -dir * diff * A1[a] * A2[qq];
    } else if (kind == 1) {
        double s1, s2;
        if (d == 0) {
            const int k = qq, j = a, i = p3;
            s1 = w[IX(k - 1, j, i)] + (w[IX(k, j, i)] - w[IX(k - 1, j, i)]) / dd2[k] * dd2[k - 1] * 0.5;
            s2 = v[IX(k, j - 1, i)] + (v[IX(k, j, i)] - v[IX(k, j - 1, i)]) / dd1[j] * dd1[j - 1] * 0.5;
        } else if (d == 1) {
            const int k = qq, i = a, j = p3;
            s1 = w[IX(k - 1, j, i)] + (w[IX(k, j, i)] - w[IX(k - 1, j, i)]) / dd2[k] * dd2[k - 1] * 0.5;
            s2 = u[IX(k, j, i - 1)] + (u[IX(k, j, i)] - u[IX(k, j, i - 1)]) / dd0[i] * dd0[i - 1] * 0.5;
        } else {
            const int j = qq, i = a, k = p3;
            s1 = u[IX(k, j, i - 1)] + (u[IX(k, j, i)] - u[IX(k, j, i - 1)]) / dd0[i] * dd0[i - 1] * 0.5;
            s2 = v[IX(k, j - 1, i)] + (v[IX(k, j, i)] - v[IX(k, j - 1, i)]) / dd1[j] * dd1[j - 1] * 0.5;
        }
        const double uquer = sqrt(s1 * s1 + s2 * s2);
        const double dds = d == 0 ? dd0[p3] : (d == 1 ? dd1[p3] : dd2[p3]);
        r = -dir * qwallfix(A, tbv, tin, uquer, dds) * (A1[a] * A2[qq]);
    } else {
        const double gamma = A.gmol / A.rho / A.prmol;
        const double* un = d == 0 ? u : (d == 1 ? v : w);
        const double unv = un[at(p2)];
        const double tout = -dir * unv >= 0.0 ? 2.0 * tbv - tin : tin;
        const double adv = -dir * unv * 0.5 * (tout + tin);
        const double diff = gamma * (tout - tin) / dxs[p2];
        r = -dir * (adv + diff) * (A1[a] * A2[qq]);
    }
    double* qf = (d == 0 ? A.qtu : (d == 1 ? A.qtv : A.qtw)) + o;
    qf[at(p2)] = r;
}

// the sources of one scalar in order (at most 8): field null = constant
struct SrcList {
    int n;
    double val[8];
    const double* field[8];
};

// fluxbalance_grid (:520-545) and sourceterm (:549-634: sourceterm_const,
// sourceterm_field, the sources in order) over the box
__global__ void k_fluxbalance(const DevGrid* __restrict__ grids, const double* __restrict__ QTU,
                              const double* __restrict__ QTV, const double* __restrict__ QTW,
                              double* __restrict__ QTT, const double* __restrict__ RDDX,
                              const double* __restrict__ RDDY, const double* __restrict__ RDDZ,
                              SrcList src) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int tt = blockIdx.x * blockDim.x + threadIdx.x;
    if (tt >= kk * jj * ii) return;
    const int k = tt % kk + 1, j = (tt / kk) % jj + 1, i = tt / (kk * jj) + 1;
    const long long o = G.ip3;
    double r = 0.0;
    if (i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2) {
        const double* qtu = QTU + o;
        const double* qtv = QTV + o;
        const double* qtw = QTW + o;
        const double net = qtu[IX(k, j, i - 1)] - qtu[IX(k, j, i)] + qtv[IX(k, j - 1, i)] - qtv[IX(k, j, i)] +
                           qtw[IX(k - 1, j, i)] - qtw[IX(k, j, i)];
        r = RDDZ[G.ipz + k - 1] * RDDY[G.ipy + j - 1] * RDDX[G.ipx + i - 1] * net;
        for (int s = 0; s < src.n; ++s)
            r = src.field[s] ? r + src.val[s] * src.field[s][o + tt] : r + src.val[s];
    }
    QTT[o + tt] = r;
}

// boussinesqterm_grid (boussinesqterm_mod.F90:92-181) and coriolis_grid
// (coriolisterm_mod.F90:100-189) at one point, over tstle4's ranges
__global__ void k_momentum_sources(const DevGrid* __restrict__ grids, double* UO, double* VO, double* WO,
                                   const double* __restrict__ U, const double* __restrict__ V,
                                   const double* __restrict__ W, const double* __restrict__ TOLD, double gx,
                                   double gy, double gz, double beta, int buoy, double o1, double o2, double o3,
                                   int cori) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int tt = blockIdx.x * blockDim.x + threadIdx.x;
    if (tt >= kk * jj * ii) return;
    const int k = tt % kk + 1, j = (tt / kk) % jj + 1, i = tt / (kk * jj) + 1;
    const long long o = G.ip3, c = IX(k, j, i);
    const int nfro = G.bc[0], nbac = G.bc[1], nrgt = G.bc[2], nlft = G.bc[3], nbot = G.bc[4], ntop = G.bc[5];
    const int nbu = (nbac == 7 || nbac == 3), nlv = (nlft == 7 || nlft == 3), ntw = (ntop == 7 || ntop == 3);
    const int nfu = nfro == 3, nrv = nrgt == 3, nbw = nbot == 3;
    const bool iin = i >= 3 && i <= ii - 2, jin = j >= 3 && j <= jj - 2, kin = k >= 3 && k <= kk - 2;
    const double *u = U + o, *v = V + o, *w = W + o, *t = TOLD ? TOLD + o : nullptr;
    if (i >= 3 - nfu && i <= ii - 3 + nbu && jin && kin) {
        double x = UO[o + c];
        if (buoy && fabs(gx) > 0.0) x = x + -gx * beta * (0.5 * (t[c] + t[IX(k, j, i + 1)]));
        if (cori && fabs(o2) + fabs(o3) > 0.0) {
            const double v2 = 0.25 * (v[IX(k, j - 1, i)] + v[IX(k, j - 1, i + 1)] + v[c] + v[IX(k, j, i + 1)]);
            const double v3 = 0.25 * (w[IX(k - 1, j, i)] + w[IX(k - 1, j, i + 1)] + w[c] + w[IX(k, j, i + 1)]);
            x = x + -2.0 * (o2 * v3 - o3 * v2);
        }
        UO[o + c] = x;
    }
    if (iin && j >= 3 - nrv && j <= jj - 3 + nlv && kin) {
        double x = VO[o + c];
        if (buoy && fabs(gy) > 0.0) x = x + -gy * beta * (0.5 * (t[c] + t[IX(k, j + 1, i)]));
        if (cori && fabs(o1) + fabs(o3) > 0.0) {
            const double v1 = 0.25 * (u[IX(k, j, i - 1)] + u[IX(k, j + 1, i - 1)] + u[c] + u[IX(k, j + 1, i)]);
            const double v3 = 0.25 * (w[IX(k - 1, j, i)] + w[IX(k - 1, j + 1, i)] + w[c] + w[IX(k, j + 1, i)]);
            x = x + -2.0 * (o3 * v1 - o1 * v3);
        }
        VO[o + c] = x;
    }
    if (iin && jin && k >= 3 - nbw && k <= kk - 3 + ntw) {
        double x = WO[o + c];
        if (buoy && fabs(gz) > 0.0) x = x + -gz * beta * (0.5 * (t[c] + t[IX(k + 1, j, i)]));
        if (cori && fabs(o1) + fabs(o2) > 0.0) {
            const double v1 = 0.25 * (u[IX(k, j, i - 1)] + u[IX(k + 1, j, i - 1)] + u[c] + u[IX(k + 1, j, i)]);
            const double v2 = 0.25 * (v[IX(k, j - 1, i)] + v[IX(k + 1, j - 1, i)] + v[c] + v[IX(k + 1, j, i)]);
            x = x + -2.0 * (o1 * v2 - o2 * v1);
        }
        WO[o + c] = x;
    }
}

// ---- ghost-cell IB of the scalars -------------------------------------------
// blockbt (blockbt_mod.F90:11-208), maskbt (scacore_mod.F90:265-306) and
// set_scastencils (gc_scastencils_mod.F90:949-1125).
constexpr int kScaIsize = 9, kScaRsize = 8, kScaNperi = 6, kScaMaxBody = 16;

__device__ __forceinline__ double mxd(double a, double b) { return a < b ? b : a; }

// blockbt_grid (:73-91): bt = the largest bp of the cell and its six face
// neighbours, on 2..n-1
__global__ void k_blockbt(const DevGrid* __restrict__ grids, const double* __restrict__ BP, double* BT) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)kk * jj * ii) return;
    const int k = (int)(q % kk) + 1, j = (int)((q / kk) % jj) + 1, i = (int)(q / ((long long)kk * jj)) + 1;
    if (i < 2 || i > ii - 1 || j < 2 || j > jj - 1 || k < 2 || k > kk - 1) return;
    const double* bp = BP + G.ip3;
    BT[G.ip3 + IX(k, j, i)] = mxd(mxd(mxd(mxd(mxd(mxd(bp[IX(k, j, i)], bp[IX(k, j, i + 1)]), bp[IX(k, j, i - 1)]),
                                                 bp[IX(k, j + 1, i)]),
                                             bp[IX(k, j - 1, i)]),
                                         bp[IX(k + 1, j, i)]),
                                     bp[IX(k - 1, j, i)]);
}

// open_scalarflux_boundary (:93-208): one CTA per grid of the level, its PAR
// faces in order; the receiver layer opens where the coarse cell lets a
// scalar flux through (hilf from ctof of BT, -1 where ctof wrote nothing)
__global__ void k_open_scaflux(const DevGrid* __restrict__ grids, const int* __restrict__ list,
                               const double* __restrict__ HILF, double* BT, int* err) {
    const DevGrid G = grids[list[blockIdx.x]];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const double* hf = HILF + G.ip3;
    double* bt = BT + G.ip3;
    for (int f = 1; f <= 6; ++f) {
        if (G.bc[f - 1] != MGLET_BC_PAR) continue;
        const int ax = (f - 1) / 2, hi = (f - 1) % 2;
        const int n = ax == 0 ? ii : (ax == 1 ? jj : kk);
        const int p2 = hi ? n - 1 : 2, p3 = hi ? n - 2 : 3;
        const int na = ax == 0 ? jj : ii, nb = ax == 2 ? jj : kk;
        for (int t = threadIdx.x; t < (na - 2) * (nb - 2); t += blockDim.x) {
            const int a = 2 + t / (nb - 2), b = 2 + t % (nb - 2);
            int k2, j2, i2, k3, j3, i3;
            if (ax == 0) { i2 = p2; i3 = p3; j2 = j3 = a; k2 = k3 = b; }
            else if (ax == 1) { j2 = p2; j3 = p3; i2 = i3 = a; k2 = k3 = b; }
            else { k2 = p2; k3 = p3; i2 = i3 = a; j2 = j3 = b; }
            const double c2 = hf[IX(k2, j2, i2)], c3 = hf[IX(k3, j3, i3)];
            if (c2 < -0.5 || c3 < -0.5) {
                atomicExch(err, 1);
                continue;
            }
            bt[IX(k3, j3, i3)] = mxd(c2 * c3, bt[IX(k3, j3, i3)]);
        }
        __syncthreads();
    }
}

// maskbt_grid (scacore_mod.F90:289-306): t *= bt on 3..n-2
__global__ void k_maskbt(const DevGrid* __restrict__ grids, double* T, const double* __restrict__ BT) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)kk * jj * ii) return;
    const int k = (int)(q % kk) + 1, j = (int)((q / kk) % jj) + 1, i = (int)(q / ((long long)kk * jj)) + 1;
    if (i < 3 || i > ii - 2 || j < 3 || j > jj - 2 || k < 3 || k > kk - 2) return;
    T[G.ip3 + q] = T[G.ip3 + q] * BT[G.ip3 + q];
}

// the conditions of the bodies for one scalar (sca%geometries)
struct ScaGeo {
    int n;
    int flag[kScaMaxBody];
    double value[kScaMaxBody];
};

// set_scastencils (:1005-1125): one thread per grid walks its cells in list
// order (a value set for one cell may feed a later cell's stencil).  tmode:
// a fixed-value body sets var(intcell) from its stencil cells and acoeffvel
// * value; else a fixed-flux body (or no body) adds areabyvol * value.
__global__ void k_scastencils(const DevGrid* __restrict__ grids, int ngrid, const long long* __restrict__ xi,
                              const double* __restrict__ xr, const long long* __restrict__ cell0, ScaGeo geo,
                              double* var, int tmode) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngrid) return;
    double* v = var + grids[g].ip3;
    for (long long cell = cell0[g]; cell < cell0[g + 1]; ++cell) {
        const long long* I = xi + cell * kScaIsize;
        const double* r = xr + cell * kScaRsize;
        const long long intcell = I[0], body = I[1];
        int bctype = 1;
        double bcval = 0.0;
        if (body > 0) {
            bctype = geo.flag[body - 1];
            bcval = geo.value[body - 1];
        }
        if (tmode) {
            double val = 0.0;
            for (long long n = 1; n <= I[2]; ++n) val = val + v[I[2 + n] - 1] * r[n];
            const double coeff = r[1 + kScaNperi];
            if (bctype == 0) {
                val = val + coeff * bcval;
                v[intcell - 1] = val;
            }
        } else if (bctype == 1) {
            v[intcell - 1] = v[intcell - 1] + r[0] * bcval;
        }
    }
}

#undef IX

}  // namespace

int launch_momentum_sources(Ctx* c) {
    if (!c->buoyancy && !c->coriolis) return 0;
    ProfScope ps_(c, "momentum_sources");
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    const double* told = nullptr;
    if (c->buoyancy) told = c->F(("T" + std::to_string(c->buoyancy_scalar) + "_OLD").c_str());
    k_momentum_sources<<<dim3((m + 255) / 256, c->ngrid), 256, 0, c->stream>>>(
        c->d_grids, c->F("UO"), c->F("VO"), c->F("WO"), c->F("U"), c->F("V"), c->F("W"), told, c->gravity[0],
        c->gravity[1], c->gravity[2], c->beta, c->buoyancy ? 1 : 0, c->omega[0], c->omega[1], c->omega[2],
        c->coriolis ? 1 : 0);
    MG_LAUNCHED(c);
    return 0;
}

int set_scalars(Ctx* c, int nsca, const double* prmol, const int32_t* kayscrawford, const double* source,
                double prturb) {
    if (nsca < 0 || nsca > 9 || (nsca && (!prmol || !kayscrawford))) {
        set_error("set_scalars: 0..9 scalars with prmol and kayscrawford");
        return MGLET_ERR_ARG;
    }
    if (nsca && c->prm.form != MGLET_FORM_PLAIN) {
        set_error("set_scalars: the plain form");
        return MGLET_ERR_UNSUPPORTED;
    }
    c->sca.clear();
    for (int l = 0; l < nsca; ++l) {
        Ctx::ScalarDef sd;
        sd.name = "T" + std::to_string(l + 1);
        sd.prmol = prmol[l];
        sd.kayscrawford = kayscrawford[l];
        if (source && source[l] != 0.0) sd.sources.push_back({"", source[l]});
        for (const std::string& n : {sd.name, "D" + sd.name, sd.name + "_OLD"}) {
            if (!c->f3.count(n))
                if (int rc = alloc_field3(c, n.c_str())) return rc;
            MG_CUDA(cudaMemsetAsync(c->F(n.c_str()), 0, (size_t)c->idim3d * sizeof(double), c->stream));
        }
        c->sca.push_back(sd);
    }
    c->prturb = prturb;
    for (const char* n : {"QTU", "QTV", "QTW", "QTT", "BT"})
        if (!c->f3.count(n))
            if (int rc = alloc_field3(c, n)) return rc;
    // blockbt: every cell open without the ghost-cell IB
    if (int rc = fill_field(c, c->F("BT"), 1.0)) return rc;
    return c->ibtype == 1 ? scalar_blockbt(c) : 0;
}

// blockbt (blockbt_mod.F90:11-70) with the ghost-cell IB: BT from BP,
// connected per level, then per level the cells behind PAR faces opened
// from ctof of BT into a scratch field preset to -1
int scalar_blockbt(Ctx* c) {
    if (!c->f3.count("BT")) return 0;
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    double* BT = c->F("BT");
    k_blockbt<<<dim3((m + 255) / 256, c->ngrid), 256, 0, c->stream>>>(c->d_grids, c->F("BP"), BT);
    MG_LAUNCHED(c);
    for (int l = c->minlevel; l <= c->maxlevel; ++l)
        if (int rc = connect(c, l, 2, nullptr, nullptr, nullptr, BT, nullptr, nullptr, true, false, 0)) return rc;
    if (!c->f3.count("BTH"))
        if (int rc = alloc_field3(c, "BTH")) return rc;
    int* d_err = nullptr;
    MG_CUDA(cudaMalloc(&d_err, sizeof(int)));
    MG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), c->stream));
    int rc = 0;
    for (int l = c->minlevel; l <= c->maxlevel && !rc; ++l) {
        if ((rc = fill_field(c, c->F("BTH"), -1.0))) break;
        if (c->minlevel != c->maxlevel) {
            if ((rc = launch_ctof(c, l, c->F("BTH"), BT))) break;
            auto it = c->d_children.find(l);
            if (l != c->minlevel && it != c->d_children.end()) {
                k_open_scaflux<<<(unsigned)c->children[l].size(), 128, 0, c->stream>>>(
                    c->d_grids, it->second, c->F("BTH"), BT, d_err);
                if (cudaGetLastError() != cudaSuccess) rc = MGLET_ERR_CUDA;
                c->launches++;
            }
        }
        if (!rc) rc = connect(c, l, 2, nullptr, nullptr, nullptr, BT, nullptr, nullptr, true, false, 0);
    }
    int herr = 0;
    cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(d_err);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "blockbt");
    if (herr) {
        set_error("blockbt: a fine cell behind a PAR face has no coarse value");
        return MGLET_ERR_ARG;
    }
    return 0;
}

// The scalar ghost-cell list of grid igrid (1-based), kept on the host and
// uploaded with every grid's list back to back.
int set_scastencils(Ctx* c, int igrid, int ncells, const int64_t* xpoli, const double* xpolr,
                    const double* xpolrvel) {
    if (igrid < 1 || igrid > c->ngrid || ncells < 0 || (ncells && (!xpoli || !xpolr || !xpolrvel))) {
        set_error("set_scastencils: bad grid or lists");
        return MGLET_ERR_ARG;
    }
    const DevGrid& G = c->grids[igrid - 1];
    const int64_t npts = (int64_t)G.kk * G.jj * G.ii;
    for (int cell = 0; cell < ncells; ++cell) {
        const int64_t* xi = xpoli + (size_t)cell * kScaIsize;
        bool bad = xi[0] < 1 || xi[0] > npts || xi[2] < 0 || xi[2] > kScaNperi || xi[1] > kScaMaxBody;
        for (int64_t n = 1; n <= xi[2] && !bad; ++n) bad = xi[2 + n] < 1 || xi[2 + n] > npts;
        if (bad) {
            set_error("set_scastencils: cell, body or stencil out of range");
            return MGLET_ERR_ARG;
        }
    }
    if ((int)c->scal.size() < c->ngrid) c->scal.resize(c->ngrid);
    Ctx::ScaList& L = c->scal[igrid - 1];
    L.ncells = ncells;
    L.xpoli.assign(xpoli, xpoli + (size_t)ncells * kScaIsize);
    L.xpolr.assign(xpolr, xpolr + (size_t)ncells * kScaRsize);
    L.xpolrvel.assign(xpolrvel, xpolrvel + (size_t)ncells * kScaRsize);
    std::vector<long long> xi, cell0(c->ngrid + 1, 0);
    std::vector<double> xr, xv;
    c->scal_maxbody = 0;
    for (int g = 0; g < c->ngrid; ++g) {
        const Ctx::ScaList& S = c->scal[g];
        cell0[g + 1] = cell0[g] + S.ncells;
        xi.insert(xi.end(), S.xpoli.begin(), S.xpoli.end());
        xr.insert(xr.end(), S.xpolr.begin(), S.xpolr.end());
        xv.insert(xv.end(), S.xpolrvel.begin(), S.xpolrvel.end());
        for (int cell = 0; cell < S.ncells; ++cell)
            c->scal_maxbody = std::max(c->scal_maxbody, (int)S.xpoli[(size_t)cell * kScaIsize + 1]);
    }
    for (void* p : {(void*)c->d_sxi, (void*)c->d_sxr, (void*)c->d_sxrv, (void*)c->d_scell0}) cudaFree(p);
    c->d_sxi = nullptr; c->d_sxr = nullptr; c->d_sxrv = nullptr; c->d_scell0 = nullptr;
    auto up = [&](void** d, const void* h, size_t n) -> int {
        MG_CUDA(cudaMalloc(d, std::max<size_t>(n, 8)));
        if (n) MG_CUDA(copy_on(c->stream, *d, h, n, cudaMemcpyHostToDevice));
        return 0;
    };
    if (int rc = up((void**)&c->d_sxi, xi.data(), xi.size() * sizeof(long long))) return rc;
    if (int rc = up((void**)&c->d_sxr, xr.data(), xr.size() * sizeof(double))) return rc;
    if (int rc = up((void**)&c->d_sxrv, xv.data(), xv.size() * sizeof(double))) return rc;
    return up((void**)&c->d_scell0, cell0.data(), cell0.size() * sizeof(long long));
}

int set_scalar_geometry(Ctx* c, int isca, int nbody, const int32_t* flag, const double* value) {
    if (isca < 1 || isca > (int)c->sca.size() || nbody < 0 || nbody > kScaMaxBody ||
        (nbody && (!flag || !value))) {
        set_error("set_scalar_geometry: bad scalar or bodies (at most 16)");
        return MGLET_ERR_ARG;
    }
    for (int b = 0; b < nbody; ++b)
        if (flag[b] != 0 && flag[b] != 1) {
            set_error("set_scalar_geometry: flag 0 (fixed value) or 1 (fixed flux)");
            return MGLET_ERR_ARG;
        }
    c->sca[isca - 1].geo_flag.assign(flag, flag + nbody);
    c->sca[isca - 1].geo_value.assign(value, value + nbody);
    return 0;
}

// set_scastencils("P", sca, t= or qtt=) on every grid
static int launch_scastencils(Ctx* c, const Ctx::ScalarDef& sd, double* var, bool tmode) {
    if (!c->d_scell0) return 0;
    if (c->scal_maxbody > (int)sd.geo_flag.size()) {
        set_error("timeintegrate_scalar: a body of the lists has no condition for " + sd.name);
        return MGLET_ERR_ARG;
    }
    ScaGeo geo{};
    geo.n = (int)sd.geo_flag.size();
    for (int b = 0; b < geo.n; ++b) {
        geo.flag[b] = sd.geo_flag[b];
        geo.value[b] = sd.geo_value[b];
    }
    k_scastencils<<<(c->ngrid + 63) / 64, 64, 0, c->stream>>>(c->d_grids, c->ngrid, c->d_sxi, c->d_sxrv,
                                                             c->d_scell0, geo, var, tmode ? 1 : 0);
    MG_LAUNCHED(c);
    return 0;
}

int add_scalar_source(Ctx* c, int isca, const char* field, double value) {
    if (isca < 1 || isca > (int)c->sca.size()) {
        set_error("add_scalar_source: no such scalar");
        return MGLET_ERR_ARG;
    }
    const std::string f = field ? field : "";
    if (!f.empty() && !c->f3.count(f)) {
        set_error("add_scalar_source: unknown field");
        return MGLET_ERR_NAME;
    }
    if (c->sca[isca - 1].sources.size() >= 8) {
        set_error("add_scalar_source: at most 8 sources");
        return MGLET_ERR_ARG;
    }
    c->sca[isca - 1].sources.push_back({f, value});
    return 0;
}

int set_scalar_bc(Ctx* c, int igrid, int iface, int kind, const int32_t* types) {
    if (igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6 || kind < 0 || kind > 2 || (kind && !types)) {
        set_error("set_scalar_bc: bad arguments");
        return MGLET_ERR_ARG;
    }
    const int t = c->grids[igrid - 1].bc[iface - 1];
    if (kind && (t == MGLET_BC_CON || t == MGLET_BC_CO1 || t == MGLET_BC_PAR)) {
        set_error("set_scalar_bc: SWA and SIO sit on boundary faces");
        return MGLET_ERR_ARG;
    }
    if (c->scabc_kind.empty()) {
        c->scabc_kind.assign(6 * (size_t)c->ngrid, 0);
        c->scabc_type.assign(6 * (size_t)c->ngrid * 9, 0);
        MG_CUDA(cudaMalloc(&c->d_scabc_kind, c->scabc_kind.size() * sizeof(int)));
        MG_CUDA(cudaMalloc(&c->d_scabc_type, c->scabc_type.size() * sizeof(int)));
    }
    const size_t x = 6 * (size_t)(igrid - 1) + iface - 1;
    c->scabc_kind[x] = kind;
    for (size_t l = 0; l < c->sca.size() && kind; ++l) {
        if (types[l] != 0 && types[l] != 1) {
            set_error("set_scalar_bc: type 0 (value) or 1 (flux)");
            return MGLET_ERR_ARG;
        }
        c->scabc_type[x * 9 + l] = types[l];
    }
    MG_CUDA(copy_on(c->stream, c->d_scabc_kind, c->scabc_kind.data(), c->scabc_kind.size() * sizeof(int),
                    cudaMemcpyHostToDevice));
    MG_CUDA(copy_on(c->stream, c->d_scabc_type, c->scabc_type.data(), c->scabc_type.size() * sizeof(int),
                    cudaMemcpyHostToDevice));
    return 0;
}

int timeintegrate_scalar(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk) {
    double frhs, fu, dtrk, dtrki;
    if (int rc = rk_coeffs(rk, irk, &frhs, &fu, &dtrk, &dtrki)) return rc;
    ProfScope ps_(c, "scalar");
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    const dim3 bg((m + 255) / 256, c->ngrid);
    int mb = 0;
    for (const DevGrid& g : c->grids)
        mb = std::max(mb, std::max((g.jj - 4) * (g.kk - 4), std::max((g.ii - 4) * (g.kk - 4), (g.ii - 4) * (g.jj - 4))) / 4);
    static const char* const qn[3] = {"QTU", "QTV", "QTW"};
    static const char* const none[3] = {nullptr, nullptr, nullptr};
    for (const Ctx::ScalarDef& sd : c->sca) {
        double* T = c->F(sd.name.c_str());
        double* DT = c->F(("D" + sd.name).c_str());
        // T_OLD = T (timeintegrate_scalar_mod.F90:56-57), read by the Boussinesq term
        MG_CUDA(cudaMemcpyAsync(c->F((sd.name + "_OLD").c_str()), T, (size_t)c->idim3d * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
        ScaArgs A{};
        A.grids = c->d_grids;
        A.t = T; A.u = c->F("U"); A.v = c->F("V"); A.w = c->F("W"); A.g = c->F("G"); A.bt = c->F("BT");
        A.qtu = c->F("QTU"); A.qtv = c->F("QTV"); A.qtw = c->F("QTW");
        A.ddx = c->L("DDX"); A.ddy = c->L("DDY"); A.ddz = c->L("DDZ");
        A.rdx = c->L("RDX"); A.rdy = c->L("RDY"); A.rdz = c->L("RDZ");
        A.gmol = c->prm.gmol; A.rho = c->prm.rho; A.prmol = sd.prmol; A.prturb = c->prturb;
        A.kayscrawford = sd.kayscrawford; A.les = c->ilesmodel != 0;
        k_tstsca4<<<bg, 256, 0, c->stream>>>(A);
        MG_LAUNCHED(c);
        if (!c->scabc_kind.empty()) {
            // SWA / SIO faces (bound_scalar_mod.F90:124-210), faces in order
            WallArgs W{};
            W.grids = c->d_grids; W.bface = c->d_bface; W.kind = c->d_scabc_kind; W.type = c->d_scabc_type;
            W.t = T; W.u = c->F("U"); W.v = c->F("V"); W.w = c->F("W");
            W.tb = field_buffer(c, sd.name);
            if (!W.tb) {
                set_error("timeintegrate_scalar: buffer allocation");
                return MGLET_ERR_CUDA;
            }
            W.qtu = c->F("QTU"); W.qtv = c->F("QTV"); W.qtw = c->F("QTW");
            W.dx = c->L("DX"); W.dy = c->L("DY"); W.dz = c->L("DZ");
            W.ddx = c->L("DDX"); W.ddy = c->L("DDY"); W.ddz = c->L("DDZ");
            W.gmol = c->prm.gmol; W.rho = c->prm.rho; W.prmol = sd.prmol;
            W.cwa = 8.3; W.cwb = 1.0 / 7.0;
            const double cpo1 = 1.0 - W.cwb, cpo2 = 1.0 + W.cwb;
            W.cpo4 = cpo2 / W.cwa * std::pow(W.gmol / W.rho, W.cwb);
            W.cpo5 = 0.5 * cpo1 * std::pow(W.cwa, cpo2 / cpo1) * std::pow(W.gmol / W.rho, cpo2);
            W.cpo6 = 0.5 * W.gmol / W.rho * std::pow(W.cwa, 2.0 / cpo1);
            W.cpo8 = 2.0 / cpo2;
            W.l = (int)(&sd - c->sca.data());
            W.les = c->ilesmodel != 0;
            int mp = 0;
            for (const DevGrid& g : c->grids) mp = std::max(mp, std::max(g.jj * g.kk, std::max(g.ii * g.kk, g.ii * g.jj)));
            for (int l = c->minlevel; l <= c->maxlevel; ++l)
                for (int f = 1; f <= 6; ++f) {
                    W.f = f;
                    W.ilevel = l;
                    k_scaflux_walls<<<dim3((mp + 127) / 128, c->ngrid), 128, 0, c->stream>>>(W);
                    MG_LAUNCHED(c);
                }
        }
        for (int l = c->minlevel; l <= c->maxlevel; ++l) {
            if (c->minlevel == c->maxlevel) break;
            if (int rc = launch_parent(c, l, qn, none, false)) return rc;
            for (int f = 1; f <= 6; ++f) {
                double* Q = c->F(qn[(f - 1) / 2]);
                const double* buf = field_buffer(c, qn[(f - 1) / 2]);
                if (!buf) {
                    set_error("timeintegrate_scalar: buffer allocation");
                    return MGLET_ERR_CUDA;
                }
                k_scaflux_par<<<dim3((mb + 127) / 128, c->ngrid), 128, 0, c->stream>>>(
                    c->d_grids, c->d_bface, f, l, Q, buf, c->F("BT"));
                MG_LAUNCHED(c);
            }
        }
        SrcList src = {};
        src.n = (int)sd.sources.size();
        for (int s = 0; s < src.n; ++s) {
            src.val[s] = sd.sources[s].second;
            src.field[s] = sd.sources[s].first.empty() ? nullptr : c->F(sd.sources[s].first.c_str());
        }
        k_fluxbalance<<<bg, 256, 0, c->stream>>>(c->d_grids, c->F("QTU"), c->F("QTV"), c->F("QTW"), c->F("QTT"),
                                                 c->L("RDDX"), c->L("RDDY"), c->L("RDDZ"), src);
        MG_LAUNCHED(c);
        const bool gc = c->ibtype == 1;
        // timeintegrate_scalar_mod.F90:71-73: the flux condition of the bodies
        if (gc)
            if (int rc = launch_scastencils(c, sd, c->F("QTT"), false)) return rc;
        if (int rc = launch_rkstep(c, T, DT, c->F("QTT"), frhs, dt * fu)) return rc;
        if (gc) {
            // :84 maskbt (a no-op with BT = 1 without the IB), :87-90 the value
            // condition of the bodies after the connect
            k_maskbt<<<bg, 256, 0, c->stream>>>(c->d_grids, T, c->F("BT"));
            MG_LAUNCHED(c);
            if (int rc = connect(c, 0, 2, nullptr, nullptr, nullptr, T, nullptr, nullptr, true, false, 0))
                return rc;
            if (int rc = launch_scastencils(c, sd, T, true)) return rc;
        }
        for (int l = c->maxlevel; l > c->minlevel; --l)
            if (int rc = launch_ftoc(c, l, T, T, 'T')) return rc;
        if (int rc = connect(c, 0, 2, nullptr, nullptr, nullptr, T, nullptr, nullptr, true, false, 0)) return rc;
    }
    return 0;
}

}  // namespace mg
