// adjoint.cu -- the discrete adjoint of the plain FP64 Runge-Kutta stage.
//
// The reference has no adjoint; this is new functionality built on the
// stage of timeintegration_mod.F90:22-142 as this library runs it (noib, one
// level, every face CON): tstle4 (kon, diff, gradp and the steady body force)
// -> rkstep -> connect(1 layer, normal, forward=1) -> mgpoisl (divcal, the
// SIP outer loop, mgpcorr, connect(2 layers, corners)).  Every operator but
// kon is linear; kon is bilinear in the transporting and the transported
// velocity and is linearised about the stored stage input.  The adjoint of
// each operator is written out as its transpose:
//
//   connect           dst <- src copies  -> lambda(src) += lambda(dst), lambda(dst) = 0,
//                     the copies grouped by the grid they read, one CTA per
//                     group walking its copies in order
//   mgpcorr           gather of lambda(dp) from the velocity faces and p
//   pressure solve    dp = L^-1 rhs with the symmetric periodic Laplacian of
//                     uniform grids: lambda(rhs) = L^-1 lambda(dp), solved by
//                     the same SIP outer loop, after the mean of lambda(dp) is
//                     taken out (the constant null space)
//   divcal            gather of lambda(u) from the two cells of each face
//   rkstep            dU = frhs dU + UO, U = U + dtfu dU
//   tstle4            per output point, the derivatives of its flux formula
//                     added into lambda(u, v, w, p) of its 3x3x3 neighbourhood;
//                     the points run in 27 colour classes (i, j, k mod 3), so
//                     no two points of a launch touch the same value and the
//                     sums are formed in a fixed order; the body force takes
//                     lambda(uo) directly
//
// No atomics anywhere: the gradient is the same bits on every run.
//
// The objective is the kinetic energy of enerfg (timeintegration_mod.F90:
// 417-452): sum vol 0.5 (up^2 + vp^2 + wp^2) / sum vol over the interior.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace mg {
namespace {

int fail(int code, const std::string& msg) {
    set_error(msg);
    return code;
}

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

struct AdjSlots {
    double* f[6];
};

// transpose of k_connect: the ghost's adjoint goes to its source.  One CTA
// per group of copies that read the same grid, the copies of a group in
// their order: within one copy every source point is distinct, and the
// groups add into disjoint grids.
__global__ void k_adj_connect(const BoxCopy* __restrict__ tasks, const int* __restrict__ start,
                              AdjSlots fs) {
    for (int ti = start[blockIdx.x]; ti < start[blockIdx.x + 1]; ++ti) {
        const BoxCopy t = tasks[ti];
        double* a = fs.f[t.slot];
        if (a) {
            const int nkj = t.nk * t.nj;
            for (int q = threadIdx.x; q < t.npts; q += blockDim.x) {
                const int k = q % t.nk, j = (q / t.nk) % t.nj, i = q / nkj;
                const long long d = t.dst + (long long)i * t.djj + (long long)j * t.dkk + k;
                const long long s = t.src + (long long)i * t.sjj + (long long)j * t.skk + k;
                const double v = a[d];
                a[d] = 0.0;
                a[s] += v;
            }
        }
        __syncthreads();
    }
}

// transpose of k_mgpcorr (noib form): lambda(dp) over the whole box
__global__ void k_adj_mgpcorr(const DevGrid* __restrict__ grids, const double* __restrict__ LU,
                              const double* __restrict__ LV, const double* __restrict__ LW,
                              const double* __restrict__ LP, double* __restrict__ LDP,
                              const double* __restrict__ RDX, const double* __restrict__ RDY,
                              const double* __restrict__ RDZ, double rfak) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    const long long o = G.ip3, c = IX(k, j, i);
    const double *rdx = RDX + G.ipx - 1, *rdy = RDY + G.ipy - 1, *rdz = RDZ + G.ipz - 1;
    double s = 0.0;
    if (i >= 2 && i <= ii - 1 && j >= 2 && j <= jj - 1 && k >= 2 && k <= kk - 1) s += LP[o + c];
    if (j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2) {
        if (i >= 2 && i <= ii - 2) s += LU[o + c] * rdx[i] * rfak;
        if (i - 1 >= 2 && i - 1 <= ii - 2) s -= LU[o + IX(k, j, i - 1)] * rdx[i - 1] * rfak;
    }
    if (i >= 3 && i <= ii - 2 && k >= 3 && k <= kk - 2) {
        if (j >= 2 && j <= jj - 2) s += LV[o + c] * rdy[j] * rfak;
        if (j - 1 >= 2 && j - 1 <= jj - 2) s -= LV[o + IX(k, j - 1, i)] * rdy[j - 1] * rfak;
    }
    if (i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2) {
        if (k >= 2 && k <= kk - 2) s += LW[o + c] * rdz[k] * rfak;
        if (k - 1 >= 2 && k - 1 <= kk - 2) s -= LW[o + IX(k - 1, j, i)] * rdz[k - 1] * rfak;
    }
    LDP[o + c] = s;
}

// per-grid sum of the interior of a field (one block per grid)
__global__ void k_interior_sum(const DevGrid* __restrict__ grids, const double* __restrict__ F,
                               double* __restrict__ out) {
    __shared__ double sh[32];
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    double s = 0.0;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        s += F[G.ip3 + IX(k, j, i)];
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) s += sh[q];
        out[blockIdx.x] = s;
    }
}

// RHS = the interior of B minus mean, 0 on the ghost layers
__global__ void k_centre_rhs(const DevGrid* __restrict__ grids, const double* __restrict__ B,
                             double* __restrict__ RHS, double mean) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    const bool in = i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2;
    RHS[G.ip3 + t] = in ? B[G.ip3 + t] - mean : 0.0;
}

// transpose of k_divcal (noib): lambda(u) += fak D^T Y, Y on the interior cells
__global__ void k_adj_divcal(const DevGrid* __restrict__ grids, double* __restrict__ LU,
                             double* __restrict__ LV, double* __restrict__ LW,
                             const double* __restrict__ Y, const double* __restrict__ RDDX,
                             const double* __restrict__ RDDY, const double* __restrict__ RDDZ,
                             double fak) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    const long long o = G.ip3;
    const double *rddx = RDDX + G.ipx - 1, *rddy = RDDY + G.ipy - 1, *rddz = RDDZ + G.ipz - 1;
    auto in = [&](int kx, int jx, int ix) {
        return ix >= 3 && ix <= ii - 2 && jx >= 3 && jx <= jj - 2 && kx >= 3 && kx <= kk - 2;
    };
    double su = 0.0, sv = 0.0, sw = 0.0;
    if (in(k, j, i)) {
        const double y = Y[o + IX(k, j, i)];
        su += y * rddx[i];
        sv += y * rddy[j];
        sw += y * rddz[k];
    }
    if (in(k, j, i + 1)) su -= Y[o + IX(k, j, i + 1)] * rddx[i + 1];
    if (in(k, j + 1, i)) sv -= Y[o + IX(k, j + 1, i)] * rddy[j + 1];
    if (in(k + 1, j, i)) sw -= Y[o + IX(k + 1, j, i)] * rddz[k + 1];
    LU[o + t] += fak * su;
    LV[o + t] += fak * sv;
    LW[o + t] += fak * sw;
}

// transpose of rkstep: dU' = frhs dU + UO, U' = U + dtfu dU'
__global__ void k_adj_rkstep(const double* __restrict__ LU, double* __restrict__ LDU,
                             double* __restrict__ LUO, double frhs, double dtfu, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const double s = LDU[t] + dtfu * LU[t];
        LUO[t] = s;
        LDU[t] = frhs * s;
    }
}

__device__ __forceinline__ double hmean(double a, double b, double gmol) {
    return a * b / (a + b < gmol ? gmol : a + b);
}

struct AdjGrid {
    int kk, jj, ii;
    const double *dx, *dy, *dz, *ddx, *ddy, *ddz, *rdx, *rdy, *rdz, *rddx, *rddy, *rddz;
    const double *u, *v, *w, *g;
    double *lu, *lv, *lw, *lp;
};

// one convective face flux q = 0.5 F (xa + xb) with F = A (c1 t1 + c2 t2):
// gq = dJ/dq scattered into the transported (la, lb) and transporting
// (lt1, lt2) adjoints
__device__ __forceinline__ void acc(double* p, double v) { *p += v; }

__device__ __forceinline__ void adj_face(double gq, double F, double xa, double xb, double* la,
                                         double* lb, double A, double c1, double* lt1, double c2,
                                         double* lt2) {
    const double gx = gq * 0.5 * F;
    acc(la, gx);
    acc(lb, gx);
    const double gF = gq * 0.5 * (xa + xb) * A;
    acc(lt1, gF * c1);
    acc(lt2, gF * c2);
}

// one viscous face flux: the output carries +cf (x1 - x0)
__device__ __forceinline__ void adj_diff(double l, double cf, double* l1, double* l0) {
    acc(l1, l * cf);
    acc(l0, -l * cf);
}

// transpose of the linearised tstle4 (kon about U, V, W; diff; gradp; body force)
__global__ void __launch_bounds__(256) k_adj_tstle4(const DevGrid* __restrict__ grids,
                                                    const double* const* __restrict__ sp,
                                                    const double* __restrict__ U,
                                                    const double* __restrict__ V,
                                                    const double* __restrict__ W,
                                                    const double* __restrict__ Gf,
                                                    const double* __restrict__ LUO,
                                                    const double* __restrict__ LVO,
                                                    const double* __restrict__ LWO,
                                                    double* LU, double* LV, double* LW, double* LP,
                                                    double* GFX, double* GFY, double* GFZ,
                                                    double gmol, double rho, int color) {
    const DevGrid Gd = grids[blockIdx.y];
    const int kk = Gd.kk, jj = Gd.jj, ii = Gd.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    if (i % 3 + 3 * (j % 3) + 9 * (k % 3) != color) return;
    const long long o = Gd.ip3;
    // every face is CON: the ranges of tstle4 are 3..n-2 for every component
    if (i < 3 || i > ii - 2 || j < 3 || j > jj - 2 || k < 3 || k > kk - 2) return;
    const double *dx = sp[0] + Gd.ipx - 1, *dy = sp[1] + Gd.ipy - 1, *dz = sp[2] + Gd.ipz - 1;
    const double *ddx = sp[3] + Gd.ipx - 1, *ddy = sp[4] + Gd.ipy - 1, *ddz = sp[5] + Gd.ipz - 1;
    const double *rdx = sp[6] + Gd.ipx - 1, *rdy = sp[7] + Gd.ipy - 1, *rdz = sp[8] + Gd.ipz - 1;
    const double *rddx = sp[9] + Gd.ipx - 1, *rddy = sp[10] + Gd.ipy - 1, *rddz = sp[11] + Gd.ipz - 1;
    const double *u = U + o, *v = V + o, *w = W + o, *gg = Gf + o;
    double *lu = LU + o, *lv = LV + o, *lw = LW + o, *lp = LP + o;
#define A(a, k, j, i) a[IX(k, j, i)]
#define P(a, k, j, i) (&a[IX(k, j, i)])
    // ---- U at (k, j, i)
    {
        const double l = LUO[o + t];
        GFX[o + t] += l;
        const double cp = 1.0 / (rho * dx[i]);
        acc(P(lp, k, j, i + 1), -cp * l);
        acc(P(lp, k, j, i), cp * l);
        // diff
        const double ax = ddy[j] * ddz[k], ay = dx[i] * ddz[k], az = dx[i] * ddy[j];
        const double fak = 1.0 / rho * rddy[j] * rdx[i] * rddz[k];
        const double ge = A(gg, k, j, i + 1), gw = A(gg, k, j, i);
        const double gn = hmean(A(gg, k, j, i), A(gg, k, j + 1, i), gmol) + hmean(A(gg, k, j, i + 1), A(gg, k, j + 1, i + 1), gmol);
        const double gs = hmean(A(gg, k, j - 1, i), A(gg, k, j, i), gmol) + hmean(A(gg, k, j - 1, i + 1), A(gg, k, j, i + 1), gmol);
        const double gt = hmean(A(gg, k, j, i), A(gg, k + 1, j, i), gmol) + hmean(A(gg, k, j, i + 1), A(gg, k + 1, j, i + 1), gmol);
        const double gb = hmean(A(gg, k - 1, j, i), A(gg, k, j, i), gmol) + hmean(A(gg, k - 1, j, i + 1), A(gg, k, j, i + 1), gmol);
        adj_diff(l, fak * ge * ax * rddx[i + 1], P(lu, k, j, i + 1), P(lu, k, j, i));
        adj_diff(l, fak * gw * ax * rddx[i], P(lu, k, j, i - 1), P(lu, k, j, i));
        adj_diff(l, fak * gn * ay * rdy[j], P(lu, k, j + 1, i), P(lu, k, j, i));
        adj_diff(l, fak * gs * ay * rdy[j - 1], P(lu, k, j - 1, i), P(lu, k, j, i));
        adj_diff(l, fak * gt * az * rdz[k], P(lu, k + 1, j, i), P(lu, k, j, i));
        adj_diff(l, fak * gb * az * rdz[k - 1], P(lu, k - 1, j, i), P(lu, k, j, i));
        // kon
        const double S = rdx[i] * rddy[j] * rddz[k];
        const double ae = 0.5 * dx[i] / ddx[i + 1], aw = 0.5 * dx[i - 1] / ddx[i];
        const double fe = ax * (A(u, k, j, i) + (A(u, k, j, i + 1) - A(u, k, j, i)) * ae);
        const double fw = ax * (A(u, k, j, i - 1) + (A(u, k, j, i) - A(u, k, j, i - 1)) * aw);
        const double fn = ay * (A(v, k, j, i) + A(v, k, j, i + 1)) * 0.5;
        const double fs = ay * (A(v, k, j - 1, i) + A(v, k, j - 1, i + 1)) * 0.5;
        const double ft = az * (A(w, k, j, i) + A(w, k, j, i + 1)) * 0.5;
        const double fb = az * (A(w, k - 1, j, i) + A(w, k - 1, j, i + 1)) * 0.5;
        adj_face(-S * l, fe, A(u, k, j, i), A(u, k, j, i + 1), P(lu, k, j, i), P(lu, k, j, i + 1), ax,
                 1.0 - ae, P(lu, k, j, i), ae, P(lu, k, j, i + 1));
        adj_face(S * l, fw, A(u, k, j, i - 1), A(u, k, j, i), P(lu, k, j, i - 1), P(lu, k, j, i), ax,
                 1.0 - aw, P(lu, k, j, i - 1), aw, P(lu, k, j, i));
        adj_face(-S * l, fn, A(u, k, j, i), A(u, k, j + 1, i), P(lu, k, j, i), P(lu, k, j + 1, i), ay,
                 0.5, P(lv, k, j, i), 0.5, P(lv, k, j, i + 1));
        adj_face(S * l, fs, A(u, k, j - 1, i), A(u, k, j, i), P(lu, k, j - 1, i), P(lu, k, j, i), ay,
                 0.5, P(lv, k, j - 1, i), 0.5, P(lv, k, j - 1, i + 1));
        adj_face(-S * l, ft, A(u, k, j, i), A(u, k + 1, j, i), P(lu, k, j, i), P(lu, k + 1, j, i), az,
                 0.5, P(lw, k, j, i), 0.5, P(lw, k, j, i + 1));
        adj_face(S * l, fb, A(u, k - 1, j, i), A(u, k, j, i), P(lu, k - 1, j, i), P(lu, k, j, i), az,
                 0.5, P(lw, k - 1, j, i), 0.5, P(lw, k - 1, j, i + 1));
    }
    // ---- V at (k, j, i)
    {
        const double l = LVO[o + t];
        GFY[o + t] += l;
        const double cp = 1.0 / (rho * dy[j]);
        acc(P(lp, k, j + 1, i), -cp * l);
        acc(P(lp, k, j, i), cp * l);
        const double ax = dy[j] * ddz[k], ay = ddx[i] * ddz[k], az = ddx[i] * dy[j];
        const double fak = 1.0 / rho * rddx[i] * rdy[j] * rddz[k];
        const double ge = hmean(A(gg, k, j, i), A(gg, k, j, i + 1), gmol) + hmean(A(gg, k, j + 1, i), A(gg, k, j + 1, i + 1), gmol);
        const double gw = hmean(A(gg, k, j, i - 1), A(gg, k, j, i), gmol) + hmean(A(gg, k, j + 1, i - 1), A(gg, k, j + 1, i), gmol);
        const double gn = A(gg, k, j + 1, i), gs = A(gg, k, j, i);
        const double gt = hmean(A(gg, k, j, i), A(gg, k + 1, j, i), gmol) + hmean(A(gg, k, j + 1, i), A(gg, k + 1, j + 1, i), gmol);
        const double gb = hmean(A(gg, k - 1, j, i), A(gg, k, j, i), gmol) + hmean(A(gg, k - 1, j + 1, i), A(gg, k, j + 1, i), gmol);
        adj_diff(l, fak * ge * ax * rdx[i], P(lv, k, j, i + 1), P(lv, k, j, i));
        adj_diff(l, fak * gw * ax * rdx[i - 1], P(lv, k, j, i - 1), P(lv, k, j, i));
        adj_diff(l, fak * gn * ay * rddy[j + 1], P(lv, k, j + 1, i), P(lv, k, j, i));
        adj_diff(l, fak * gs * ay * rddy[j], P(lv, k, j - 1, i), P(lv, k, j, i));
        adj_diff(l, fak * gt * az * rdz[k], P(lv, k + 1, j, i), P(lv, k, j, i));
        adj_diff(l, fak * gb * az * rdz[k - 1], P(lv, k - 1, j, i), P(lv, k, j, i));
        const double S = rddx[i] * rdy[j] * rddz[k];
        const double an = 0.5 * dy[j] / ddy[j + 1], as = 0.5 * dy[j - 1] / ddy[j];
        const double fe = ax * (A(u, k, j, i) + A(u, k, j + 1, i)) * 0.5;
        const double fw = ax * (A(u, k, j, i - 1) + A(u, k, j + 1, i - 1)) * 0.5;
        const double fn = ay * (A(v, k, j, i) + (A(v, k, j + 1, i) - A(v, k, j, i)) * an);
        const double fs = ay * (A(v, k, j - 1, i) + (A(v, k, j, i) - A(v, k, j - 1, i)) * as);
        const double ft = az * (A(w, k, j, i) + A(w, k, j + 1, i)) * 0.5;
        const double fb = az * (A(w, k - 1, j, i) + A(w, k - 1, j + 1, i)) * 0.5;
        adj_face(-S * l, fe, A(v, k, j, i), A(v, k, j, i + 1), P(lv, k, j, i), P(lv, k, j, i + 1), ax,
                 0.5, P(lu, k, j, i), 0.5, P(lu, k, j + 1, i));
        adj_face(S * l, fw, A(v, k, j, i - 1), A(v, k, j, i), P(lv, k, j, i - 1), P(lv, k, j, i), ax,
                 0.5, P(lu, k, j, i - 1), 0.5, P(lu, k, j + 1, i - 1));
        adj_face(-S * l, fn, A(v, k, j, i), A(v, k, j + 1, i), P(lv, k, j, i), P(lv, k, j + 1, i), ay,
                 1.0 - an, P(lv, k, j, i), an, P(lv, k, j + 1, i));
        adj_face(S * l, fs, A(v, k, j - 1, i), A(v, k, j, i), P(lv, k, j - 1, i), P(lv, k, j, i), ay,
                 1.0 - as, P(lv, k, j - 1, i), as, P(lv, k, j, i));
        adj_face(-S * l, ft, A(v, k, j, i), A(v, k + 1, j, i), P(lv, k, j, i), P(lv, k + 1, j, i), az,
                 0.5, P(lw, k, j, i), 0.5, P(lw, k, j + 1, i));
        adj_face(S * l, fb, A(v, k - 1, j, i), A(v, k, j, i), P(lv, k - 1, j, i), P(lv, k, j, i), az,
                 0.5, P(lw, k - 1, j, i), 0.5, P(lw, k - 1, j + 1, i));
    }
    // ---- W at (k, j, i)
    {
        const double l = LWO[o + t];
        GFZ[o + t] += l;
        const double cp = 1.0 / (rho * dz[k]);
        acc(P(lp, k + 1, j, i), -cp * l);
        acc(P(lp, k, j, i), cp * l);
        const double ax = ddy[j] * dz[k], ay = ddx[i] * dz[k], az = ddx[i] * ddy[j];
        const double fak = 1.0 / rho * rddx[i] * rddy[j] * rdz[k];
        const double ge = hmean(A(gg, k, j, i), A(gg, k, j, i + 1), gmol) + hmean(A(gg, k + 1, j, i), A(gg, k + 1, j, i + 1), gmol);
        const double gw = hmean(A(gg, k, j, i - 1), A(gg, k, j, i), gmol) + hmean(A(gg, k + 1, j, i - 1), A(gg, k + 1, j, i), gmol);
        const double gn = hmean(A(gg, k, j, i), A(gg, k, j + 1, i), gmol) + hmean(A(gg, k + 1, j, i), A(gg, k + 1, j + 1, i), gmol);
        const double gs = hmean(A(gg, k, j - 1, i), A(gg, k, j, i), gmol) + hmean(A(gg, k + 1, j - 1, i), A(gg, k + 1, j, i), gmol);
        const double gt = A(gg, k + 1, j, i), gb = A(gg, k, j, i);
        adj_diff(l, fak * ge * ax * rdx[i], P(lw, k, j, i + 1), P(lw, k, j, i));
        adj_diff(l, fak * gw * ax * rdx[i - 1], P(lw, k, j, i - 1), P(lw, k, j, i));
        adj_diff(l, fak * gn * ay * rdy[j], P(lw, k, j + 1, i), P(lw, k, j, i));
        adj_diff(l, fak * gs * ay * rdy[j - 1], P(lw, k, j - 1, i), P(lw, k, j, i));
        adj_diff(l, fak * gt * az * rddz[k + 1], P(lw, k + 1, j, i), P(lw, k, j, i));
        adj_diff(l, fak * gb * az * rddz[k], P(lw, k - 1, j, i), P(lw, k, j, i));
        const double S = rddx[i] * rddy[j] * rdz[k];
        const double at = 0.5 * dz[k] / ddz[k + 1], ab = 0.5 * dz[k - 1] / ddz[k];
        const double fe = ax * (A(u, k, j, i) + A(u, k + 1, j, i)) * 0.5;
        const double fw = ax * (A(u, k, j, i - 1) + A(u, k + 1, j, i - 1)) * 0.5;
        const double fn = ay * (A(v, k, j, i) + A(v, k + 1, j, i)) * 0.5;
        const double fs = ay * (A(v, k, j - 1, i) + A(v, k + 1, j - 1, i)) * 0.5;
        const double ft = az * (A(w, k, j, i) + (A(w, k + 1, j, i) - A(w, k, j, i)) * at);
        const double fb = az * (A(w, k - 1, j, i) + (A(w, k, j, i) - A(w, k - 1, j, i)) * ab);
        adj_face(-S * l, fe, A(w, k, j, i), A(w, k, j, i + 1), P(lw, k, j, i), P(lw, k, j, i + 1), ax,
                 0.5, P(lu, k, j, i), 0.5, P(lu, k + 1, j, i));
        adj_face(S * l, fw, A(w, k, j, i - 1), A(w, k, j, i), P(lw, k, j, i - 1), P(lw, k, j, i), ax,
                 0.5, P(lu, k, j, i - 1), 0.5, P(lu, k + 1, j, i - 1));
        adj_face(-S * l, fn, A(w, k, j, i), A(w, k, j + 1, i), P(lw, k, j, i), P(lw, k, j + 1, i), ay,
                 0.5, P(lv, k, j, i), 0.5, P(lv, k + 1, j, i));
        adj_face(S * l, fs, A(w, k, j - 1, i), A(w, k, j, i), P(lw, k, j - 1, i), P(lw, k, j, i), ay,
                 0.5, P(lv, k, j - 1, i), 0.5, P(lv, k + 1, j - 1, i));
        adj_face(-S * l, ft, A(w, k, j, i), A(w, k + 1, j, i), P(lw, k, j, i), P(lw, k + 1, j, i), az,
                 1.0 - at, P(lw, k, j, i), at, P(lw, k + 1, j, i));
        adj_face(S * l, fb, A(w, k - 1, j, i), A(w, k, j, i), P(lw, k - 1, j, i), P(lw, k, j, i), az,
                 1.0 - ab, P(lw, k - 1, j, i), ab, P(lw, k, j, i));
    }
#undef P
#undef A
}

// dJ/du of the enerfg energy: every face gathers from its two interior cells
__global__ void k_energy_grad(const DevGrid* __restrict__ grids, const double* const* __restrict__ sp,
                              const double* __restrict__ U, const double* __restrict__ V,
                              const double* __restrict__ W, double* __restrict__ LU,
                              double* __restrict__ LV, double* __restrict__ LW, double rvol) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    const long long o = G.ip3;
    const double *dx = sp[0] + G.ipx - 1, *dy = sp[1] + G.ipy - 1, *dz = sp[2] + G.ipz - 1;
    const double *ddx = sp[3] + G.ipx - 1, *ddy = sp[4] + G.ipy - 1, *ddz = sp[5] + G.ipz - 1;
    const double *u = U + o, *v = V + o, *w = W + o;
    auto in = [&](int kx, int jx, int ix) {
        return ix >= 3 && ix <= ii - 2 && jx >= 3 && jx <= jj - 2 && kx >= 3 && kx <= kk - 2;
    };
    // up(cell c) = u(c-1) + (u(c) - u(c-1)) b, b = 0.5 dx(c-1) / ddx(c)
    double su = 0.0, sv = 0.0, sw = 0.0;
    for (int s = 0; s < 2; ++s) {
        {   // cell i + s along x holds u(k, j, i) as its u(c) (s = 0) or u(c-1) (s = 1)
            const int c = i + s;
            if (in(k, j, c)) {
                const double b = 0.5 * dx[c - 1] / ddx[c];
                const double up = u[IX(k, j, c - 1)] + (u[IX(k, j, c)] - u[IX(k, j, c - 1)]) * b;
                su += ddx[c] * ddy[j] * ddz[k] * up * (s == 0 ? b : 1.0 - b);
            }
        }
        {
            const int c = j + s;
            if (in(k, c, i)) {
                const double b = 0.5 * dy[c - 1] / ddy[c];
                const double vp = v[IX(k, c - 1, i)] + (v[IX(k, c, i)] - v[IX(k, c - 1, i)]) * b;
                sv += ddx[i] * ddy[c] * ddz[k] * vp * (s == 0 ? b : 1.0 - b);
            }
        }
        {
            const int c = k + s;
            if (in(c, j, i)) {
                const double b = 0.5 * dz[c - 1] / ddz[c];
                const double wp = w[IX(c - 1, j, i)] + (w[IX(c, j, i)] - w[IX(c - 1, j, i)]) * b;
                sw += ddx[i] * ddy[j] * ddz[c] * wp * (s == 0 ? b : 1.0 - b);
            }
        }
    }
    LU[o + t] = su * rvol;
    LV[o + t] = sv * rvol;
    LW[o + t] = sw * rvol;
}

#undef IX

const double* const* spacing_table(Ctx* c) {
    if (!c->d_sptab) {
        const char* n[12] = {"DX", "DY", "DZ", "DDX", "DDY", "DDZ", "RDX", "RDY", "RDZ", "RDDX", "RDDY", "RDDZ"};
        const double* h[12];
        for (int q = 0; q < 12; ++q) h[q] = c->L(n[q]);
        if (cudaMalloc(&c->d_sptab, sizeof(h)) != cudaSuccess) return nullptr;
        if (copy_on(c->stream, c->d_sptab, h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess)
            return nullptr;
    }
    return reinterpret_cast<const double* const*>(c->d_sptab);
}

dim3 box_grid(Ctx* c) {
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    return dim3((m + 255) / 256, c->ngrid);
}

int adj_connect(Ctx* c, int ilevel, int layers, int slots, bool corners, bool normal, int fwd,
                double* const f[6]) {
    const ConnectPlan* cplan = nullptr;
    if (int rc = get_plan(c, ilevel, layers, slots, corners, normal, fwd, &cplan)) return rc;
    if (cplan->ntasks == 0) return 0;
    ConnectPlan* plan = const_cast<ConnectPlan*>(cplan);
    if (!plan->d_bysrc) {
        // group the copies by the grid holding their source (stable: the
        // copies of a group keep the plan's order)
        std::vector<BoxCopy> tasks(plan->ntasks);
        MG_CUDA(copy_on(c->stream, tasks.data(), plan->d_tasks, tasks.size() * sizeof(BoxCopy),
                        cudaMemcpyDeviceToHost));
        auto src_grid = [&](long long src) {
            int g = 0;
            for (int q = 0; q < c->ngrid; ++q)
                if (c->grids[q].ip3 <= src) g = q;
            return g;
        };
        std::vector<std::pair<int, int>> key(tasks.size());
        for (size_t q = 0; q < tasks.size(); ++q) key[q] = {src_grid(tasks[q].src), (int)q};
        std::stable_sort(key.begin(), key.end());
        std::vector<BoxCopy> sorted;
        std::vector<int> start;
        for (size_t q = 0; q < key.size(); ++q) {
            if (q == 0 || key[q].first != key[q - 1].first) start.push_back((int)q);
            sorted.push_back(tasks[key[q].second]);
        }
        start.push_back((int)key.size());
        MG_CUDA(cudaMalloc(&plan->d_bysrc, sorted.size() * sizeof(BoxCopy)));
        MG_CUDA(copy_on(c->stream, plan->d_bysrc, sorted.data(), sorted.size() * sizeof(BoxCopy),
                        cudaMemcpyHostToDevice));
        MG_CUDA(cudaMalloc(&plan->d_srcstart, start.size() * sizeof(int)));
        MG_CUDA(copy_on(c->stream, plan->d_srcstart, start.data(), start.size() * sizeof(int),
                        cudaMemcpyHostToDevice));
        plan->nsrc = (int)start.size() - 1;
    }
    AdjSlots fs;
    for (int q = 0; q < 6; ++q) fs.f[q] = f[q];
    k_adj_connect<<<plan->nsrc, 128, 0, c->stream>>>(plan->d_bysrc, plan->d_srcstart, fs);
    MG_LAUNCHED(c);
    return 0;
}

}  // namespace

int adjoint_ready(Ctx* c) {
    if (c->prm.form != MGLET_FORM_PLAIN)
        return fail(MGLET_ERR_UNSUPPORTED, "adjoint: the plain FP64 form only");
    if (c->part)
        return fail(MGLET_ERR_UNSUPPORTED, "adjoint: one rank (no grid partition)");
    if (c->minlevel != c->maxlevel || c->ibtype != 0)
        return fail(MGLET_ERR_UNSUPPORTED, "adjoint: one grid level without immersed boundary");
    if (c->prm.psolver == MGLET_PSOLVER_SOR)
        return fail(MGLET_ERR_UNSUPPORTED, "adjoint: the SIP pressure solver");
    if (c->ilesmodel != 0)
        return fail(MGLET_ERR_UNSUPPORTED, "adjoint: constant viscosity (no LES model)");
    for (const DevGrid& G : c->grids)
        for (int f = 0; f < 6; ++f)
            if (G.bc[f] != MGLET_BC_CON)
                return fail(MGLET_ERR_UNSUPPORTED, "adjoint: every face CON (periodic boxes)");
    // the transposed pressure solve uses the symmetry of the Laplacian of
    // uniform grids
    for (const char* n : {"DDX", "DDY", "DDZ", "DX", "DY", "DZ"}) {
        const long long len = n[std::strlen(n) - 1] == 'X' ? c->idimx : (n[std::strlen(n) - 1] == 'Y' ? c->idimy : c->idimz);
        std::vector<double> h((size_t)len);
        MG_CUDA(copy_on(c->stream, h.data(), c->L(n), h.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (double x : h)
            if (x != h[0]) return fail(MGLET_ERR_UNSUPPORTED, "adjoint: uniform grid spacing");
    }
    for (const char* n : {"LU", "LV", "LW", "LP", "LDU", "LDV", "LDW", "LDP", "GFX", "GFY", "GFZ"})
        if (!c->f3.count(n))
            if (int rc = alloc_field3(c, n)) return rc;
    return 0;
}

// The adjoint of one stage: U, V, W hold the stage input, the L* fields the
// adjoint of the stage output; on return the L* fields hold the adjoint of
// the stage input and GF* has gained dJ/df of this stage.
int adjoint_stage(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk) {
    double frhs, fu, dtrk, dtrki;
    if (int rc = rk_coeffs(rk, irk, &frhs, &fu, &dtrk, &dtrki)) return rc;
    const double dtm = dtrk * dt, prefak = c->prm.rho / dtm, rfak = dtm / c->prm.rho;
    double *LU = c->F("LU"), *LV = c->F("LV"), *LW = c->F("LW"), *LP = c->F("LP");
    double *LDP = c->F("LDP");
    const int l0 = c->minlevel;
    const dim3 bg = box_grid(c);
    // mgpoisl's closing connect(2 layers, corners) of U, V, W, P
    {
        double* f[6] = {LU, LV, LW, LP, nullptr, nullptr};
        if (int rc = adj_connect(c, l0, 2, 15, true, false, 0, f)) return rc;
    }
    // mgpcorr, then the ghost faces of dp (the connects of hilf and dp)
    k_adj_mgpcorr<<<bg, 256, 0, c->stream>>>(c->d_grids, LU, LV, LW, LP, LDP, c->L("RDX"), c->L("RDY"),
                                             c->L("RDZ"), rfak);
    MG_LAUNCHED(c);
    {
        double* f[6] = {nullptr, nullptr, nullptr, LDP, nullptr, nullptr};
        if (int rc = adj_connect(c, 0, 1, 8, false, false, 0, f)) return rc;
    }
    // dp = L^-1 rhs: lambda(rhs) = L^-1 (lambda(dp) - mean) by the SIP outer loop
    {
        k_interior_sum<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, LDP, c->d_gridred);
        MG_LAUNCHED(c);
        std::vector<double> sums(c->ngrid);
        MG_CUDA(copy_on(c->stream, sums.data(), c->d_gridred, sums.size() * sizeof(double),
                        cudaMemcpyDeviceToHost));
        double tot = 0.0;
        long long ncell = 0;
        for (int g = 0; g < c->ngrid; ++g) {
            tot += sums[g];
            const DevGrid& G = c->grids[g];
            ncell += (long long)(G.kk - 4) * (G.jj - 4) * (G.ii - 4);
        }
        double* rhs = c->F("RHS");
        k_centre_rhs<<<bg, 256, 0, c->stream>>>(c->d_grids, LDP, rhs, tot / (double)ncell);
        MG_LAUNCHED(c);
        mglet_stage_stats st;
        if (int rc = solve_pressure_system(c, 0.0, &st, true)) return rc;
    }
    k_adj_divcal<<<bg, 256, 0, c->stream>>>(c->d_grids, LU, LV, LW, c->F("DP"), c->L("RDDX"),
                                            c->L("RDDY"), c->L("RDDZ"), prefak);
    MG_LAUNCHED(c);
    // connect(1 layer, normal, forward=1) after the RK update
    {
        double* f[6] = {LU, LV, LW, nullptr, nullptr, nullptr};
        if (int rc = adj_connect(c, l0, 1, 7, false, true, 1, f)) return rc;
    }
    // rkstep of U, V, W: lambda(UO) into UO, VO, WO
    const long long n = c->idim3d;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_adj_rkstep<<<blocks, 256, 0, c->stream>>>(LU, c->F("LDU"), c->F("UO"), frhs, dt * fu, n);
    k_adj_rkstep<<<blocks, 256, 0, c->stream>>>(LV, c->F("LDV"), c->F("VO"), frhs, dt * fu, n);
    k_adj_rkstep<<<blocks, 256, 0, c->stream>>>(LW, c->F("LDW"), c->F("WO"), frhs, dt * fu, n);
    MG_LAUNCHED(c);
    const double* const* sp = spacing_table(c);
    if (!sp) return fail(MGLET_ERR_CUDA, "adjoint: spacing table");
    for (int color = 0; color < 27; ++color) {
        k_adj_tstle4<<<bg, 256, 0, c->stream>>>(c->d_grids, sp, c->F("U"), c->F("V"), c->F("W"),
                                                c->F("G"), c->F("UO"), c->F("VO"), c->F("WO"), LU, LV,
                                                LW, LP, c->F("GFX"), c->F("GFY"), c->F("GFZ"),
                                                c->prm.gmol, c->prm.rho, color);
        MG_LAUNCHED(c);
    }
    return 0;
}

// L* = dJ/d(U, V, W) of the enerfg energy of the current state; returns J
int energy_gradient_init(Ctx* c, double* J) {
    if (int rc = launch_itinfo(c, 1.0)) return rc;
    std::vector<double> red((size_t)4 * c->ngrid);
    MG_CUDA(copy_on(c->stream, red.data(), c->d_gridred, red.size() * sizeof(double),
                    cudaMemcpyDeviceToHost));
    double es = 0.0, vol = 0.0;
    for (int g = 0; g < c->ngrid; ++g) {
        const double ge = red[4 * g + 2] / red[4 * g + 3], gv = red[4 * g + 3];
        es = (vol + gv > 0.0) ? (es * vol + ge * gv) / (vol + gv) : 0.0;
        vol = vol + gv;
    }
    *J = es;
    const double* const* sp = spacing_table(c);
    if (!sp) return fail(MGLET_ERR_CUDA, "adjoint: spacing table");
    k_energy_grad<<<box_grid(c), 256, 0, c->stream>>>(c->d_grids, sp, c->F("U"), c->F("V"), c->F("W"),
                                                      c->F("LU"), c->F("LV"), c->F("LW"), 1.0 / vol);
    MG_LAUNCHED(c);
    const size_t bytes = (size_t)c->idim3d * sizeof(double);
    for (const char* n : {"LP", "LDU", "LDV", "LDW", "GFX", "GFY", "GFZ"})
        MG_CUDA(cudaMemsetAsync(c->F(n), 0, bytes, c->stream));
    return 0;
}

// the adjoint of the initial connect(2 layers, corners): ghost adjoints of
// the initial state onto the interior points they copy
int adjoint_fold_initial(Ctx* c) {
    double* f[6] = {c->F("LU"), c->F("LV"), c->F("LW"), c->F("LP"), nullptr, nullptr};
    return adj_connect(c, 0, 2, 15, true, false, 0, f);
}

// dJ/df of the kinetic energy after nsteps time steps from the current
// state: the forward run keeps the state (U, V, W, P, DU, DV, DW) every
// ncheck steps; each segment is run forward again from its checkpoint
// keeping every stage's input velocity, and its stages are run backwards
// through adjoint_stage.  GF* receive dJ/df, L* dJ/d(u, v, w, p) of the
// initial state; the context ends in the final forward state.
int energy_gradient(Ctx* c, int nsteps, int ncheck, double dt, const mglet_rk_scheme* rk, double* J) {
    if (int rc = adjoint_ready(c)) return rc;
    if (nsteps < 1 || ncheck < 1 || !rk || rk->nrk < 1 || !J)
        return fail(MGLET_ERR_ARG, "energy_gradient: nsteps, ncheck >= 1 and a scheme");
    const int nrk = rk->nrk;
    const size_t fb = (size_t)c->idim3d * sizeof(double);
    const char* st7[7] = {"U", "V", "W", "P", "DU", "DV", "DW"};
    const int nck = (nsteps + ncheck - 1) / ncheck;
    const int seg = std::min(ncheck, nsteps);
    double *ck = nullptr, *stg = nullptr, *fin = nullptr;
    auto release = [&]() {
        cudaFree(ck);
        cudaFree(stg);
        cudaFree(fin);
    };
    if (cudaMalloc(&ck, (size_t)nck * 7 * fb) != cudaSuccess ||
        cudaMalloc(&stg, (size_t)seg * nrk * 3 * fb) != cudaSuccess ||
        cudaMalloc(&fin, 7 * fb) != cudaSuccess) {
        release();
        return fail(MGLET_ERR_CUDA, "energy_gradient: checkpoint memory");
    }
    auto save = [&](double* dst) -> int {
        for (int q = 0; q < 7; ++q)
            MG_CUDA(cudaMemcpyAsync((char*)dst + q * fb, c->F(st7[q]), fb, cudaMemcpyDeviceToDevice, c->stream));
        return 0;
    };
    auto load = [&](const double* src) -> int {
        for (int q = 0; q < 7; ++q)
            MG_CUDA(cudaMemcpyAsync(c->F(st7[q]), (const char*)src + q * fb, fb, cudaMemcpyDeviceToDevice, c->stream));
        return 0;
    };
    int rc = 0;
    for (int s = 0; s < nsteps && !rc; ++s) {
        if (s % ncheck == 0) rc = save(ck + (size_t)(s / ncheck) * 7 * (fb / sizeof(double)));
        for (int irk = 1; irk <= nrk && !rc; ++irk) rc = timeintegrate(c, dt, irk, rk, nullptr);
    }
    if (!rc) rc = save(fin);
    if (!rc) rc = energy_gradient_init(c, J);
    for (int g = nck - 1; g >= 0 && !rc; --g) {
        const int s0 = g * ncheck, s1 = std::min(nsteps, s0 + ncheck);
        rc = load(ck + (size_t)g * 7 * (fb / sizeof(double)));
        int q = 0;
        for (int s = s0; s < s1 && !rc; ++s)
            for (int irk = 1; irk <= nrk && !rc; ++irk, ++q) {
                for (int m = 0; m < 3 && !rc; ++m)
                    if (cudaMemcpyAsync((char*)stg + ((size_t)q * 3 + m) * fb, c->F(st7[m]), fb,
                                        cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
                        rc = fail(MGLET_ERR_CUDA, "energy_gradient: stage copy");
                if (!rc) rc = timeintegrate(c, dt, irk, rk, nullptr);
            }
        for (int qq = q - 1; qq >= 0 && !rc; --qq) {
            for (int m = 0; m < 3 && !rc; ++m)
                if (cudaMemcpyAsync(c->F(st7[m]), (const char*)stg + ((size_t)qq * 3 + m) * fb, fb,
                                    cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
                    rc = fail(MGLET_ERR_CUDA, "energy_gradient: stage copy");
            if (!rc) rc = adjoint_stage(c, dt, qq % nrk + 1, rk);
        }
    }
    if (!rc) rc = adjoint_fold_initial(c);
    if (!rc) rc = load(fin);
    if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = fail(MGLET_ERR_CUDA, "energy_gradient: synchronize");
    release();
    return rc;
}

}  // namespace mg
