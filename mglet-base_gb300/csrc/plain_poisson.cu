// plain_poisson.cu -- FP64 parity form of the pressure-Poisson machinery.
// Compiled with -fmad=false (reference operation order, separate rounding).
//
//   giteig                 src/ib/noib_mod.F90:81-250
//   divcal (noib)          src/ib/noib_mod.F90:253-354
//   laplacephi_grid        src/flow/laplacephi_mod.F90:134-165
//   sip_hyperplane_lu      src/flow/sip_hyperplane_mod.F90:106-257
//   sip_classic_init       src/flow/sip_classic_mod.F90:17-127
//   sipiter1/2 hyperplane  src/flow/sip_hyperplane_mod.F90:450-569
//   sipiter1/2 classic     src/flow/sip_classic_mod.F90:143-198
//   relax (SOR)            src/flow/sor_mod.F90:102-203
//   rescal + maxabscal     src/flow/pressuresolver_mod.F90:623-742
//   accumulate_pcorr       src/flow/pressuresolver_mod.F90:882-908
//   mgpcorr_grid           src/flow/pressuresolver_mod.F90:787-879
//
// The SIP recurrences run as i+j+k hyperplane wavefronts: one CTA per grid
// walks the 70 planes of a 24^3 grid, every thread of the CTA taking points
// of the current plane; the plane barrier is __syncthreads().  Each point
// evaluates the reference's expression in the reference's order, so the
// schedule does not change any rounding.
#include <algorithm>

#include "internal.h"

namespace mg {
MG_PLAIN_BEGIN
namespace {

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

// Fortran default-kind literals of the SIP factorisation, widened to FP64
// (sip_hyperplane_mod.F90:123,202).
__device__ __constant__ double c_alfa = (double)0.92f;
__device__ __constant__ double c_tiny = (double)1.0e-20f;

__device__ __forceinline__ double block_max(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    __syncthreads();
    return v;   // valid in thread 0
}

// ---------------------------------------------------------------------------
// giteig: 1-D neighbour coefficients and the 3-D diagonal with BP and wall
// corrections.  One CTA per grid.
__global__ void k_giteig(const DevGrid* __restrict__ grids, const double* __restrict__ DX,
                         const double* __restrict__ DY, const double* __restrict__ DZ,
                         double* AW, double* AE, double* AS, double* AN, double* AB, double* AT,
                         double* AP, const double* __restrict__ BP) {
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const double* dx = DX + G.ipx - 1;
    const double* dy = DY + G.ipy - 1;
    const double* dz = DZ + G.ipz - 1;
    double* aw = AW + G.ipx - 1; double* ae = AE + G.ipx - 1;
    double* as = AS + G.ipy - 1; double* an = AN + G.ipy - 1;
    double* ab = AB + G.ipz - 1; double* at = AT + G.ipz - 1;
    double* ap = AP + G.ip3;
    const double* bp = BP + G.ip3;
    for (int q = threadIdx.x; q < ii + jj + kk; q += blockDim.x) {
        if (q < ii) {
            int i = q + 1;
            if (i >= 3 && i <= ii - 2) {
                ae[i] = 2.0 / ((dx[i - 1] + dx[i]) * dx[i]);
                aw[i] = 2.0 / ((dx[i - 1] + dx[i]) * dx[i - 1]);
            }
        } else if (q < ii + jj) {
            int j = q - ii + 1;
            if (j >= 3 && j <= jj - 2) {
                an[j] = 2.0 / ((dy[j - 1] + dy[j]) * dy[j]);
                as[j] = 2.0 / ((dy[j - 1] + dy[j]) * dy[j - 1]);
            }
        } else {
            int k = q - ii - jj + 1;
            if (k >= 3 && k <= kk - 2) {
                at[k] = 2.0 / ((dz[k - 1] + dz[k]) * dz[k]);
                ab[k] = 2.0 / ((dz[k - 1] + dz[k]) * dz[k - 1]);
            }
        }
    }
    __syncthreads();
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const bool wf = G.bc[0] == 2 || G.bc[0] == 5 || G.bc[0] == 6 || G.bc[0] == 19;
    const bool wb = G.bc[1] == 2 || G.bc[1] == 5 || G.bc[1] == 6;
    const bool wr = G.bc[2] == 2 || G.bc[2] == 5 || G.bc[2] == 6 || G.bc[2] == 19;
    const bool wl = G.bc[3] == 2 || G.bc[3] == 5 || G.bc[3] == 6;
    const bool wbo = G.bc[4] == 2 || G.bc[4] == 5 || G.bc[4] == 6 || G.bc[4] == 19;
    const bool wt = G.bc[5] == 2 || G.bc[5] == 5 || G.bc[5] == 6;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        double a = -2.0 / (dx[i - 1] * dx[i]) - 2.0 / (dy[j - 1] * dy[j]) - 2.0 / (dz[k - 1] * dz[k]);
        a = a + aw[i] * (1.0 - bp[IX(k, j, i - 1)] * bp[IX(k, j, i)]) +
            ae[i] * (1.0 - bp[IX(k, j, i)] * bp[IX(k, j, i + 1)]) +
            as[j] * (1.0 - bp[IX(k, j - 1, i)] * bp[IX(k, j, i)]) +
            an[j] * (1.0 - bp[IX(k, j, i)] * bp[IX(k, j + 1, i)]) +
            ab[k] * (1.0 - bp[IX(k - 1, j, i)] * bp[IX(k, j, i)]) +
            at[k] * (1.0 - bp[IX(k, j, i)] * bp[IX(k + 1, j, i)]);
        if (wf && i == 3) a = a + aw[3] * (bp[IX(k, j, 2)] * bp[IX(k, j, 3)]);
        if (wb && i == ii - 2) a = a + ae[ii - 2] * (bp[IX(k, j, ii - 2)] * bp[IX(k, j, ii - 1)]);
        if (wr && j == 3) a = a + as[3] * (bp[IX(k, 2, i)] * bp[IX(k, 3, i)]);
        if (wl && j == jj - 2) a = a + an[jj - 2] * (bp[IX(k, jj - 2, i)] * bp[IX(k, jj - 1, i)]);
        if (wbo && k == 3) a = a + ab[3] * (bp[IX(2, j, i)] * bp[IX(3, j, i)]);
        if (wt && k == kk - 2) a = a + at[kk - 2] * (bp[IX(kk - 2, j, i)] * bp[IX(kk - 1, j, i)]);
        ap[IX(k, j, i)] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (wf) aw[3] = 0.0;
        if (wb) ae[ii - 2] = 0.0;
        if (wr) as[3] = 0.0;
        if (wl) an[jj - 2] = 0.0;
        if (wbo) ab[3] = 0.0;
        if (wt) at[kk - 2] = 0.0;
    }
}

// ---------------------------------------------------------------------------
// SIP incomplete-LU factorisation in hyperplane order.  tmp holds 7 zeroed
// per-grid scratch slabs (lw, ls, lb, lpr, ue, un, ut in natural layout);
// the result goes to the coefficient fields either in plane order (iacc,
// hyperplane solver) or in natural order (classic solver).
struct LuArgs {
    const DevGrid* grids;
    int g0;
    const int* mip; const int* idx;     // table of the (uniform or per-class) shape
    const int* const* mips; const int* const* idxs;
    const double *aw, *ae, *as, *an, *ab, *at, *ap, *bp;
    double *lw, *ls, *lb, *lpr, *ue, *un, *ut;
    double* tmp;
    long long tmpstride;
    int planeorder;
};

__global__ void k_sip_lu(LuArgs a) {
    const int gi = a.g0 + blockIdx.x;
    const DevGrid G = a.grids[gi];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int* mip = a.mips[G.cls];
    const int* idx = a.idxs[G.cls];
    const long long npt = (long long)kk * jj * ii;
    double* T = a.tmp + (long long)blockIdx.x * 7 * npt;
    double *lw_t = T, *ls_t = T + npt, *lb_t = T + 2 * npt, *lpr_t = T + 3 * npt,
           *ue_t = T + 4 * npt, *un_t = T + 5 * npt, *ut_t = T + 6 * npt;
    const double* aw = a.aw + G.ipx - 1; const double* ae = a.ae + G.ipx - 1;
    const double* as = a.as + G.ipy - 1; const double* an = a.an + G.ipy - 1;
    const double* ab = a.ab + G.ipz - 1; const double* at = a.at + G.ipz - 1;
    const double* ap = a.ap + G.ip3;
    const double* bp = a.bp + G.ip3;
    const long long o = G.ip3;
    const int n3dmin = 9, n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    for (int m = n3dmin; m <= n3dmax; ++m) {
        const int lm = mip[m], lp = mip[m + 1] - lm;
        for (int ip = threadIdx.x; ip < lp; ip += blockDim.x) {
            const int iacc = lm + ip;
            const int id = idx[iacc];
            const int km = id - 1, jm = id - kk, im = id - kk * jj;
            const int k = id % kk + 1, j = (id / kk) % jj + 1, i = id / (kk * jj) + 1;
            const double bu_im = bp[IX(k, j, i - 1)] * bp[IX(k, j, i)];
            const double bv_jm = bp[IX(k, j - 1, i)] * bp[IX(k, j, i)];
            const double bw_km = bp[IX(k - 1, j, i)] * bp[IX(k, j, i)];
            const double bu = bp[IX(k, j, i)] * bp[IX(k, j, i + 1)];
            const double bv = bp[IX(k, j, i)] * bp[IX(k, j + 1, i)];
            const double bw = bp[IX(k, j, i)] * bp[IX(k + 1, j, i)];
            double lw = aw[i] * bu_im / (1.0 + c_alfa * (un_t[im] + ut_t[im]));
            double ls = as[j] * bv_jm / (1.0 + c_alfa * (ue_t[jm] + ut_t[jm]));
            double lb = ab[k] * bw_km / (1.0 + c_alfa * (un_t[km] + ue_t[km]));
            double p1 = c_alfa * (lb * ue_t[km] + ls * ue_t[jm]);
            double p2 = c_alfa * (lb * un_t[km] + lw * un_t[im]);
            double p3 = c_alfa * (lw * ut_t[im] + ls * ut_t[jm]);
            double lpr = 1.0 / (ap[id] + p1 + p2 + p3 - lb * ut_t[km] - lw * ue_t[im] -
                                ls * un_t[jm] + c_tiny);
            double ue = (ae[i] * bu - p1) * lpr;
            double un = (an[j] * bv - p2) * lpr;
            double ut = (at[k] * bw - p3) * lpr;
            lw = lw * lpr;
            ls = ls * lpr;
            lb = lb * lpr;
            lw_t[id] = lw; ls_t[id] = ls; lb_t[id] = lb; lpr_t[id] = lpr;
            ue_t[id] = ue; un_t[id] = un; ut_t[id] = ut;
            const long long dst = a.planeorder ? o + iacc : o + id;
            a.lw[dst] = lw; a.ls[dst] = ls; a.lb[dst] = lb; a.lpr[dst] = lpr;
            a.ue[dst] = ue; a.un[dst] = un; a.ut[dst] = ut;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// sipiter1 (hyperplane): forward substitution, planes m = 9 .. n3dmax.
struct SipArgs {
    const DevGrid* grids;
    const int* const* mips; const int* const* idxs;
    const double* rhs; double* res; double* phi;
    const double *c0, *c1, *c2, *c3;   // lw ls lb lpr  |  ue un ut
    int ilevel;                         // the grids of this level (<= 0: all)
};

__global__ void __launch_bounds__(512) k_sipiter1_hp(SipArgs a) {
    const DevGrid G = a.grids[blockIdx.x];
    if (a.ilevel > 0 && G.level != a.ilevel) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int* mip = a.mips[G.cls];
    const int* idx = a.idxs[G.cls];
    const long long o = G.ip3;
    const double* rhs = a.rhs + o;
    double* res = a.res + o;
    const double *lw = a.c0 + o, *ls = a.c1 + o, *lb = a.c2 + o, *lpr = a.c3 + o;
    const int kj = kk * jj;
    const int n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    // (loading the next plane's values ahead of the barrier, as sipiter2
    // does, measured slower here: 2.2 against 1.44 ms on 4096 x 24^3 grids,
    // at three and at four CTAs per SM; so did CTAs of 256 or 1024 threads,
    // 2.08 and 2.05 ms)
    for (int m = 9; m <= n3dmax; ++m) {
        const int lm = mip[m], lp = mip[m + 1] - lm;
        for (int ip = threadIdx.x; ip < lp; ip += blockDim.x) {
            const int iacc = lm + ip;
            const int id = idx[iacc];
            double r = (rhs[id] + res[id]) * lpr[iacc];
            r = r - lb[iacc] * res[id - 1] - ls[iacc] * res[id - kk] - lw[iacc] * res[id - kj];
            res[id] = r;
        }
        __syncthreads();
    }
}

// sipiter2 (hyperplane): backward substitution, then phi += res.
__global__ void __launch_bounds__(512) k_sipiter2_hp(SipArgs a) {
    const DevGrid G = a.grids[blockIdx.x];
    if (a.ilevel > 0 && G.level != a.ilevel) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int* mip = a.mips[G.cls];
    const int* idx = a.idxs[G.cls];
    const long long o = G.ip3;
    double* res = a.res + o;
    double* phi = a.phi + o;
    const double *ue = a.c0 + o, *un = a.c1 + o, *ut = a.c2 + o;
    const int kj = kk * jj;
    const int n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    // pipelined as sipiter1: the own value and coefficients of the next
    // plane's first point per thread are loaded before the barrier
    int id = 0;
    double own = 0.0, ct = 0.0, cn = 0.0, ce = 0.0;
    int lm = mip[n3dmax], lp = mip[n3dmax + 1] - lm;
    if ((int)threadIdx.x < lp) {
        const int iacc = lm + threadIdx.x;
        id = idx[iacc];
        own = res[id];
        ct = ut[iacc]; cn = un[iacc]; ce = ue[iacc];
    }
    for (int m = n3dmax; m >= 9; --m) {
        if ((int)threadIdx.x < lp)
            res[id] = own - ct * res[id + 1] - cn * res[id + kk] - ce * res[id + kj];
        for (int ip = threadIdx.x + blockDim.x; ip < lp; ip += blockDim.x) {
            const int iacc = lm + ip;
            const int jd = idx[iacc];
            double r = res[jd] - ut[iacc] * res[jd + 1] - un[iacc] * res[jd + kk] -
                       ue[iacc] * res[jd + kj];
            res[jd] = r;
        }
        if (m > 9) {
            lm = mip[m - 1];
            lp = mip[m] - lm;
            if ((int)threadIdx.x < lp) {
                const int iacc = lm + threadIdx.x;
                id = idx[iacc];
                own = res[id];
                ct = ut[iacc]; cn = un[iacc]; ce = ue[iacc];
            }
        }
        __syncthreads();
    }
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        const long long c = IX(k, j, i);
        phi[c] = phi[c] + res[c];
    }
}

// sipiter1 (classic): columns (j, i) on the diagonal i+j = d in parallel.
__global__ void k_sipiter1_cl(SipArgs a) {
    const DevGrid G = a.grids[blockIdx.x];
    if (a.ilevel > 0 && G.level != a.ilevel) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const long long o = G.ip3;
    const double* rhs = a.rhs + o;
    double* res = a.res + o;
    const double *lw = a.c0 + o, *ls = a.c1 + o, *lb = a.c2 + o, *lpr = a.c3 + o;
    for (int d = 6; d <= (ii - 2) + (jj - 2); ++d) {
        const int i0 = max(3, d - (jj - 2)), i1 = min(ii - 2, d - 3);
        for (int i = i0 + (int)threadIdx.x; i <= i1; i += blockDim.x) {
            const int j = d - i;
            for (int k = 3; k <= kk - 2; ++k) {
                const long long c = IX(k, j, i);
                double r = (rhs[c] + res[c]) * lpr[c];
                r = r - lw[c] * res[IX(k, j, i - 1)] - ls[c] * res[IX(k, j - 1, i)];
                res[c] = r;
            }
            for (int k = 3; k <= kk - 2; ++k) {
                const long long c = IX(k, j, i);
                res[c] = res[c] - lb[c] * res[IX(k - 1, j, i)];
            }
        }
        __syncthreads();
    }
}

// sipiter2 (classic)
__global__ void k_sipiter2_cl(SipArgs a) {
    const DevGrid G = a.grids[blockIdx.x];
    if (a.ilevel > 0 && G.level != a.ilevel) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const long long o = G.ip3;
    double* res = a.res + o;
    double* phi = a.phi + o;
    const double *ue = a.c0 + o, *un = a.c1 + o, *ut = a.c2 + o;
    for (int d = (ii - 2) + (jj - 2); d >= 6; --d) {
        const int i0 = max(3, d - (jj - 2)), i1 = min(ii - 2, d - 3);
        for (int i = i0 + (int)threadIdx.x; i <= i1; i += blockDim.x) {
            const int j = d - i;
            for (int k = 3; k <= kk - 2; ++k) {
                const long long c = IX(k, j, i);
                res[c] = res[c] - un[c] * res[IX(k, j + 1, i)] - ue[c] * res[IX(k, j, i + 1)];
            }
            for (int k = kk - 2; k >= 3; --k) {
                const long long c = IX(k, j, i);
                res[c] = res[c] - ut[c] * res[IX(k + 1, j, i)];
            }
        }
        __syncthreads();
    }
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        const long long c = IX(k, j, i);
        phi[c] = phi[c] + res[c];
    }
}

// relax: one red-black colour, all grids (no BP for noib).
__global__ void k_sor(const DevGrid* __restrict__ grids, int rb, double* DP,
                      const double* __restrict__ RHS, const double* __restrict__ RAP,
                      const double* __restrict__ AW, const double* __restrict__ AE,
                      const double* __restrict__ AS, const double* __restrict__ AN,
                      const double* __restrict__ AB, const double* __restrict__ AT, double omg,
                      int ilevel) {
    const DevGrid G = grids[blockIdx.y];
    if (ilevel > 0 && G.level != ilevel) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj * nk) return;
    const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
    int ks, ke;
    if ((i + j) % 2 == rb) { ks = 4; ke = kk - 2; } else { ks = 3; ke = kk - 3; }
    if (k < ks || k > ke || ((k - ks) & 1)) return;
    const long long o = G.ip3;
    double* dp = DP + o;
    const double *aw = AW + G.ipx - 1, *ae = AE + G.ipx - 1, *as = AS + G.ipy - 1,
                 *an = AN + G.ipy - 1, *ab = AB + G.ipz - 1, *at = AT + G.ipz - 1;
    const long long c = IX(k, j, i);
    double res = (aw[i] * dp[IX(k, j, i - 1)] + ae[i] * dp[IX(k, j, i + 1)] +
                  as[j] * dp[IX(k, j - 1, i)] + an[j] * dp[IX(k, j + 1, i)] +
                  ab[k] * dp[IX(k - 1, j, i)] + at[k] * dp[IX(k + 1, j, i)] - RHS[o + c]) *
                 RAP[o + c];
    dp[c] = (1.0 - omg) * dp[c] - omg * res;
}

// ---------------------------------------------------------------------------
__global__ void k_divcal(const DevGrid* __restrict__ grids, double* DIV, const double* __restrict__ U,
                         const double* __restrict__ V, const double* __restrict__ W,
                         const double* __restrict__ RDDX, const double* __restrict__ RDDY,
                         const double* __restrict__ RDDZ, double fak,
                         const double* __restrict__ SDIV, const double* __restrict__ BP) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj * nk) return;
    const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
    const long long o = G.ip3;
    const double *u = U + o, *v = V + o, *w = W + o;
    const double rddx = RDDX[G.ipx + i - 1], rddy = RDDY[G.ipy + j - 1], rddz = RDDZ[G.ipz + k - 1];
    double d = fak * ((u[IX(k, j, i)] - u[IX(k, j, i - 1)]) * rddx +
                      (v[IX(k, j, i)] - v[IX(k, j - 1, i)]) * rddy +
                      (w[IX(k, j, i)] - w[IX(k - 1, j, i)]) * rddz);
    if (SDIV) {   // ghost-cell IB: gc_mod.F90:278-347 passes sdiv and bp (noib_mod.F90:328-353)
        d = d + fak * SDIV[o + IX(k, j, i)];
        d = BP[o + IX(k, j, i)] * d;   // the ghost layers of div stay 0 = bp * 0
    }
    DIV[o + IX(k, j, i)] = d;
}

// Per grid: is BP exactly 1.0 on the box 2..n-1 in every direction (every
// point laplacephi reads)?  Then each bp factor of laplacephi is a product
// with 1.0, which rounds to the other operand, and the kernel may drop it
// with the same bits (the no-IB grids: noib_mod.F90 leaves bp at 1).
__global__ void k_bp_ones(const DevGrid* __restrict__ grids, const double* __restrict__ BP, int* ones) {
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int nk = kk - 2, nj = jj - 2, ni = ii - 2;
    const double* bp = BP + G.ip3;
    int bad = 0;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 2, j = (t / nk) % nj + 2, i = t / (nk * nj) + 2;
        bad |= !(bp[IX(k, j, i)] == 1.0);
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) ones[blockIdx.x] = !bad;
}

__global__ void k_laplacephi(const DevGrid* __restrict__ grids, int ilevel, double* RES,
                             const double* __restrict__ PHI, const double* __restrict__ AP,
                             const double* __restrict__ BP, const double* __restrict__ AW,
                             const double* __restrict__ AE, const double* __restrict__ AS,
                             const double* __restrict__ AN, const double* __restrict__ AB,
                             const double* __restrict__ AT, const int* __restrict__ bpone) {
    const DevGrid G = grids[blockIdx.y];
    if (ilevel > 0 && G.level != ilevel) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj * nk) return;
    const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
    const long long o = G.ip3;
    const double *phi = PHI + o, *bp = BP + o;
    const double aw = AW[G.ipx + i - 1], ae = AE[G.ipx + i - 1], as = AS[G.ipy + j - 1],
                 an = AN[G.ipy + j - 1], ab = AB[G.ipz + k - 1], at = AT[G.ipz + k - 1];
    if (bpone[blockIdx.y]) {
        RES[o + IX(k, j, i)] = -aw * phi[IX(k, j, i - 1)] - ae * phi[IX(k, j, i + 1)] -
                               as * phi[IX(k, j - 1, i)] - an * phi[IX(k, j + 1, i)] -
                               ab * phi[IX(k - 1, j, i)] - at * phi[IX(k + 1, j, i)] -
                               AP[o + IX(k, j, i)] * phi[IX(k, j, i)];
        return;
    }
    RES[o + IX(k, j, i)] = -aw * phi[IX(k, j, i - 1)] * bp[IX(k, j, i - 1)] * bp[IX(k, j, i)] -
                           ae * phi[IX(k, j, i + 1)] * bp[IX(k, j, i)] * bp[IX(k, j, i + 1)] -
                           as * phi[IX(k, j - 1, i)] * bp[IX(k, j - 1, i)] * bp[IX(k, j, i)] -
                           an * phi[IX(k, j + 1, i)] * bp[IX(k, j, i)] * bp[IX(k, j + 1, i)] -
                           ab * phi[IX(k - 1, j, i)] * bp[IX(k - 1, j, i)] * bp[IX(k, j, i)] -
                           at * phi[IX(k + 1, j, i)] * bp[IX(k, j, i)] * bp[IX(k + 1, j, i)] -
                           AP[o + IX(k, j, i)] * phi[IX(k, j, i)];
}

// rescal (rhs += res on the interior) fused with maxabscal_grid; with RES
// null only the maximum (after ftoc has restricted rhs into coarse grids).
__global__ void __launch_bounds__(256) k_rescal_maxabs(const DevGrid* __restrict__ grids, double* RHS,
                                                       const double* __restrict__ RES,
                                                       double* __restrict__ gridmax) {
    __shared__ double sh[32];
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const long long o = G.ip3;
    double m = 0.0;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        const long long c = o + IX(k, j, i);
        double r = RHS[c];
        if (RES) {
            r = r + RES[c];
            RHS[c] = r;
        }
        m = fmax(fabs(r), m);
    }
    m = block_max(m, sh);
    if (threadIdx.x == 0) gridmax[blockIdx.x] = m;
}

// maxabs over grids with the level scale 2^(maxlevel-level).
__global__ void k_maxabs_final(const DevGrid* __restrict__ grids, int ngrid, int maxlevel,
                               const double* __restrict__ gridmax, double* out) {
    __shared__ double sh[32];
    double m = 0.0;
    for (int g = threadIdx.x; g < ngrid; g += blockDim.x)
        if (!grids[g].halo)   // a copy of another rank's grid
            m = fmax(fabs(gridmax[g] * ldexp(1.0, maxlevel - grids[g].level)), m);
    m = block_max(m, sh);
    if (threadIdx.x == 0) out[0] = m;
}

__global__ void k_accumulate(double* __restrict__ dp, double* __restrict__ hilf, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; t < n; t += stride) {
        dp[t] = dp[t] + hilf[t];
        hilf[t] = 0.0;
    }
}

__global__ void k_mgpcorr(const DevGrid* __restrict__ grids, double* U, double* V, double* W,
                          double* P, const double* __restrict__ DP, const double* __restrict__ RDX,
                          const double* __restrict__ RDY, const double* __restrict__ RDZ,
                          double rfak, const double* __restrict__ BPF) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    const long long o = G.ip3;
    const double* dp = DP + o;
    const long long c = IX(k, j, i);
    if (BPF) {   // pressuresolver_mod.F90:808-844, the bp form (ghost-cell IB)
        const double* bp = BPF + o;
        if (i >= 2 && i <= ii - 1 && j >= 2 && j <= jj - 1 && k >= 2 && k <= kk - 1)
            P[o + c] = P[o + c] + dp[c] * bp[c];
        if (i >= 2 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2)
            U[o + c] = U[o + c] + (dp[c] - dp[IX(k, j, i + 1)]) * bp[c] * bp[IX(k, j, i + 1)] *
                                      RDX[G.ipx + i - 1] * rfak;
        if (i >= 3 && i <= ii - 2 && j >= 2 && j <= jj - 2 && k >= 3 && k <= kk - 2)
            V[o + c] = V[o + c] + (dp[c] - dp[IX(k, j + 1, i)]) * bp[c] * bp[IX(k, j + 1, i)] *
                                      RDY[G.ipy + j - 1] * rfak;
        if (i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 2 && k <= kk - 2)
            W[o + c] = W[o + c] + (dp[c] - dp[IX(k + 1, j, i)]) * bp[c] * bp[IX(k + 1, j, i)] *
                                      RDZ[G.ipz + k - 1] * rfak;
        return;
    }
    // with bp = 1 (noib) the products by bp are exact, so they are left out
    if (i >= 2 && i <= ii - 1 && j >= 2 && j <= jj - 1 && k >= 2 && k <= kk - 1)
        P[o + c] = P[o + c] + dp[c];
    if (i >= 2 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2)
        U[o + c] = U[o + c] + (dp[c] - dp[IX(k, j, i + 1)]) * RDX[G.ipx + i - 1] * rfak;
    if (i >= 3 && i <= ii - 2 && j >= 2 && j <= jj - 2 && k >= 3 && k <= kk - 2)
        V[o + c] = V[o + c] + (dp[c] - dp[IX(k, j + 1, i)]) * RDY[G.ipy + j - 1] * rfak;
    if (i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 2 && k <= kk - 2)
        W[o + c] = W[o + c] + (dp[c] - dp[IX(k + 1, j, i)]) * RDZ[G.ipz + k - 1] * rfak;
}

int interior_points_max(Ctx* c) {
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, (g.kk - 4) * (g.jj - 4) * (g.ii - 4));
    return m;
}

int box_points_max(Ctx* c) {
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    return m;
}

// device arrays of per-class table pointers (built lazily)
struct TablePtrs {
    const int** mips = nullptr;
    const int** idxs = nullptr;
};
std::map<Ctx*, TablePtrs> g_tables;

int table_ptrs(Ctx* c, TablePtrs& out) {
    auto it = g_tables.find(c);
    if (it != g_tables.end()) { out = it->second; return 0; }
    std::vector<const int*> hm, hi;
    for (const HpTable& t : c->hp) { hm.push_back(t.d_mip); hi.push_back(t.d_idx); }
    TablePtrs tp;
    MG_CUDA(cudaMalloc(&tp.mips, hm.size() * sizeof(int*)));
    MG_CUDA(cudaMalloc(&tp.idxs, hi.size() * sizeof(int*)));
    MG_CUDA(copy_on(c->stream, tp.mips, hm.data(), hm.size() * sizeof(int*), cudaMemcpyHostToDevice));
    MG_CUDA(copy_on(c->stream, tp.idxs, hi.data(), hi.size() * sizeof(int*), cudaMemcpyHostToDevice));
    g_tables[c] = tp;
    out = tp;
    return 0;
}

}  // namespace

void release_tables(Ctx* c) {
    auto it = g_tables.find(c);
    if (it == g_tables.end()) return;
    cudaFree(it->second.mips);
    cudaFree(it->second.idxs);
    g_tables.erase(it);
}

int launch_giteig(Ctx* c) {
    ProfScope ps_(c, "giteig");
    k_giteig<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, c->L("DX"), c->L("DY"), c->L("DZ"),
                                              c->L("GSAW"), c->L("GSAE"), c->L("GSAS"),
                                              c->L("GSAN"), c->L("GSAB"), c->L("GSAT"),
                                              c->F("GSAP"), c->F("BP"));
    MG_LAUNCHED(c);
    return 0;
}

static int launch_lu(Ctx* c, int planeorder) {
    TablePtrs tp;
    if (int rc = table_ptrs(c, tp)) return rc;
    const long long npt = box_points_max(c);
    const int chunk = std::max(1, std::min(c->ngrid, 512));
    double* tmp = nullptr;
    MG_CUDA(cudaMalloc(&tmp, (size_t)chunk * 7 * npt * sizeof(double)));
    LuArgs a{};
    a.grids = c->d_grids;
    a.mips = tp.mips; a.idxs = tp.idxs;
    a.mip = nullptr; a.idx = nullptr;
    a.aw = c->L("GSAW"); a.ae = c->L("GSAE"); a.as = c->L("GSAS");
    a.an = c->L("GSAN"); a.ab = c->L("GSAB"); a.at = c->L("GSAT");
    a.ap = c->F("GSAP"); a.bp = c->F("BP");
    a.lw = c->F("SIPLW"); a.ls = c->F("SIPLS"); a.lb = c->F("SIPLB"); a.lpr = c->F("SIPLPR");
    a.ue = c->F("SIPUE"); a.un = c->F("SIPUN"); a.ut = c->F("SIPUT");
    a.tmp = tmp;
    a.tmpstride = 7 * npt;
    a.planeorder = planeorder;
    int rc = 0;
    for (int g0 = 0; g0 < c->ngrid; g0 += chunk) {
        const int n = std::min(chunk, c->ngrid - g0);
        cudaMemsetAsync(tmp, 0, (size_t)n * 7 * npt * sizeof(double), c->stream);
        a.g0 = g0;
        k_sip_lu<<<n, 512, 0, c->stream>>>(a);
        c->launches++;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { rc = cuda_fail(e, "k_sip_lu"); break; }
    }
    cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    return rc;
}

int launch_sip_lu_hp(Ctx* c) {
    ProfScope ps_(c, "sip_lu_hp"); return launch_lu(c, 1); }
int launch_sip_lu_classic(Ctx* c) {
    ProfScope ps_(c, "sip_lu_classic"); return launch_lu(c, 0); }

int launch_sipiter1(Ctx* c, int ilevel, const double* rhs, double* res) {
    ProfScope ps_(c, "sipiter1");
    TablePtrs tp;
    if (int rc = table_ptrs(c, tp)) return rc;
    SipArgs a{};
    a.grids = c->d_grids; a.mips = tp.mips; a.idxs = tp.idxs;
    a.rhs = rhs; a.res = res; a.phi = nullptr;
    a.c0 = c->F("SIPLW"); a.c1 = c->F("SIPLS"); a.c2 = c->F("SIPLB"); a.c3 = c->F("SIPLPR");
    a.ilevel = ilevel;
    if (c->prm.psolver == MGLET_PSOLVER_CLASSIC)
        k_sipiter1_cl<<<c->ngrid, 32, 0, c->stream>>>(a);
    else
        k_sipiter1_hp<<<c->ngrid, 512, 0, c->stream>>>(a);
    MG_LAUNCHED(c);
    return 0;
}

int launch_sipiter2(Ctx* c, int ilevel, double* phi, double* res) {
    ProfScope ps_(c, "sipiter2");
    TablePtrs tp;
    if (int rc = table_ptrs(c, tp)) return rc;
    SipArgs a{};
    a.grids = c->d_grids; a.mips = tp.mips; a.idxs = tp.idxs;
    a.rhs = nullptr; a.res = res; a.phi = phi;
    a.c0 = c->F("SIPUE"); a.c1 = c->F("SIPUN"); a.c2 = c->F("SIPUT"); a.c3 = nullptr;
    a.ilevel = ilevel;
    if (c->prm.psolver == MGLET_PSOLVER_CLASSIC)
        k_sipiter2_cl<<<c->ngrid, 32, 0, c->stream>>>(a);
    else
        k_sipiter2_hp<<<c->ngrid, 512, 0, c->stream>>>(a);
    MG_LAUNCHED(c);
    return 0;
}

int launch_sor(Ctx* c, int ilevel, double* dp, const double* rhs) {
    ProfScope ps_(c, "sor");
    dim3 grid((interior_points_max(c) + 255) / 256, c->ngrid);
    for (int rb = 0; rb <= 1; ++rb) {
        k_sor<<<grid, 256, 0, c->stream>>>(c->d_grids, rb, dp, rhs, c->F("SOR_RAP"), c->L("GSAW"),
                                           c->L("GSAE"), c->L("GSAS"), c->L("GSAN"),
                                           c->L("GSAB"), c->L("GSAT"), c->prm.omega, ilevel);
        MG_LAUNCHED(c);
    }
    return 0;
}

int launch_divcal(Ctx* c, double* div, const double* u, const double* v, const double* w,
                  double fak) {
    ProfScope ps_(c, "divcal");
    dim3 grid((interior_points_max(c) + 255) / 256, c->ngrid);
    const bool gc = c->ibtype == 1;
    k_divcal<<<grid, 256, 0, c->stream>>>(c->d_grids, div, u, v, w, c->L("RDDX"), c->L("RDDY"),
                                          c->L("RDDZ"), fak, gc ? c->F("SDIV") : nullptr,
                                          gc ? c->F("BP") : nullptr);
    MG_LAUNCHED(c);
    return 0;
}

int launch_bp_ones(Ctx* c) {
    k_bp_ones<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, c->F("BP"), c->d_bpone);
    MG_LAUNCHED(c);
    return 0;
}

int launch_laplacephi(Ctx* c, int ilevel, double* res, const double* phi) {
    ProfScope ps_(c, "laplacephi");
    dim3 grid((interior_points_max(c) + 255) / 256, c->ngrid);
    k_laplacephi<<<grid, 256, 0, c->stream>>>(c->d_grids, ilevel, res, phi, c->F("GSAP"), c->F("BP"),
                                              c->L("GSAW"), c->L("GSAE"), c->L("GSAS"),
                                              c->L("GSAN"), c->L("GSAB"), c->L("GSAT"), c->d_bpone);
    MG_LAUNCHED(c);
    return 0;
}

int launch_rescal_maxabs(Ctx* c, double* rhs, const double* res) {
    ProfScope ps_(c, "rescal_maxabs");
    k_rescal_maxabs<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, rhs, res, c->d_gridred);
    MG_LAUNCHED(c);
    k_maxabs_final<<<1, 1024, 0, c->stream>>>(c->d_grids, c->ngrid, c->maxlevel, c->d_gridred,
                                              c->d_scalar);
    MG_LAUNCHED(c);
    return 0;
}

int launch_accumulate(Ctx* c, double* dp, double* hilf) {
    ProfScope ps_(c, "accumulate");
    long long n = c->idim3d;
    int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_accumulate<<<blocks, 256, 0, c->stream>>>(dp, hilf, n);
    MG_LAUNCHED(c);
    return 0;
}

int launch_mgpcorr(Ctx* c, double* u, double* v, double* w, double* p, const double* dp,
                   double rfak) {
    ProfScope ps_(c, "mgpcorr");
    dim3 grid((box_points_max(c) + 255) / 256, c->ngrid);
    k_mgpcorr<<<grid, 256, 0, c->stream>>>(c->d_grids, u, v, w, p, dp, c->L("RDX"), c->L("RDY"),
                                           c->L("RDZ"), rfak,
                                           c->ibtype == 1 ? c->F("BP") : nullptr);
    MG_LAUNCHED(c);
    return 0;
}

MG_PLAIN_END
}  // namespace mg
