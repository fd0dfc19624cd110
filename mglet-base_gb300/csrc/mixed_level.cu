// mixed_level.cu -- grid hierarchies in the batched mixed form.
//
// The multi-level pressure solve of mgpoisl (src/flow/pressuresolver_mod.F90:
// 160-357) runs its inner SIP iterations level by level; between the levels
// the reference moves the correction with ctof, parent and bound_pressure and
// after them restricts it with ftoc.  The mixed form keeps hilf and the
// residual in the inner solver's padded plane order (FP32 hilf, float-float
// residual), so these operators are restated here on that layout:
//
//   ctof (injection)        src/ib/ctof/ctof1_mod.F90:167-331
//   parent (scalar slab)    src/core/parent_core_mod.F90:190-255
//   bound_pressure          src/flow/bound_pressure_mod.F90:106-609 (no-BP form)
//   ftoc 'P' / 'R'          src/ib/ftoc_mod.F90:581-626,
//                           src/ib/noib_restrict_mod.F90:126-298 (volume mean)
//
// parent and bound_pressure are fused: the PAR buffer value a block of ghosts
// needs is the coarse cell the parent's slab holds, read straight from the
// coarse grid's plane-ordered hilf (its neighbour's, or its own PAR ghost
// plane, where the slab lies on the coarse grid's ghost layer).  The ghost
// values go to a per-grid ghost plane that the pre-pass and the outer step
// gather across PAR faces.  Grids with a PAR face also take their RK update
// here, after tstle4_par has corrected their fluxes.
#include <algorithm>
#include <vector>

#include "mixed_level.h"

namespace mg {
namespace {

// Plane-order geometry of the (common) grid shape
struct PlaneMap {
    const int* tpos;            // [nm][ni]: position of (io, jo) in plane m is tpos[m*ni+io] + jo
    int ni, nj, nk, npp, fs;
    __device__ __forceinline__ int pos(int io, int jo, int ko) const {
        return tpos[(io + jo + ko) * ni + io] + jo;
    }
};

__device__ __forceinline__ int fidx(const PlaneMap& m, int axis, int ko, int jo, int io) {
    return axis == 0 ? ko + jo * m.nk : (axis == 1 ? ko + io * m.nk : jo + io * m.nj);
}

// ctof: every interior point of a fine grid takes the coarse cell that holds
// it (ctof1_mod.F90's injection; i = 3 + io lies in the parent's cell
// iposition - 1 + (i - 1) / 2).
__global__ void k_mx_ctof(const DevGrid* __restrict__ grids, const int4* __restrict__ hier,
                          const int* __restrict__ list, PlaneMap m, float* H, const int* ctl) {
    if (ctl[0]) return;
    const int g = list[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.ni * m.nj * m.nk) return;
    const int ko = t % m.nk, jo = (t / m.nk) % m.nj, io = t / (m.nk * m.nj);
    const int4 h = hier[g];
    const int ioc = h.y - 4 + (io + 2) / 2, joc = h.z - 4 + (jo + 2) / 2, koc = h.w - 4 + (ko + 2) / 2;
    if (ioc < 0 || ioc >= m.ni || joc < 0 || joc >= m.nj || koc < 0 || koc >= m.nk) return;
    H[(long long)g * m.npp + m.pos(io, jo, ko)] = H[(long long)h.x * m.npp + m.pos(ioc, joc, koc)];
}

struct BpArgs {
    const DevGrid* grids;
    const int4* hier;
    const int* list;            // grids of the level with a PAR face
    const int* fnbr;            // [ngrid][6] face neighbours
    const int* facepos;         // [6][fs]
    PlaneMap m;
    const float* H;
    float* PG;                  // [ngrid][6][fs]
    const double *dx, *dy, *dz, *ddx, *ddy, *ddz;
    const double* BP;           // ghost-cell IB: the BP field (null: the no-BP form)
    const int* ctl;
};

// hilf of the parent p at its interior point (io, jo, ko), one coordinate of
// which may lie on the ghost layer (-1 or n): there the value the reference's
// coarse ghost holds -- the face neighbour's boundary plane (connect), the
// parent's own PAR ghost plane, or zero (walls, inflow, outflow).
__device__ float coarse_hilf(const BpArgs& A, int p, int io, int jo, int ko) {
    const PlaneMap& m = A.m;
    const bool xi = io < 0 || io >= m.ni, xj = jo < 0 || jo >= m.nj, xk = ko < 0 || ko >= m.nk;
    if (!xi && !xj && !xk) return A.H[(long long)p * m.npp + m.pos(io, jo, ko)];
    // one coordinate on the ghost layer, the others inside (properly nested
    // grids); anything else reads zero rather than outside the arrays
    if ((int)xi + (int)xj + (int)xk != 1 || io < -1 || io > m.ni || jo < -1 || jo > m.nj || ko < -1 ||
        ko > m.nk)
        return 0.f;
    const int axis = xi ? 0 : (xj ? 1 : 2);
    const int hi = xi ? io >= m.ni : (xj ? jo >= m.nj : ko >= m.nk);
    const int f = 2 * axis + hi;
    const int nb = A.fnbr[6 * p + f];
    if (nb >= 0) {
        // the neighbour's interior point next to the shared face
        if (axis == 0) io = hi ? 0 : m.ni - 1;
        else if (axis == 1) jo = hi ? 0 : m.nj - 1;
        else ko = hi ? 0 : m.nk - 1;
        return A.H[(long long)nb * m.npp + m.pos(io, jo, ko)];
    }
    if (A.grids[p].bc[f] == MGLET_BC_PAR) return A.PG[((long long)p * 6 + f) * m.fs + fidx(m, axis, ko, jo, io)];
    return 0.f;
}

// parent + bound_pressure of hilf for the PAR faces of one level: one thread
// per 2x2 block of a face (bound_pressure's blocks), grid = list[blockIdx.y],
// face = blockIdx.z.
__global__ void k_mx_bound_pressure(BpArgs A) {
    if (A.ctl[0]) return;
    const int g = A.list[blockIdx.y];
    const int f = blockIdx.z;
    const DevGrid G = A.grids[g];
    if (G.bc[f] != MGLET_BC_PAR) return;
    const PlaneMap& m = A.m;
    const int axis = f / 2;
    const bool lo = (f % 2) == 0;
    const int nn = axis == 0 ? G.ii : (axis == 1 ? G.jj : G.kk);
    const int n2 = lo ? 2 : nn - 1, n3 = lo ? 3 : nn - 2, n4 = lo ? 4 : nn - 3;
    const int st2 = lo ? 2 : nn - 2;
    const int nmin = n3 < n4 ? n3 : n4;
    const int na = axis == 2 ? G.jj : G.kk, nb = axis == 0 ? G.jj : G.ii;
    const int nba = (na - 4) / 2, nbb = (nb - 4) / 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nba * nbb) return;
    const int a = 3 + 2 * (q % nba), b = 3 + 2 * (q / nba);
    const double* ddx = A.ddx + G.ipx - 1;
    const double* ddy = A.ddy + G.ipy - 1;
    const double* ddz = A.ddz + G.ipz - 1;
    const double* dn = axis == 0 ? ddx : (axis == 1 ? ddy : ddz);
    const double* dstag = axis == 0 ? A.dx + G.ipx - 1 : (axis == 1 ? A.dy + G.ipy - 1 : A.dz + G.ipz - 1);
    const float* Hg = A.H + (long long)g * m.npp;
    // (a, b, n) in face coordinates -> fine interior (io, jo, ko)
    auto fine = [&](int aa, int bb, int n) -> float {
        int k, j, i;
        if (axis == 0) { k = aa; j = bb; i = n; }
        else if (axis == 1) { k = aa; j = n; i = bb; }
        else { k = n; j = aa; i = bb; }
        return Hg[m.pos(i - 3, j - 3, k - 3)];
    };
    // pressureftocone_A / _B: the (BP-weighted) volume mean of the 2x2x2
    // interior block next to the face
    int k0, j0, i0;
    if (axis == 0) { k0 = a; j0 = b; i0 = nmin; }
    else if (axis == 1) { k0 = a; j0 = nmin; i0 = b; }
    else { k0 = nmin; j0 = a; i0 = b; }
    const double* bp = A.BP ? A.BP + G.ip3 : nullptr;
    const int kk = G.kk, jj = G.jj;
    auto bix = [&](int kx, int jx, int ix) -> long long {
        return (long long)(ix - 1) * kk * jj + (long long)(jx - 1) * kk + (kx - 1);
    };
    double pc, bpc = 1.0;
    if (!bp) {
        double sump = 0.0, sumvol = 0.0;
        for (int l = 0; l <= 1; ++l)
            for (int mm = 0; mm <= 1; ++mm)
                for (int n = 0; n <= 1; ++n) {
                    const double vol = ddz[k0 + n] * ddy[j0 + mm] * ddx[i0 + l];
                    sump = sump + (double)Hg[m.pos(i0 + l - 3, j0 + mm - 3, k0 + n - 3)] * vol;
                    sumvol = sumvol + vol;
                }
        pc = sump / sumvol;
    } else {
        double sumbp = 0.0;
        for (int l = 0; l <= 1; ++l)
            for (int mm = 0; mm <= 1; ++mm)
                for (int n = 0; n <= 1; ++n) sumbp = sumbp + bp[bix(k0 + n, j0 + mm, i0 + l)];
        bpc = fmin(sumbp, 1.0);
        pc = 0.0;
        if (bpc >= 0.5) {
            double sump = 0.0, sumvol = 0.0;
            for (int l = 0; l <= 1; ++l)
                for (int mm = 0; mm <= 1; ++mm)
                    for (int n = 0; n <= 1; ++n) {
                        const double vol = bp[bix(k0 + n, j0 + mm, i0 + l)] * ddz[k0 + n] * ddy[j0 + mm] *
                                           ddx[i0 + l];
                        sump = sump + (double)Hg[m.pos(i0 + l - 3, j0 + mm - 3, k0 + n - 3)] * vol;
                        sumvol = sumvol + vol;
                    }
            pc = sump / sumvol;
        }
    }
    // the parent's slab cell of this block (parent_core_mod.F90:190-255 for a
    // scalar: both block corners odd, so the slab value itself)
    const int4 h = A.hier[g];
    const int p = h.x;
    int is = h.y - 2, js = h.z - 2, ks = h.w - 2;
    if (f == 0) is = h.y - 1;
    else if (f == 1) is = h.y + (G.ii - 4) / 2;
    else if (f == 2) js = h.z - 1;
    else if (f == 3) js = h.z + (G.jj - 4) / 2;
    else if (f == 4) ks = h.w - 1;
    else ks = h.w + (G.kk - 4) / 2;
    const int jc = 2 + (a - 1) / 2, ic = 2 + (b - 1) / 2;
    int kc, jcc, icc;
    if (axis == 0) { kc = ks + jc - 1; jcc = js + ic - 1; icc = is; }
    else if (axis == 1) { kc = ks + jc - 1; jcc = js; icc = is + ic - 1; }
    else { kc = ks; jcc = js + jc - 1; icc = is + ic - 1; }
    const double pbv = (double)coarse_hilf(A, p, icc - 3, jcc - 3, kc - 3);
    double fak = 1.0;
    if (bp) {
        // bound_pressure's open-area factor of the block's four face pairs
        const double* da = axis == 2 ? ddy : ddz;
        const double* db = axis == 0 ? ddy : ddx;
        auto fp = [&](int aa, int bb, int n) -> long long {
            if (axis == 0) return bix(aa, bb, n);
            if (axis == 1) return bix(aa, n, bb);
            return bix(n, aa, bb);
        };
        if (bpc < 0.5) pc = pbv;
        const double s11 = bp[fp(a, b, n2)] * bp[fp(a, b, n3)];
        const double s12 = bp[fp(a, b + 1, n2)] * bp[fp(a, b + 1, n3)];
        const double s13 = bp[fp(a + 1, b, n2)] * bp[fp(a + 1, b, n3)];
        const double s14 = bp[fp(a + 1, b + 1, n2)] * bp[fp(a + 1, b + 1, n3)];
        fak = (s11 * db[b] * da[a] + s12 * db[b + 1] * da[a] + s13 * db[b] * da[a + 1] +
               s14 * db[b + 1] * da[a + 1]) /
              ((db[b] + db[b + 1]) * (da[a] + da[a + 1]));
        if (fak < (double)0.1f) fak = 1.0;
        fak = 1.0 / fak;
    }
    const double fac = fak * dstag[st2] / (dn[n3] + dn[n2]);
    float* pg = A.PG + ((long long)g * 6 + f) * m.fs;
    for (int l = 0; l <= 1; ++l)
        for (int n = 0; n <= 1; ++n) {
            const double v = (double)fine(a + n, b + l, n3) + fac * (pbv - pc);
            int ko, jo, io;
            if (axis == 0) { ko = a + n - 3; jo = b + l - 3; io = 0; }
            else if (axis == 1) { ko = a + n - 3; jo = 0; io = b + l - 3; }
            else { ko = 0; jo = a + n - 3; io = b + l - 3; }
            pg[fidx(m, axis, ko, jo, io)] = (float)v;
        }
}

// ftoc of a cell-centred field from the fine grids of one level into their
// parents: the volume mean of each 2x2x2 block (noib_restrict 'P', also the
// 'R' of the residual).  LO null: FP32 H; else the float-float pair (H, LO).
// With BP (ghost-cell IB) the forms of gc_restrict_mod.F90: restrict_p, the
// mean over the open cells (hilf), and restrict_r, the BP-weighted sum over
// the block volume (the residual).
__global__ void k_mx_ftoc(const DevGrid* __restrict__ grids, const int4* __restrict__ hier,
                          const int* __restrict__ list, PlaneMap m, float* H, float* LO,
                          const double* __restrict__ DDX, const double* __restrict__ DDY,
                          const double* __restrict__ DDZ, const double* __restrict__ BP,
                          const int* ctl) {
    if (ctl[0]) return;
    const int g = list[blockIdx.y];
    const DevGrid G = grids[g];
    const int nci = m.ni / 2, ncj = m.nj / 2, nck = m.nk / 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nci * ncj * nck) return;
    const int k = 3 + 2 * (q % nck), j = 3 + 2 * ((q / nck) % ncj), i = 3 + 2 * (q / (nck * ncj));
    const double* ddx = DDX + G.ipx - 1;
    const double* ddy = DDY + G.ipy - 1;
    const double* ddz = DDZ + G.ipz - 1;
    const long long base = (long long)g * m.npp;
    auto F = [&](int kx, int jx, int ix) -> double {
        const long long o = base + m.pos(ix - 3, jx - 3, kx - 3);
        return LO ? (double)H[o] + (double)LO[o] : (double)H[o];
    };
    double val;
    if (!LO) {
        // the FP32 correction: its mean in FP32 (the FP64 units of this part
        // issue at a small fraction of the FP32 rate)
        auto Ff = [&](int kx, int jx, int ix) -> float { return H[base + m.pos(ix - 3, jx - 3, kx - 3)]; };
        const float zx[2] = {(float)ddx[i], (float)ddx[i + 1]}, zy[2] = {(float)ddy[j], (float)ddy[j + 1]};
        const float zz[2] = {(float)ddz[k], (float)ddz[k + 1]};
        const double* bp = BP ? BP + G.ip3 : nullptr;
        const int kk = G.kk, jj = G.jj;
        float spv = 0.f, sv = 0.f;
        for (int l = 0; l < 2; ++l)
            for (int mq = 0; mq < 2; ++mq)
                for (int n = 0; n < 2; ++n) {
                    float vol = zz[l] * zy[mq] * zx[n];
                    if (bp)
                        vol *= (float)bp[(long long)(i + n - 1) * kk * jj + (long long)(j + mq - 1) * kk + (k + l - 1)];
                    spv += Ff(k + l, j + mq, i + n) * vol;
                    sv += vol;
                }
        const float hv = sv > 0.f ? spv / sv : 0.f;
        const int4 h = hier[g];
        const int ioc = h.y + (i - 3) / 2 - 3, joc = h.z + (j - 3) / 2 - 3, koc = h.w + (k - 3) / 2 - 3;
        if (ioc < 0 || ioc >= m.ni || joc < 0 || joc >= m.nj || koc < 0 || koc >= m.nk) return;
        H[(long long)h.x * m.npp + m.pos(ioc, joc, koc)] = hv;
        return;
    }
    if (!BP) {
        const double s = F(k, j, i) * ddz[k] * ddy[j] * ddx[i] + F(k, j, i + 1) * ddz[k] * ddy[j] * ddx[i + 1] +
                         F(k, j + 1, i) * ddz[k] * ddy[j + 1] * ddx[i] +
                         F(k, j + 1, i + 1) * ddz[k] * ddy[j + 1] * ddx[i + 1] +
                         F(k + 1, j, i) * ddz[k + 1] * ddy[j] * ddx[i] +
                         F(k + 1, j, i + 1) * ddz[k + 1] * ddy[j] * ddx[i + 1] +
                         F(k + 1, j + 1, i) * ddz[k + 1] * ddy[j + 1] * ddx[i] +
                         F(k + 1, j + 1, i + 1) * ddz[k + 1] * ddy[j + 1] * ddx[i + 1];
        val = s / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
    } else {
        const int kk = G.kk, jj = G.jj;
        const double* bp = BP + G.ip3;
        auto B = [&](int kx, int jx, int ix) -> double {
            return bp[(long long)(ix - 1) * kk * jj + (long long)(jx - 1) * kk + (kx - 1)];
        };
        const int cj[4] = {j, j, j + 1, j + 1}, ci[4] = {i, i + 1, i, i + 1};
        double spv = 0.0, sv = 0.0;
        for (int l = 0; l < 2; ++l)
            for (int q4 = 0; q4 < 4; ++q4) {
                const int kq = k + l;
                const double vol = B(kq, cj[q4], ci[q4]) * ddz[kq] * ddy[cj[q4]] * ddx[ci[q4]];
                spv = spv + F(kq, cj[q4], ci[q4]) * vol;
                sv = sv + vol;
            }
        if (LO)   // restrict_r
            val = spv / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
        else      // restrict_p
            val = sv > 0.0 ? spv / sv : 0.0;
    }
    const int4 h = hier[g];
    const int ioc = h.y + (i - 3) / 2 - 3, joc = h.z + (j - 3) / 2 - 3, koc = h.w + (k - 3) / 2 - 3;
    if (ioc < 0 || ioc >= m.ni || joc < 0 || joc >= m.nj || koc < 0 || koc >= m.nk) return;
    const long long o = (long long)h.x * m.npp + m.pos(ioc, joc, koc);
    const float hv = (float)val;
    H[o] = hv;
    if (LO) LO[o] = (float)(val - (double)hv);
}

// max |rhs| per grid (maxabscal_grid after the restriction of the residual
// into the coarse grids), of its leading float as the outer step forms it
__global__ void k_mx_gridmax(int npp, const float* __restrict__ H, double* gridmax, const int* ctl) {
    if (ctl[0]) return;
    __shared__ float sh[32];
    const long long base = (long long)blockIdx.x * npp;
    float v = 0.f;
    for (int q = threadIdx.x; q < npp; q += blockDim.x) v = fmaxf(fabsf(H[base + q]), v);
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) gridmax[blockIdx.x] = (double)v;
    }
}

// Per grid: do the transported point values PWU, PWV, PWW differ from U, V,
// W anywhere on the box 2..n-1 the flux kernel reads (ghost-cell IB)?  Such
// grids take the FP64 tstle4 of the point values and the separate RK update.
__global__ void k_mx_pwflag(const DevGrid* __restrict__ grids, const double* __restrict__ U,
                            const double* __restrict__ V, const double* __restrict__ W,
                            const double* __restrict__ PU, const double* __restrict__ PV,
                            const double* __restrict__ PW, unsigned char* flag) {
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int nk = kk - 2, nj = jj - 2, ni = ii - 2;
    int d = 0;
    for (int t = threadIdx.x; t < nk * nj * ni; t += blockDim.x) {
        const int k = t % nk + 2, j = (t / nk) % nj + 2, i = t / (nk * nj) + 2;
        const long long c = G.ip3 + (long long)(i - 1) * kk * jj + (long long)(j - 1) * kk + (k - 1);
        d |= (U[c] != PU[c]) | (V[c] != PV[c]) | (W[c] != PW[c]);
    }
    d = __syncthreads_or(d);
    if (threadIdx.x == 0) flag[blockIdx.x] = d ? 1 : 0;
}

// rkstep (rungekutta_mod.F90:315-333) over the whole box of the grids whose
// fluxes came from UO, VO, WO -- a PAR face (tstle4_par corrected them) or a
// flag in sel (FP64 fluxes of the point values) -- in the mixed form's
// arithmetic (FP32 register, FP64 field); UO.. are cleared for the next
// stage, as tstle4 starts from zero fluxes.
__global__ void k_mx_rk_par(const DevGrid* __restrict__ grids, const unsigned char* __restrict__ sel,
                            double* U, double* V, double* W, float* DU, float* DV, float* DW,
                            double* UO, double* VO, double* WO, const double* __restrict__ sprm) {
    const DevGrid G = grids[blockIdx.y];
    bool par = false;
    for (int f = 0; f < 6; ++f) par |= G.bc[f] == MGLET_BC_PAR;
    if (!par && !(sel && sel[blockIdx.y])) return;
    const long long n = (long long)G.kk * G.jj * G.ii;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const long long c = G.ip3 + t;
    const float frhs = (float)sprm[0], fdt = (float)sprm[1];
    const float du = frhs * DU[c] + (float)UO[c];
    const float dv = frhs * DV[c] + (float)VO[c];
    const float dw = frhs * DW[c] + (float)WO[c];
    DU[c] = du; DV[c] = dv; DW[c] = dw;
    U[c] = U[c] + (double)(fdt * du);
    V[c] = V[c] + (double)(fdt * dv);
    W[c] = W[c] + (double)(fdt * dw);
    UO[c] = 0.0; VO[c] = 0.0; WO[c] = 0.0;
}

PlaneMap plane_map(const SipState& st) {
    return PlaneMap{st.d_tpos, st.ni, st.nj, st.nk, st.npp, st.fs};
}

int upload(Ctx* c, const std::vector<int>& h, int** d) {
    if (h.empty()) return 0;
    MG_CUDA(cudaMalloc(d, h.size() * sizeof(int)));
    MG_CUDA(copy_on(c->stream, *d, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
    return 0;
}

}  // namespace

int mx_level_prepare(Ctx* c, SipState& st, LevelState& lv) {
    if (lv.ready) return 0;
    const int nl = c->maxlevel - c->minlevel + 1;
    lv.grids.assign(nl, {});
    lv.pars.assign(nl, {});
    lv.d_grids.assign(nl, nullptr);
    lv.d_pars.assign(nl, nullptr);
    bool anypar = false;
    for (int g = 0; g < c->ngrid; ++g) {
        const DevGrid& G = c->grids[g];
        const int l = G.level - c->minlevel;
        lv.grids[l].push_back(g);
        bool par = false;
        for (int f = 0; f < 6; ++f) par |= G.bc[f] == MGLET_BC_PAR;
        if (par) {
            lv.pars[l].push_back(g);
            anypar = true;
            if (c->hier.empty() || c->hier[g].x < 0) {
                set_error("mixed form: a grid with a PAR face has no parent");
                return MGLET_ERR_ARG;
            }
        }
        if (par) lv.parall.push_back(g);
        if (l > 0 && (c->hier.empty() || c->hier[g].x < 0)) {
            set_error("mixed form: a fine grid without parent (mglet_gpu_set_hierarchy first)");
            return MGLET_ERR_ARG;
        }
    }
    for (int l = 0; l < nl; ++l) {
        if (int rc = upload(c, lv.grids[l], &lv.d_grids[l])) return rc;
        if (int rc = upload(c, lv.pars[l], &lv.d_pars[l])) return rc;
    }
    if (int rc = upload(c, lv.parall, &lv.d_parall)) return rc;
    if (!lv.ibflag.empty()) {
        // ghost-cell IB: per-grid flags, set at every stage by k_mx_pwflag
        MG_CUDA(cudaMalloc(&lv.d_skip, (size_t)c->ngrid));
        MG_CUDA(zero_on(c->stream, lv.d_skip, (size_t)c->ngrid));
    }
    if (anypar && !st.pg) {
        const size_t n = (size_t)c->ngrid * 6 * st.fs * sizeof(float);
        MG_CUDA(cudaMalloc(&st.pg, n));
        MG_CUDA(zero_on(c->stream, st.pg, n));
    }
    // UO, VO, WO start at zero: the flux kernel writes their interior for
    // the grids with PAR faces, tstle4_par adds, k_mx_rk_par clears them
    for (const char* nm : {"UO", "VO", "WO"})
        MG_CUDA(zero_on(c->stream, c->F(nm), (size_t)c->idim3d * sizeof(double)));
    // the level operators' boundary buffers and the per-level connect
    // plans of the stage, built before any capture
    for (const char* nm : {"U", "V", "W", "P", "DP"})
        if (!field_buffer(c, nm)) return cuda_fail(cudaErrorMemoryAllocation, "mixed level buffers");
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        const ConnectPlan* pl;
        if (int rc = get_plan(c, l, 1, 7, false, true, 1, &pl)) return rc;
        if (int rc = get_plan(c, l, 2, 15, true, false, 0, &pl)) return rc;
    }
    lv.ready = true;
    return 0;
}

void mx_level_release(LevelState& lv) {
    for (int* p : lv.d_grids) cudaFree(p);
    for (int* p : lv.d_pars) cudaFree(p);
    cudaFree(lv.d_parall);
    cudaFree(lv.d_skip);
    lv = LevelState();
}

int mx_ctof(Ctx* c, SipState& st, const LevelState& lv, int ilevel, const int* ctl) {
    const int l = ilevel - c->minlevel;
    if (l <= 0 || lv.grids[l].empty()) return 0;
    ProfScope ps_(c, "mx_ctof");
    const dim3 grid((st.ni * st.nj * st.nk + 255) / 256, (unsigned)lv.grids[l].size());
    k_mx_ctof<<<grid, 256, 0, c->stream>>>(c->d_grids, c->d_hier, lv.d_grids[l], plane_map(st),
                                           st.h32, ctl);
    MG_LAUNCHED(c);
    return 0;
}

int mx_bound_pressure(Ctx* c, SipState& st, const LevelState& lv, int ilevel, const int* ctl) {
    const int l = ilevel - c->minlevel;
    if (lv.pars[l].empty()) return 0;
    ProfScope ps_(c, "mx_bound_pressure");
    BpArgs A{};
    A.grids = c->d_grids;
    A.hier = c->d_hier;
    A.list = lv.d_pars[l];
    A.fnbr = st.d_fnbr;
    A.facepos = st.d_facepos;
    A.m = plane_map(st);
    A.H = st.h32;
    A.PG = st.pg;
    A.dx = c->L("DX"); A.dy = c->L("DY"); A.dz = c->L("DZ");
    A.ddx = c->L("DDX"); A.ddy = c->L("DDY"); A.ddz = c->L("DDZ");
    A.BP = c->ibtype == 1 ? c->F("BP") : nullptr;
    A.ctl = ctl;
    const int nbmax = std::max(st.nk * st.nj, std::max(st.nk * st.ni, st.nj * st.ni)) / 4;
    const dim3 grid((nbmax + 127) / 128, (unsigned)lv.pars[l].size(), 6);
    k_mx_bound_pressure<<<grid, 128, 0, c->stream>>>(A);
    MG_LAUNCHED(c);
    return 0;
}

int mx_ftoc(Ctx* c, SipState& st, const LevelState& lv, int ilevel, bool rhs, const int* ctl) {
    const int l = ilevel - c->minlevel;
    if (l <= 0 || lv.grids[l].empty()) return 0;
    ProfScope ps_(c, "mx_ftoc");
    const int nq = (st.ni / 2) * (st.nj / 2) * (st.nk / 2);
    const dim3 grid((nq + 127) / 128, (unsigned)lv.grids[l].size());
    k_mx_ftoc<<<grid, 128, 0, c->stream>>>(c->d_grids, c->d_hier, lv.d_grids[l], plane_map(st),
                                           rhs ? st.rhs32 : st.h32, rhs ? st.rhsl : nullptr,
                                           c->L("DDX"), c->L("DDY"), c->L("DDZ"),
                                           c->ibtype == 1 ? c->F("BP") : nullptr, ctl);
    MG_LAUNCHED(c);
    return 0;
}

int mx_gridmax(Ctx* c, SipState& st, const int* ctl) {
    ProfScope ps_(c, "mx_gridmax");
    k_mx_gridmax<<<c->ngrid, 256, 0, c->stream>>>(st.npp, st.rhs32, c->d_gridred, ctl);
    MG_LAUNCHED(c);
    return 0;
}

int mx_rk_par(Ctx* c, const LevelState& lv, float* du, float* dv, float* dw, const double* sprm) {
    if (lv.parall.empty()) return 0;
    ProfScope ps_(c, "mx_rk_par");
    long long npts = 0;
    for (const DevGrid& G : c->grids) npts = std::max(npts, (long long)G.kk * G.jj * G.ii);
    const dim3 grid((unsigned)((npts + 255) / 256), (unsigned)c->ngrid);
    k_mx_rk_par<<<grid, 256, 0, c->stream>>>(c->d_grids, nullptr, c->F("U"), c->F("V"), c->F("W"),
                                             du, dv, dw, c->F("UO"), c->F("VO"), c->F("WO"), sprm);
    MG_LAUNCHED(c);
    return 0;
}

int mx_pw_flags(Ctx* c, const LevelState& lv) {
    if (!lv.d_skip) return 0;
    ProfScope ps_(c, "mx_pwflag");
    k_mx_pwflag<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, c->F("U"), c->F("V"), c->F("W"), c->F("PWU"),
                                                  c->F("PWV"), c->F("PWW"), lv.d_skip);
    MG_LAUNCHED(c);
    return 0;
}

}  // namespace mg
