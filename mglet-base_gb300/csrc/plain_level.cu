// plain_level.cu -- the inter-level operators of a grid hierarchy, FP64.
//
// parent (src/ib/parent/parent1_mod.F90 with parent_core_mod.F90): the PAR
// face buffers of fine grids prolonged from their parents' boundary slabs;
// the PAR branch of bound_flow (src/flow/bound_flow_mod.F90:139-256,
// 377-494, 613-730); bound_pressure (src/flow/bound_pressure_mod.F90:106-609);
// ftoc with the no-IB restriction (src/ib/ftoc_mod.F90:581-626,
// src/ib/noib_restrict_mod.F90:126-298); ctof (src/ib/ctof/ctof1_mod.F90:
// 167-331).  On one GPU the reference's MPI messages become direct reads of
// the other grid's slab; every fine grid, face and point is independent,
// except that the faces of one grid run in order 1..6 (bound_flow edges).
// Compiled without FMA contraction: every value matches the CPU
// restatement bit for bit.
#include <algorithm>
#include <cstring>
#include <limits>
#include <vector>

#include "internal.h"

namespace mg {
namespace {

// default-kind literal 0.1 of the PAR branches, as a REAL64 build widens it
constexpr float kPoint1f = 0.1f;

struct FaceIx {
    int axis, kk, jj;
    __device__ long long at(int a, int b, int n) const {
        int k, j, i;
        if (axis == 0) { k = a; j = b; i = n; }
        else if (axis == 1) { k = a; j = n; i = b; }
        else { k = n; j = a; i = b; }
        return (long long)(i - 1) * kk * jj + (long long)(j - 1) * kk + (k - 1);
    }
};

// ---- PAR branch of bound_flow -------------------------------------------
struct ParArgs {
    const DevGrid* grids;
    const int* list;            // grids with a PAR face iface
    const BFace* bface;
    const double *ub, *vb, *wb, *bp;
    const double *ddx, *ddy, *ddz;
    double *u, *v, *w;
    int iface, ilevel;
};

// One thread per tangential position (a, b): the tangential components, and
// at odd a, b >= 3 also the 2x2 block of face-normal fine faces.  The two
// loops of the reference touch disjoint elements, so they share a launch.
__global__ void k_bound_par(ParArgs A) {
    const int g = A.list[blockIdx.y];
    const DevGrid G = A.grids[g];
    if (A.ilevel && G.level != A.ilevel) return;
    const int axis = (A.iface - 1) / 2;
    const bool lo = (A.iface % 2) == 1;
    const int nn = axis == 0 ? G.ii : (axis == 1 ? G.jj : G.kk);
    const int n2 = lo ? 2 : nn - 1, n3 = lo ? 3 : nn - 2, n4 = lo ? 4 : nn - 3;
    const int st2 = lo ? 2 : nn - 2;
    const int na = axis == 2 ? G.jj : G.kk, nb = axis == 0 ? G.jj : G.ii;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= na * nb) return;
    const int a = q % na + 1, b = q / na + 1;
    const FaceIx F{axis, G.kk, G.jj};
    const long long o = G.ip3;
    double *u = A.u + o, *v = A.v + o, *w = A.w + o;
    const double* bp = A.bp + o;
    const long long bo = A.bface[6 * g + A.iface - 1].off;
    const double *ub = A.ub + bo, *vb = A.vb + bo, *wb = A.wb + bo;
    const double* da = (axis == 2 ? A.ddy + G.ipy : A.ddz + G.ipz) - 1;   // 1-based
    const double* db = (axis == 0 ? A.ddy + G.ipy : A.ddx + G.ipx) - 1;
    double* vn = axis == 0 ? u : (axis == 1 ? v : w);
    const double* bn = axis == 0 ? ub : (axis == 1 ? vb : wb);
    double* t1 = axis == 0 ? v : u;
    double* t2 = axis == 2 ? v : w;
    const double* b1 = axis == 0 ? vb : ub;
    const double* b2 = axis == 2 ? vb : wb;
    auto bi = [&](int x, int y) -> long long { return (long long)(x - 1) + (long long)(y - 1) * na; };
    if (a >= 2 && a <= na - 1 && b >= 2 && b <= nb - 1) {
        const double s1 = bp[F.at(a, b, n2)] * bp[F.at(a, b + 1, n2)];
        const double s2 = bp[F.at(a, b, n2)] * bp[F.at(a + 1, b, n2)];
        t1[F.at(a, b, n2)] = (b1[bi(a, b)] - 0.5 * (t1[F.at(a, b, n3)] - t1[F.at(a, b, n4)])) * s1 +
                             (1.0 - s1) * t1[F.at(a, b, n2)];
        // the y faces take this slope from the ghost plane (bright)
        const double slope2 = axis == 1 ? (t2[F.at(a, b, n2)] - t2[F.at(a, b, n4)])
                                        : (t2[F.at(a, b, n3)] - t2[F.at(a, b, n4)]);
        t2[F.at(a, b, n2)] = (b2[bi(a, b)] - 0.5 * slope2) * s2 + (1.0 - s2) * t2[F.at(a, b, n2)];
    }
    if (a < 3 || a > na - 2 || b < 3 || b > nb - 2 || ((a - 3) & 1) || ((b - 3) & 1)) return;
    const double sbn = bp[F.at(a, b, n2)];
    const int fa[4] = {a, a, a + 1, a + 1}, fb[4] = {b, b + 1, b, b + 1};
    double sb[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = fa[k], y = fb[k];
        if (sbn > 0.5)
            sb[k] = bp[F.at(x, y, n2)] * bp[F.at(x, y, n3)];
        else
            sb[k] = fmin(bp[F.at(x, y, n3)] + bp[F.at(x, y, n2)] + bp[F.at(x, y, n4)] +
                             bp[F.at(x, y - 1, n3)] + bp[F.at(x, y + 1, n3)] + bp[F.at(x - 1, y, n3)] +
                             bp[F.at(x + 1, y, n3)],
                         1.0);
    }
    // x faces multiply by the b spacing first, y and z faces by the a spacing
    const double area = axis == 0 ? (db[b] + db[b + 1]) * (da[a] + da[a + 1])
                                  : (da[a] + da[a + 1]) * (db[b] + db[b + 1]);
    double fak;
    if (axis == 0)
        fak = 1.0 / area * (sb[0] * db[b] * da[a] + sb[1] * db[b + 1] * da[a] + sb[2] * db[b] * da[a + 1] +
                            sb[3] * db[b + 1] * da[a + 1]);
    else
        fak = 1.0 / area * (sb[0] * da[a] * db[b] + sb[1] * da[a] * db[b + 1] + sb[2] * da[a + 1] * db[b] +
                            sb[3] * da[a + 1] * db[b + 1]);
    if (fak < (double)kPoint1f) fak = 1.0;
    fak = 1.0 / fak;
    double fv[4], f[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        fv[k] = vn[F.at(fa[k], fb[k], st2)];
        const double x = fv[k] * (1.0 - sb[k]);
        f[k] = axis == 0 ? x * db[fb[k]] * da[fa[k]] : x * da[fa[k]] * db[fb[k]];
    }
    const double fine = (f[0] + f[1] + f[2] + f[3]) / area;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        vn[F.at(fa[k], fb[k], st2)] =
            (bn[bi(fa[k], fb[k])] - fine) * fak * sb[k] + (1.0 - sb[k]) * fv[k] * sbn;
}

// ---- parent: prolongation into PAR face buffers --------------------------
struct ParentArgs {
    const DevGrid* grids;
    const int4* hier;
    const int* list;            // grids of the level with a PAR face iface
    const BFace* bface;
    const double* fc[6];        // coarse fields of the slots
    double* buf[6];             // their boundary buffers
    int comp[6];                // 1..3 vector component (staggered along x/y/z), 0 scalar
    int iface;
};

// One thread per element (j, i) of the fine face buffer (jj2d x ii2d):
// prolong2 of prolong1 of the parent's slab, evaluated in place.
__global__ void k_parent(ParentArgs A) {
    const int g = A.list[blockIdx.y];
    const int slot = blockIdx.z;
    const DevGrid G = A.grids[g];
    const int4 H = A.hier[g];
    const DevGrid P = A.grids[H.x];
    const int iface = A.iface, comp = A.comp[slot];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    int jj2d, ii2d, st1 = 0, st2 = 0;
    if (iface <= 2) { ii2d = jj; jj2d = kk; }
    else if (iface <= 4) { ii2d = ii; jj2d = kk; }
    else { ii2d = ii; jj2d = jj; }
    if (iface <= 2) { st2 = comp == 2; st1 = comp == 3; }
    else if (iface <= 4) { st2 = comp == 1; st1 = comp == 3; }
    else { st2 = comp == 1; st1 = comp == 2; }
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= jj2d * ii2d) return;
    const int j = q % jj2d + 1, i = q / jj2d + 1;
    // the parent slab (parent_core_mod.F90:190-255)
    int icomp = 0;
    if ((iface == 1 || iface == 2) && comp == 1) icomp = 1;
    if ((iface == 3 || iface == 4) && comp == 2) icomp = 2;
    if ((iface == 5 || iface == 6) && comp == 3) icomp = 3;
    const int ipos = H.y, jpos = H.z, kpos = H.w;
    int is = ipos - 2, js = jpos - 2, ks = kpos - 2;
    if (iface == 1) is = ipos - 1;
    else if (iface == 2) is = ipos + (ii - 4) / 2 - (icomp == 1 ? 1 : 0);
    else if (iface == 3) js = jpos - 1;
    else if (iface == 4) js = jpos + (jj - 4) / 2 - (icomp == 2 ? 1 : 0);
    else if (iface == 5) ks = kpos - 1;
    else ks = kpos + (kk - 4) / 2 - (icomp == 3 ? 1 : 0);
    const double* fc = A.fc[slot] + P.ip3;
    // in(jc, ic): slab element with first index jc, second ic (1-based)
    auto in = [&](int jc, int ic) -> double {
        int kc, jcc, icc;
        if (iface <= 2) { kc = ks + jc - 1; jcc = js + ic - 1; icc = is; }
        else if (iface <= 4) { kc = ks + jc - 1; jcc = js; icc = is + ic - 1; }
        else { kc = ks; jcc = js + jc - 1; icc = is + ic - 1; }
        return fc[(long long)(icc - 1) * P.kk * P.jj + (long long)(jcc - 1) * P.kk + (kc - 1)];
    };
    // prolong1 value tmp(j, ic)
    auto tmp = [&](int ic) -> double {
        if (j & 1) {
            const int jc = 2 + (j - 1) / 2;
            const double x = in(jc, ic);
            return st1 ? 0.5 * (x + in(jc - 1, ic)) : x;
        }
        return in(2 + (j - 2) / 2, ic);
    };
    double out;
    if (i & 1) {
        const int ic = 2 + (i - 1) / 2;
        const double x = tmp(ic);
        out = st2 ? 0.5 * (x + tmp(ic - 1)) : x;
    } else {
        out = tmp(2 + (i - 2) / 2);
    }
    A.buf[slot][A.bface[6 * g + iface - 1].off + (long long)(j - 1) + (long long)(i - 1) * jj2d] = out;
}

// ---- bound_pressure -------------------------------------------------------
struct BpArgs {
    const DevGrid* grids;
    const int* list;
    const BFace* bface;
    const double* buf;
    const double* bp;           // null: the no-BP forms
    const double *ddx, *ddy, *ddz, *dx, *dy, *dz;
    double* p;
    int iface, ilevel;
};

// One thread per 2x2 block of the face (bfront/bright/bbottom and _bp)
__global__ void k_bound_pressure(BpArgs A) {
    const int g = A.list[blockIdx.y];
    const DevGrid G = A.grids[g];
    if (G.level != A.ilevel) return;
    const int axis = (A.iface - 1) / 2;
    const bool lo = (A.iface % 2) == 1;
    const int nn = axis == 0 ? G.ii : (axis == 1 ? G.jj : G.kk);
    const int n2 = lo ? 2 : nn - 1, n3 = lo ? 3 : nn - 2, n4 = lo ? 4 : nn - 3;
    const int st2 = lo ? 2 : nn - 2;
    const int nmin = n3 < n4 ? n3 : n4;
    const int na = axis == 2 ? G.jj : G.kk, nb = axis == 0 ? G.jj : G.ii;
    const int nba = (na - 4) / 2, nbb = (nb - 4) / 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nba * nbb) return;
    const int a = 3 + 2 * (q % nba), b = 3 + 2 * (q / nba);
    const FaceIx F{axis, G.kk, G.jj};
    const long long o = G.ip3;
    double* p = A.p + o;
    const double* bp = A.bp ? A.bp + o : nullptr;
    const double* ddx = A.ddx + G.ipx - 1;
    const double* ddy = A.ddy + G.ipy - 1;
    const double* ddz = A.ddz + G.ipz - 1;
    const double* dn = axis == 0 ? ddx : (axis == 1 ? ddy : ddz);
    const double* dstag = axis == 0 ? A.dx + G.ipx - 1 : (axis == 1 ? A.dy + G.ipy - 1 : A.dz + G.ipz - 1);
    const double* da = axis == 2 ? ddy : ddz;
    const double* db = axis == 0 ? ddy : ddx;
    const double pbv = A.buf[A.bface[6 * g + A.iface - 1].off + (long long)(a - 1) + (long long)(b - 1) * na];
    int k, j, i;
    if (axis == 0) { k = a; j = b; i = nmin; }
    else if (axis == 1) { k = a; j = nmin; i = b; }
    else { k = nmin; j = a; i = b; }
    const int kk = G.kk, jj = G.jj;
    auto ix = [&](int kx, int jx, int ix_) -> long long {
        return (long long)(ix_ - 1) * kk * jj + (long long)(jx - 1) * kk + (kx - 1);
    };
    // pressureftocone_A / _B
    double pc, bpc;
    if (!bp) {
        bpc = 1.0;
        double sump = 0.0, sumvol = 0.0;
        for (int l = 0; l <= 1; ++l)
            for (int m = 0; m <= 1; ++m)
                for (int n = 0; n <= 1; ++n) {
                    const double vol = ddz[k + n] * ddy[j + m] * ddx[i + l];
                    sump = sump + p[ix(k + n, j + m, i + l)] * vol;
                    sumvol = sumvol + vol;
                }
        pc = sump / sumvol;
    } else {
        double sumbp = 0.0;
        for (int l = 0; l <= 1; ++l)
            for (int m = 0; m <= 1; ++m)
                for (int n = 0; n <= 1; ++n) sumbp = sumbp + bp[ix(k + n, j + m, i + l)];
        bpc = fmin(sumbp, 1.0);
        if (bpc < 0.5) {
            pc = 0.0;
        } else {
            double sump = 0.0, sumvol = 0.0;
            for (int l = 0; l <= 1; ++l)
                for (int m = 0; m <= 1; ++m)
                    for (int n = 0; n <= 1; ++n) {
                        const double vol = bp[ix(k + n, j + m, i + l)] * ddz[k + n] * ddy[j + m] * ddx[i + l];
                        sump = sump + p[ix(k + n, j + m, i + l)] * vol;
                        sumvol = sumvol + vol;
                    }
            pc = sump / sumvol;
        }
    }
    double fak = 1.0;
    if (bp) {
        if (bpc < 0.5) pc = pbv;
        const double s11 = bp[F.at(a, b, n2)] * bp[F.at(a, b, n3)];
        const double s12 = bp[F.at(a, b + 1, n2)] * bp[F.at(a, b + 1, n3)];
        const double s13 = bp[F.at(a + 1, b, n2)] * bp[F.at(a + 1, b, n3)];
        const double s14 = bp[F.at(a + 1, b + 1, n2)] * bp[F.at(a + 1, b + 1, n3)];
        fak = (s11 * db[b] * da[a] + s12 * db[b + 1] * da[a] + s13 * db[b] * da[a + 1] + s14 * db[b + 1] * da[a + 1]) /
              ((db[b] + db[b + 1]) * (da[a] + da[a + 1]));
        if (fak < (double)kPoint1f) fak = 1.0;
        fak = 1.0 / fak;
    }
    // the block's four ghost values all read the interior plane, which
    // this launch does not write
    for (int l = 0; l <= 1; ++l)
        for (int n = 0; n <= 1; ++n) {
            const long long dst = F.at(a + n, b + l, n2), src = F.at(a + n, b + l, n3);
            if (bp)
                p[dst] = p[src] + fak * dstag[st2] / (dn[n3] + dn[n2]) * (pbv - pc);
            else
                p[dst] = p[src] + dstag[st2] / (dn[n3] + dn[n2]) * (pbv - pc);
        }
}

// ---- ftoc (no-IB restriction) ---------------------------------------------
struct FtocArgs {
    const DevGrid* grids;
    const int4* hier;
    const int* list;            // fine grids of the level
    const double* ff;
    double* fc;
    const double *ddx, *ddy, *ddz;
    const double* bp;
    // per grid: the faces (bit 2a low, 2a+1 high along axis a) whose coarse
    // faces a later sibling restricts too; the later grid's value stands
    const int* skip;
    // U V W, P for the scalar (volume) mean, G and H for the ghost-cell
    // forms of P and R
    char flag;
};

__global__ void k_ftoc(FtocArgs A) {
    const int g = A.list[blockIdx.y];
    const DevGrid G = A.grids[g];
    const int4 H = A.hier[g];
    const DevGrid P = A.grids[H.x];
    const char f = A.flag;
    const double* bp = A.bp + G.ip3;
    const int is = f == 'U' ? 2 : 3, js = f == 'V' ? 2 : 3, ks = f == 'W' ? 2 : 3;
    const int ie = G.ii - is, je = G.jj - js, ke = G.kk - ks;
    const int ni = (ie - is) / 2 + 1, nj = (je - js) / 2 + 1, nk = (ke - ks) / 2 + 1;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ni * nj * nk) return;
    const int k = ks + 2 * (q % nk), j = js + 2 * ((q / nk) % nj), i = is + 2 * (q / (nk * nj));
    // a staggered face two siblings share is written once, by the later
    // grid, as the reference's grid-ordered unpack leaves it
    const int sk = A.skip[g];
    if ((f == 'U' && ((i == is && (sk & 1)) || (i == ie && (sk & 2)))) ||
        (f == 'V' && ((j == js && (sk & 4)) || (j == je && (sk & 8)))) ||
        (f == 'W' && ((k == ks && (sk & 16)) || (k == ke && (sk & 32)))))
        return;
    const int kk = G.kk, jj = G.jj;
    const double* fv = A.ff + G.ip3;
    const double* ddx = A.ddx + G.ipx - 1;
    const double* ddy = A.ddy + G.ipy - 1;
    const double* ddz = A.ddz + G.ipz - 1;
    auto F = [&](int kx, int jx, int ix) -> double {
        return fv[(long long)(ix - 1) * kk * jj + (long long)(jx - 1) * kk + (kx - 1)];
    };
    double val;
    if (f == 'U') {
        const double s = F(k, j, i) * ddy[j] * ddz[k] + F(k, j + 1, i) * ddy[j + 1] * ddz[k] +
                         F(k + 1, j, i) * ddy[j] * ddz[k + 1] + F(k + 1, j + 1, i) * ddy[j + 1] * ddz[k + 1];
        val = s / ((ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
    } else if (f == 'V') {
        const double s = F(k, j, i) * ddx[i] * ddz[k] + F(k, j, i + 1) * ddx[i + 1] * ddz[k] +
                         F(k + 1, j, i) * ddx[i] * ddz[k + 1] + F(k + 1, j, i + 1) * ddx[i + 1] * ddz[k + 1];
        val = s / ((ddx[i] + ddx[i + 1]) * (ddz[k] + ddz[k + 1]));
    } else if (f == 'W') {
        const double s = F(k, j, i) * ddx[i] * ddy[j] + F(k, j, i + 1) * ddx[i + 1] * ddy[j] +
                         F(k, j + 1, i) * ddx[i] * ddy[j + 1] + F(k, j + 1, i + 1) * ddx[i + 1] * ddy[j + 1];
        val = s / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]));
    } else if (f == 'G' || f == 'H') {
        // gc_restrict_mod.F90:59-171 restrict_p (G) and :174-259 restrict_r (H)
        const int cj[4] = {j, j, j + 1, j + 1}, ci[4] = {i, i + 1, i, i + 1};
        auto B = [&](int kx, int jx, int ix) -> double {
            return bp[(long long)(ix - 1) * kk * jj + (long long)(jx - 1) * kk + (kx - 1)];
        };
        double spv = 0.0, sv = 0.0;
        bool first = true;
        for (int l = 0; l < 2; ++l)
            for (int m = 0; m < 4; ++m) {
                const int kq = k + l;
                double pv, vol = 0.0;
                if (f == 'G') {
                    vol = B(kq, cj[m], ci[m]) * ddz[kq] * ddy[cj[m]] * ddx[ci[m]];
                    pv = F(kq, cj[m], ci[m]) * vol;
                } else {
                    pv = F(kq, cj[m], ci[m]) * B(kq, cj[m], ci[m]) * ddz[kq] * ddy[cj[m]] * ddx[ci[m]];
                }
                spv = first ? pv : spv + pv;
                sv = first ? vol : sv + vol;
                first = false;
            }
        if (f == 'G')
            val = sv > 0.0 ? spv / sv : 0.0;
        else
            val = spv / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
    } else {
        const double s = F(k, j, i) * ddz[k] * ddy[j] * ddx[i] + F(k, j, i + 1) * ddz[k] * ddy[j] * ddx[i + 1] +
                         F(k, j + 1, i) * ddz[k] * ddy[j + 1] * ddx[i] +
                         F(k, j + 1, i + 1) * ddz[k] * ddy[j + 1] * ddx[i + 1] +
                         F(k + 1, j, i) * ddz[k + 1] * ddy[j] * ddx[i] +
                         F(k + 1, j, i + 1) * ddz[k + 1] * ddy[j] * ddx[i + 1] +
                         F(k + 1, j + 1, i) * ddz[k + 1] * ddy[j + 1] * ddx[i] +
                         F(k + 1, j + 1, i + 1) * ddz[k + 1] * ddy[j + 1] * ddx[i + 1];
        val = s / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
    }
    const int ic0 = f == 'U', jc0 = f == 'V', kc0 = f == 'W';
    const int ic = H.y + (i - 3 + ic0) / 2 - ic0;
    const int jc = H.z + (j - 3 + jc0) / 2 - jc0;
    const int kc = H.w + (k - 3 + kc0) / 2 - kc0;
    A.fc[P.ip3 + (long long)(ic - 1) * P.kk * P.jj + (long long)(jc - 1) * P.kk + (kc - 1)] = val;
}

// ---- ctof (injection) -----------------------------------------------------
__global__ void k_ctof(const DevGrid* __restrict__ grids, const int4* __restrict__ hier,
                       const int* __restrict__ list, double* ff, const double* __restrict__ fc) {
    const int g = list[blockIdx.y];
    const DevGrid G = grids[g];
    const int4 H = hier[g];
    const DevGrid P = grids[H.x];
    const long long n = (long long)G.kk * G.jj * G.ii;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int k = (int)(q % G.kk) + 1, j = (int)((q / G.kk) % G.jj) + 1, i = (int)(q / ((long long)G.kk * G.jj)) + 1;
    const int ic = H.y - 1 + (i - 1) / 2, jc = H.z - 1 + (j - 1) / 2, kc = H.w - 1 + (k - 1) / 2;
    ff[G.ip3 + q] = fc[P.ip3 + (long long)(ic - 1) * P.kk * P.jj + (long long)(jc - 1) * P.kk + (kc - 1)];
}


// ---- tstle4_par (tstle4_mod.F90:532-1753) --------------------------------
// One CTA per grid with a PAR face, the reference's blocks in its order
// (upwind front, back, right, left, bottom, top; then the momentum-
// conserving fluxes back, front, top, bottom, left, right), each block's
// loop nests spread over the threads and closed by __syncthreads.  The
// work arrays of one block are two planes in shared memory: S the standard
// flux (the reference's wc*(..., i+-1) plane), N the flux of the coarse
// velocities and its interpolation (the wc*(..., i) plane).
struct ParFluxArgs {
    const DevGrid* grids;
    const int* list;
    double *uo, *vo, *wo;
    const double *u, *v, *w, *ut, *vt, *wt;
    const double *dx, *dy, *dz, *ddx, *ddy, *ddz, *rdx, *rdy, *rdz, *rddx, *rddy, *rddz;
};

// a flattened loop over a in [alo, ahi] step sa (outer) and b in [blo, bhi]
// step sb (inner), then the block barrier
#define PAR_LOOP2(a, alo, ahi, sa, b, blo, bhi, sb, ...)                                       \
    {                                                                                           \
        const int na_ = (ahi) >= (alo) ? ((ahi) - (alo)) / (sa) + 1 : 0;                        \
        const int nb_ = (bhi) >= (blo) ? ((bhi) - (blo)) / (sb) + 1 : 0;                        \
        for (int q_ = threadIdx.x; q_ < na_ * nb_; q_ += blockDim.x) {                          \
            const int a = (alo) + (q_ / nb_) * (sa);                                            \
            const int b = (blo) + (q_ % nb_) * (sb);                                            \
            __VA_ARGS__                                                                         \
        }                                                                                       \
        __syncthreads();                                                                        \
    }

__global__ void k_tstle4_par(ParFluxArgs A) {
    extern __shared__ double psm2[];
    const int g = A.list[blockIdx.x];
    const DevGrid G = A.grids[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int nfro = G.bc[0], nbac = G.bc[1], nrgt = G.bc[2], nlft = G.bc[3], nbot = G.bc[4],
              ntop = G.bc[5];
    const long long o = G.ip3;
    double *uo = A.uo + o, *vo = A.vo + o, *wo = A.wo + o;
    const double *u = A.u + o, *v = A.v + o, *w = A.w + o;
    const double *ut = A.ut + o, *vt = A.vt + o, *wt = A.wt + o;
    const double *dx = A.dx + G.ipx - 1, *dy = A.dy + G.ipy - 1, *dz = A.dz + G.ipz - 1;
    const double *ddx = A.ddx + G.ipx - 1, *ddy = A.ddy + G.ipy - 1, *ddz = A.ddz + G.ipz - 1;
    const double *rdx = A.rdx + G.ipx - 1, *rdy = A.rdy + G.ipy - 1, *rdz = A.rdz + G.ipz - 1;
    const double *rddx = A.rddx + G.ipx - 1, *rddy = A.rddy + G.ipy - 1, *rddz = A.rddz + G.ipz - 1;
    const int pl = max(kk * jj, max(kk * ii, jj * ii));
    double* S = psm2;
    double* N = psm2 + pl;
    const double wkon = 1.0;
    auto X = [&](int k, int j, int i) -> long long {
        return (long long)(i - 1) * kk * jj + (long long)(j - 1) * kk + (k - 1);
    };
#define F3(a, k, j, i) a[X(k, j, i)]
    // planes: x faces (k, j), z faces (j, i), y faces (k, i)
    auto PX = [&](int k, int j) { return (k - 1) + (j - 1) * kk; };
    auto PZ = [&](int j, int i) { return (j - 1) + (i - 1) * jj; };
    auto PY = [&](int k, int i) { return (k - 1) + (i - 1) * kk; };

    // ---- upwind in the second-to-last layer
    if (nfro == 8) {
        const int i = 4;
        PAR_LOOP2(j, 3, jj - 2, 1, k, 3, kk - 2, 1, {
            const double dyj = dy[j], ddyj = ddy[j];
            const double fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            const double fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            const double dzk = dz[k], rdzk = rdz[k], ddzk = ddz[k], rddzk = rddz[k];
            const double avx = dyj * ddzk, awx = ddyj * dzk;
            const double fvw = avx * (F3(ut, k, j, i - 1) + F3(ut, k, j + 1, i - 1)) * 0.5;
            const double qv = 0.5 * (fvw - fabs(fvw)) *
                              (0.5 * F3(v, k, j, i) - 1.5 * F3(v, k, j, i - 1) + F3(v, k, j, i - 2)) * 0.5 * 0.5;
            F3(vo, k, j, i) = F3(vo, k, j, i) + fkdtv * rddzk * (-qv);
            F3(vo, k, j, i - 1) = F3(vo, k, j, i - 1) + fkdtv * rddzk * (+qv);
            const double fww = awx * (F3(ut, k, j, i - 1) + F3(ut, k + 1, j, i - 1)) * 0.5;
            const double qw = 0.5 * (fww - fabs(fww)) *
                              (0.5 * F3(w, k, j, i) - 1.5 * F3(w, k, j, i - 1) + F3(w, k, j, i - 2)) * 0.5 * 0.5;
            F3(wo, k, j, i) = F3(wo, k, j, i) + fkdtw * rdzk * (-qw);
            F3(wo, k, j, i - 1) = F3(wo, k, j, i - 1) + fkdtw * rdzk * (+qw);
        })
    }
    if (nbac == 8) {
        const int i = ii - 2;
        PAR_LOOP2(j, 3, jj - 2, 1, k, 3, kk - 2, 1, {
            const double dyj = dy[j], ddyj = ddy[j];
            const double fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            const double fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            const double dzk = dz[k], rdzk = rdz[k], ddzk = ddz[k], rddzk = rddz[k];
            const double avx = dyj * ddzk, awx = ddyj * dzk;
            const double fvw = avx * (F3(ut, k, j, i - 1) + F3(ut, k, j + 1, i - 1)) * 0.5;
            const double qv = 0.5 * (fvw + fabs(fvw)) *
                              (0.5 * F3(v, k, j, i - 1) - 1.5 * F3(v, k, j, i) + F3(v, k, j, i + 1)) * 0.5 * 0.5;
            F3(vo, k, j, i) = F3(vo, k, j, i) + fkdtv * rddzk * (-qv);
            F3(vo, k, j, i - 1) = F3(vo, k, j, i - 1) + fkdtv * rddzk * (+qv);
            const double fww = awx * (F3(ut, k, j, i - 1) + F3(ut, k + 1, j, i - 1)) * 0.5;
            const double qw = 0.5 * (fww + fabs(fww)) *
                              (0.5 * F3(w, k, j, i - 1) - 1.5 * F3(w, k, j, i) + F3(w, k, j, i + 1)) * 0.5 * 0.5;
            F3(wo, k, j, i) = F3(wo, k, j, i) + fkdtw * rdzk * (-qw);
            F3(wo, k, j, i - 1) = F3(wo, k, j, i - 1) + fkdtw * rdzk * (+qw);
        })
    }
    if (nrgt == 8 || nlft == 8) {
        for (int side = 0; side < 2; ++side) {
            const bool lft = side == 1;
            if ((lft ? nlft : nrgt) != 8) continue;
            const int j = lft ? jj - 2 : 4;
            PAR_LOOP2(i, 3, ii - 2, 1, k, 3, kk - 2, 1, {
                const double dxi = dx[i], ddxi = ddx[i];
                const double fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
                const double fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
                const double dzk = dz[k], rdzk = rdz[k], ddzk = ddz[k], rddzk = rddz[k];
                const double auy = dxi * ddzk, awy = ddxi * dzk;
                const double fus = auy * (F3(vt, k, j - 1, i) + F3(vt, k, j - 1, i + 1)) * 0.5;
                const double qu = lft ? 0.5 * (fus + fabs(fus)) *
                                            (0.5 * F3(u, k, j - 1, i) - 1.5 * F3(u, k, j, i) + F3(u, k, j + 1, i)) * 0.5 * 0.5
                                      : 0.5 * (fus - fabs(fus)) *
                                            (0.5 * F3(u, k, j, i) - 1.5 * F3(u, k, j - 1, i) + F3(u, k, j - 2, i)) * 0.5 * 0.5;
                F3(uo, k, j, i) = F3(uo, k, j, i) + fkdtu * rddzk * (-qu);
                F3(uo, k, j - 1, i) = F3(uo, k, j - 1, i) + fkdtu * rddzk * (+qu);
                const double fws = awy * (F3(vt, k, j - 1, i) + F3(vt, k + 1, j - 1, i)) * 0.5;
                const double qw = lft ? 0.5 * (fws + fabs(fws)) *
                                            (0.5 * F3(w, k, j - 1, i) - 1.5 * F3(w, k, j, i) + F3(w, k, j + 1, i)) * 0.5 * 0.5
                                      : 0.5 * (fws - fabs(fws)) *
                                            (0.5 * F3(w, k, j, i) - 1.5 * F3(w, k, j - 1, i) + F3(w, k, j - 2, i)) * 0.5 * 0.5;
                F3(wo, k, j, i) = F3(wo, k, j, i) + fkdtw * rdzk * (-qw);
                F3(wo, k, j - 1, i) = F3(wo, k, j - 1, i) + fkdtw * rdzk * (+qw);
            })
        }
    }
    for (int side = 0; side < 2; ++side) {
        const bool top = side == 1;
        if ((top ? ntop : nbot) != 8) continue;
        const int k = top ? kk - 2 : 4;
        PAR_LOOP2(i, 3, ii - 2, 1, j, 3, jj - 2, 1, {
            const double dxi = dx[i], ddxi = ddx[i];
            const double fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            const double fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            const double dyj = dy[j], ddyj = ddy[j];
            const double auz = dxi * ddyj, avz = ddxi * dyj;
            const double rddzk = rddz[k];
            const double fub = auz * (F3(wt, k - 1, j, i) + F3(wt, k - 1, j, i + 1)) * 0.5;
            const double qu = top ? 0.5 * (fub + fabs(fub)) *
                                        (0.5 * F3(u, k - 1, j, i) - 1.5 * F3(u, k, j, i) + F3(u, k + 1, j, i)) * 0.5 * 0.5
                                  : 0.5 * (fub - fabs(fub)) *
                                        (0.5 * F3(u, k, j, i) - 1.5 * F3(u, k - 1, j, i) + F3(u, k - 2, j, i)) * 0.5 * 0.5;
            F3(uo, k, j, i) = F3(uo, k, j, i) + fkdtu * rddzk * (-qu);
            F3(uo, k - 1, j, i) = F3(uo, k - 1, j, i) + fkdtu * rddzk * (+qu);
            const double fvb = avz * (F3(wt, k - 1, j, i) + F3(wt, k - 1, j + 1, i)) * 0.5;
            const double qv = top ? 0.5 * (fvb + fabs(fvb)) *
                                        (0.5 * F3(v, k - 1, j, i) - 1.5 * F3(v, k, j, i) + F3(v, k + 1, j, i)) * 0.5 * 0.5
                                  : 0.5 * (fvb - fabs(fvb)) *
                                        (0.5 * F3(v, k, j, i) - 1.5 * F3(v, k - 1, j, i) + F3(v, k - 2, j, i)) * 0.5 * 0.5;
            F3(vo, k, j, i) = F3(vo, k, j, i) + fkdtv * rddzk * (-qv);
            F3(vo, k - 1, j, i) = F3(vo, k - 1, j, i) + fkdtv * rddzk * (+qv);
        })
    }

    // ---- BACK and FRONT (x faces): w cell, then v cell; e = +1 back
    for (int side = 0; side < 2; ++side) {
        const bool back = side == 0;
        if ((back ? nbac : nfro) != 8) continue;
        const int i = back ? ii - 2 : 3;
        const int it = back ? i : i - 1;          // ut plane
        const int iw = back ? i + 1 : i - 1;      // the other w/v plane of the flux
        // w cell
        PAR_LOOP2(j, 3, jj - 2, 1, k, 2, kk - 2, 1, {
            const double awx = ddy[j] * dz[k];
            const double f = awx * (F3(ut, k, j, it) + F3(ut, k + 1, j, it)) * 0.5;
            S[PX(k, j)] = 0.5 * f * (F3(w, k, j, i) + F3(w, k, j, iw));
        })
        PAR_LOOP2(j, 3, jj - 2, 2, k, 2, kk - 2, 2, {
            const double awx = ddy[j] * dz[k];
            double f;
            if (k == 2)
                f = awx * (2 * F3(ut, k, j, it) + 2 * F3(ut, k, j + 1, it) + F3(ut, k + 1, j, it) +
                           F3(ut, k + 1, j + 1, it) + F3(ut, k + 2, j, it) + F3(ut, k + 2, j + 1, it)) * 0.125;
            else if (k == kk - 2)
                f = awx * (F3(ut, k - 1, j, it) + F3(ut, k - 1, j + 1, it) + F3(ut, k, j, it) + F3(ut, k, j + 1, it) +
                           2 * F3(ut, k + 1, j, it) + 2 * F3(ut, k + 1, j + 1, it)) * 0.125;
            else
                f = awx * (F3(ut, k - 1, j, it) + F3(ut, k - 1, j + 1, it) + F3(ut, k, j, it) + F3(ut, k, j + 1, it) +
                           F3(ut, k + 1, j, it) + F3(ut, k + 1, j + 1, it) + F3(ut, k + 2, j, it) +
                           F3(ut, k + 2, j + 1, it)) * 0.125;
            N[PX(k, j)] = 0.5 * f * (F3(w, k, j, i) + F3(w, k, j, iw));
            N[PX(k, j + 1)] = 0.5 * f * (F3(w, k, j + 1, i) + F3(w, k, j + 1, iw));
        })
        PAR_LOOP2(j, 3, jj - 2, 1, k, 2, kk - 4, 2, { N[PX(k + 1, j)] = 0.5 * (N[PX(k, j)] + N[PX(k + 2, j)]); })
        PAR_LOOP2(j, 3, jj - 2, 1, k, 2, kk - 2, 1, {
            const double fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            const double rdzk = rdz[k];
            if (back)
                F3(wo, k, j, i) = F3(wo, k, j, i) + fkdtw * rdzk * (-S[PX(k, j)] + N[PX(k, j)]);
            else
                F3(wo, k, j, i) = F3(wo, k, j, i) + fkdtw * rdzk * (S[PX(k, j)] - N[PX(k, j)]);
        })
        // v cell
        PAR_LOOP2(j, 2, jj - 2, 1, k, 3, kk - 2, 1, {
            const double avx = ddz[k] * dy[j];
            const double f = avx * (F3(ut, k, j, it) + F3(ut, k, j + 1, it)) * 0.5;
            S[PX(k, j)] = 0.5 * f * (F3(v, k, j, i) + F3(v, k, j, iw));
        })
        PAR_LOOP2(j, 2, jj - 2, 2, k, 3, kk - 2, 2, {
            const double avx = ddz[k] * dy[j];
            double f;
            if (j == 2)
                f = avx * (2 * F3(ut, k, j, it) + 2 * F3(ut, k + 1, j, it) + F3(ut, k, j + 1, it) +
                           F3(ut, k + 1, j + 1, it) + F3(ut, k, j + 2, it) + F3(ut, k + 1, j + 2, it)) * 0.125;
            else if (j == jj - 2)
                f = avx * (F3(ut, k, j - 1, it) + F3(ut, k + 1, j - 1, it) + F3(ut, k, j, it) + F3(ut, k + 1, j, it) +
                           2 * F3(ut, k, j + 1, it) + 2 * F3(ut, k + 1, j + 1, it)) * 0.125;
            else
                f = avx * (F3(ut, k, j - 1, it) + F3(ut, k + 1, j - 1, it) + F3(ut, k, j, it) + F3(ut, k + 1, j, it) +
                           F3(ut, k, j + 1, it) + F3(ut, k + 1, j + 1, it) + F3(ut, k, j + 2, it) +
                           F3(ut, k + 1, j + 2, it)) * 0.125;
            N[PX(k, j)] = 0.5 * f * (F3(v, k, j, i) + F3(v, k, j, iw));
            N[PX(k + 1, j)] = 0.5 * f * (F3(v, k + 1, j, i) + F3(v, k + 1, j, iw));
        })
        PAR_LOOP2(j, 2, jj - 4, 2, k, 3, kk - 2, 1, { N[PX(k, j + 1)] = 0.5 * (N[PX(k, j)] + N[PX(k, j + 2)]); })
        PAR_LOOP2(j, 2, jj - 2, 1, k, 3, kk - 2, 1, {
            const double fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            const double rddzk = rddz[k];
            if (back)
                F3(vo, k, j, i) = F3(vo, k, j, i) + fkdtv * rddzk * (N[PX(k, j)] - S[PX(k, j)]);
            else
                F3(vo, k, j, i) = F3(vo, k, j, i) + fkdtv * rddzk * (-N[PX(k, j)] + S[PX(k, j)]);
        })
    }

    // ---- TOP and BOTTOM (z faces): u cell, then v cell
    for (int side = 0; side < 2; ++side) {
        const bool top = side == 0;
        if ((top ? ntop : nbot) != 8) continue;
        const int k = top ? kk - 2 : 3;
        const int kw = top ? k : k - 1;
        const int kn = top ? k + 1 : k - 1;
        PAR_LOOP2(i, 2, ii - 2, 1, j, 3, jj - 2, 1, {
            const double auz = dx[i] * ddy[j];
            const double f = auz * (F3(wt, kw, j, i) + F3(wt, kw, j, i + 1)) * 0.5;
            S[PZ(j, i)] = 0.5 * f * (F3(u, k, j, i) + F3(u, kn, j, i));
        })
        PAR_LOOP2(i, 2, ii - 2, 2, j, 3, jj - 2, 2, {
            const double auz = dx[i] * ddy[j];
            double f;
            if (i == 2)
                f = auz * (2 * F3(wt, kw, j, i) + 2 * F3(wt, kw, j + 1, i) + F3(wt, kw, j, i + 1) +
                           F3(wt, kw, j + 1, i + 1) + F3(wt, kw, j, i + 2) + F3(wt, kw, j + 1, i + 2)) * 0.125;
            else if (i == ii - 2)
                f = auz * (F3(wt, kw, j, i - 1) + F3(wt, kw, j + 1, i - 1) + F3(wt, kw, j, i) + F3(wt, kw, j + 1, i) +
                           2 * F3(wt, kw, j, i + 1) + 2 * F3(wt, kw, j + 1, i + 1)) * 0.125;
            else
                f = auz * (F3(wt, kw, j, i - 1) + F3(wt, kw, j + 1, i - 1) + F3(wt, kw, j, i) + F3(wt, kw, j + 1, i) +
                           F3(wt, kw, j, i + 1) + F3(wt, kw, j + 1, i + 1) + F3(wt, kw, j, i + 2) +
                           F3(wt, kw, j + 1, i + 2)) * 0.125;
            N[PZ(j, i)] = 0.5 * f * (F3(u, k, j, i) + F3(u, kn, j, i));
            N[PZ(j + 1, i)] = 0.5 * f * (F3(u, k, j + 1, i) + F3(u, kn, j + 1, i));
        })
        PAR_LOOP2(i, 2, ii - 4, 2, j, 3, jj - 2, 1, { N[PZ(j, i + 1)] = 0.5 * (N[PZ(j, i)] + N[PZ(j, i + 2)]); })
        PAR_LOOP2(i, 2, ii - 2, 1, j, 3, jj - 2, 1, {
            const double fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            const double rddzk = rddz[k];
            if (top)
                F3(uo, k, j, i) = F3(uo, k, j, i) + fkdtu * rddzk * (N[PZ(j, i)] - S[PZ(j, i)]);
            else
                F3(uo, k, j, i) = F3(uo, k, j, i) + fkdtu * rddzk * (-N[PZ(j, i)] + S[PZ(j, i)]);
        })
        PAR_LOOP2(i, 3, ii - 2, 1, j, 2, jj - 2, 1, {
            const double avz = ddx[i] * dy[j];
            const double f = avz * (F3(wt, kw, j, i) + F3(wt, kw, j + 1, i)) * 0.5;
            S[PZ(j, i)] = 0.5 * f * (F3(v, k, j, i) + F3(v, kn, j, i));
        })
        PAR_LOOP2(i, 3, ii - 2, 2, j, 2, jj - 2, 2, {
            const double avz = ddx[i] * dy[j];
            double f;
            if (j == 2)
                f = avz * (2 * F3(wt, kw, j, i) + 2 * F3(wt, kw, j, i + 1) + F3(wt, kw, j + 1, i) +
                           F3(wt, kw, j + 1, i + 1) + F3(wt, kw, j + 2, i) + F3(wt, kw, j + 2, i + 1)) * 0.125;
            else if (j == jj - 2)
                f = avz * (F3(wt, kw, j - 1, i) + F3(wt, kw, j - 1, i + 1) + F3(wt, kw, j, i) + F3(wt, kw, j, i + 1) +
                           2 * F3(wt, kw, j + 1, i) + 2 * F3(wt, kw, j + 1, i + 1)) * 0.125;
            else
                f = avz * (F3(wt, kw, j - 1, i) + F3(wt, kw, j - 1, i + 1) + F3(wt, kw, j, i) + F3(wt, kw, j, i + 1) +
                           F3(wt, kw, j + 1, i) + F3(wt, kw, j + 1, i + 1) + F3(wt, kw, j + 2, i) +
                           F3(wt, kw, j + 2, i + 1)) * 0.125;
            N[PZ(j, i)] = 0.5 * f * (F3(v, k, j, i) + F3(v, kn, j, i));
            N[PZ(j, i + 1)] = 0.5 * f * (F3(v, k, j, i + 1) + F3(v, kn, j, i + 1));
        })
        PAR_LOOP2(i, 3, ii - 2, 1, j, 2, jj - 4, 2, { N[PZ(j + 1, i)] = 0.5 * (N[PZ(j, i)] + N[PZ(j + 2, i)]); })
        PAR_LOOP2(i, 3, ii - 2, 1, j, 2, jj - 2, 1, {
            const double fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            const double rddzk = rddz[k];
            if (top)
                F3(vo, k, j, i) = F3(vo, k, j, i) + fkdtv * rddzk * (N[PZ(j, i)] - S[PZ(j, i)]);
            else
                F3(vo, k, j, i) = F3(vo, k, j, i) + fkdtv * rddzk * (-N[PZ(j, i)] + S[PZ(j, i)]);
        })
    }

    // ---- LEFT and RIGHT (y faces): u cell, then w cell
    for (int side = 0; side < 2; ++side) {
        const bool left = side == 0;
        if ((left ? nlft : nrgt) != 8) continue;
        const int j = left ? jj - 2 : 3;
        const int jv = left ? j : j - 1;
        const int jn = left ? j + 1 : j - 1;
        PAR_LOOP2(i, 2, ii - 2, 1, k, 3, kk - 2, 1, {
            const double auy = dx[i] * ddz[k];
            const double f = auy * (F3(vt, k, jv, i) + F3(vt, k, jv, i + 1)) * 0.5;
            S[PY(k, i)] = 0.5 * f * (F3(u, k, j, i) + F3(u, k, jn, i));
        })
        PAR_LOOP2(i, 2, ii - 2, 2, k, 3, kk - 2, 2, {
            const double auy = dx[i] * ddz[k];
            double f;
            if (i == 2)
                f = auy * (2 * F3(vt, k, jv, i) + 2 * F3(vt, k + 1, jv, i) + F3(vt, k, jv, i + 1) +
                           F3(vt, k + 1, jv, i + 1) + F3(vt, k, jv, i + 2) + F3(vt, k + 1, jv, i + 2)) * 0.125;
            else if (i == ii - 2)
                f = auy * (F3(vt, k, jv, i - 1) + F3(vt, k + 1, jv, i - 1) + F3(vt, k, jv, i) + F3(vt, k + 1, jv, i) +
                           2 * F3(vt, k, jv, i + 1) + 2 * F3(vt, k + 1, jv, i + 1)) * 0.125;
            else
                f = auy * (F3(vt, k, jv, i - 1) + F3(vt, k + 1, jv, i - 1) + F3(vt, k, jv, i) + F3(vt, k + 1, jv, i) +
                           F3(vt, k, jv, i + 1) + F3(vt, k + 1, jv, i + 1) + F3(vt, k, jv, i + 2) +
                           F3(vt, k + 1, jv, i + 2)) * 0.125;
            N[PY(k, i)] = 0.5 * f * (F3(u, k, j, i) + F3(u, k, jn, i));
            N[PY(k + 1, i)] = 0.5 * f * (F3(u, k + 1, j, i) + F3(u, k + 1, jn, i));
        })
        PAR_LOOP2(i, 2, ii - 4, 2, k, 3, kk - 2, 1, { N[PY(k, i + 1)] = 0.5 * (N[PY(k, i)] + N[PY(k, i + 2)]); })
        PAR_LOOP2(i, 2, ii - 2, 1, k, 3, kk - 2, 1, {
            const double fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            const double rddzk = rddz[k];
            if (left)
                F3(uo, k, j, i) = F3(uo, k, j, i) + fkdtu * rddzk * (N[PY(k, i)] - S[PY(k, i)]);
            else
                F3(uo, k, j, i) = F3(uo, k, j, i) + fkdtu * rddzk * (-N[PY(k, i)] + S[PY(k, i)]);
        })
        PAR_LOOP2(i, 3, ii - 2, 1, k, 2, kk - 2, 1, {
            const double awy = ddx[i] * dz[k];
            const double f = awy * (F3(vt, k, jv, i) + F3(vt, k + 1, jv, i)) * 0.5;
            S[PY(k, i)] = 0.5 * f * (F3(w, k, j, i) + F3(w, k, jn, i));
        })
        // the reference runs the interior k loop with step 1; its odd k
        // entries are overwritten by the interpolation below, so step 2 is
        // the same result
        PAR_LOOP2(i, 3, ii - 2, 2, k, 2, kk - 2, 2, {
            const double awy = ddx[i] * dz[k];
            double f;
            if (k == 2)
                f = awy * (2 * F3(vt, k, jv, i) + 2 * F3(vt, k, jv, i + 1) + F3(vt, k + 1, jv, i) +
                           F3(vt, k + 1, jv, i + 1) + F3(vt, k + 2, jv, i) + F3(vt, k + 2, jv, i + 1)) * 0.125;
            else if (k == kk - 2)
                f = awy * (F3(vt, k - 1, jv, i) + F3(vt, k - 1, jv, i + 1) + F3(vt, k, jv, i) + F3(vt, k, jv, i + 1) +
                           2 * F3(vt, k + 1, jv, i) + 2 * F3(vt, k + 1, jv, i + 1)) * 0.125;
            else
                f = awy * (F3(vt, k - 1, jv, i) + F3(vt, k - 1, jv, i + 1) + F3(vt, k, jv, i) + F3(vt, k, jv, i + 1) +
                           F3(vt, k + 1, jv, i) + F3(vt, k + 1, jv, i + 1) + F3(vt, k + 2, jv, i) +
                           F3(vt, k + 2, jv, i + 1)) * 0.125;
            N[PY(k, i)] = 0.5 * f * (F3(w, k, j, i) + F3(w, k, jn, i));
            N[PY(k, i + 1)] = 0.5 * f * (F3(w, k, j, i + 1) + F3(w, k, jn, i + 1));
        })
        PAR_LOOP2(i, 3, ii - 2, 1, k, 2, kk - 4, 2, { N[PY(k + 1, i)] = 0.5 * (N[PY(k, i)] + N[PY(k + 2, i)]); })
        PAR_LOOP2(i, 3, ii - 2, 1, k, 2, kk - 2, 1, {
            const double fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            const double rdzk = rdz[k];
            if (left)
                F3(wo, k, j, i) = F3(wo, k, j, i) + fkdtw * rdzk * (-S[PY(k, i)] + N[PY(k, i)]);
            else
                F3(wo, k, j, i) = F3(wo, k, j, i) + fkdtw * rdzk * (S[PY(k, i)] - N[PY(k, i)]);
        })
    }
#undef F3
}
#undef PAR_LOOP2

// ---- the viscosity field G (lesmodel_mod.F90:63-80, 573-764) --------------
// G = gmol inside every grid, 0 on its ghost layers
__global__ void k_init_g(const DevGrid* __restrict__ grids, double* Gf, double gmol) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    const bool in = i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2;
    Gf[G.ip3 + t] = in ? gmol : 0.0;
}

// bfront / bright / bbottom of G for face f (1..6) of the grids of ilevel
__global__ void k_bound_g(const DevGrid* __restrict__ grids, const BFace* __restrict__ bface,
                          int f, int ilevel, double* Gf, const double* __restrict__ BPF,
                          const double* __restrict__ buf, double geps) {
    const DevGrid G = grids[blockIdx.y];
    if (G.level != ilevel) return;
    const int t = G.bc[f - 1];
    const bool wall = t == MGLET_BC_NOS || t == MGLET_BC_SLI;
    const bool copy = t == MGLET_BC_FIX || t == MGLET_BC_OP1;
    const bool par = t == MGLET_BC_PAR;
    if (!wall && !copy && !par) return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int d = (f - 1) / 2;
    const int na = d == 0 ? jj : ii, nq = d == 2 ? jj : kk;
    const int q0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (q0 >= na * nq) return;
    const int a = q0 / nq + 1, q = q0 % nq + 1;
    if (par && (a < 2 || a > na - 1 || q < 2 || q > nq - 1)) return;
    const int n = d == 0 ? ii : (d == 1 ? jj : kk);
    const int p2 = f % 2 == 1 ? 2 : n - 1, p3 = f % 2 == 1 ? 3 : n - 2;
    auto at = [&](int p) -> long long {
        if (d == 0) return (long long)(p - 1) * kk * jj + (long long)(a - 1) * kk + (q - 1);
        if (d == 1) return (long long)(a - 1) * kk * jj + (long long)(p - 1) * kk + (q - 1);
        return (long long)(a - 1) * kk * jj + (long long)(q - 1) * kk + (p - 1);
    };
    double* gv = Gf + G.ip3;
    const long long x = at(p2);
    if (wall) {
        gv[x] = geps;
    } else if (copy) {
        gv[x] = gv[at(p3)];
    } else {
        const double sbp = BPF[G.ip3 + x];
        const double* b = buf + bface[6 * blockIdx.y + f - 1].off;
        gv[x] = b[(q - 1) + (long long)(a - 1) * nq] * sbp + (1.0 - sbp) * gv[x];
    }
}

// ---- par_ftoc_norm (par_ftoc_mod.F90:36-318) ------------------------------
// One block per message, one thread per coarse face: the area mean (or the
// sum) of the 2x2 fine faces of the PAR plane (pack_single), written where
// unpack_single puts it.
__global__ void k_par_ftoc(const DevGrid* __restrict__ grids, const PfTask* __restrict__ tasks,
                           double* U, double* V, double* W, const double* __restrict__ DDX,
                           const double* __restrict__ DDY, const double* __restrict__ DDZ, int sum) {
    const PfTask T = tasks[blockIdx.y];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= T.na * T.nb) return;
    const int a = q / T.nb, b = q % T.nb;
    const DevGrid G = grids[T.gf];
    const DevGrid C = grids[T.gc];
    const int d = (T.iface - 1) / 2;
    double* field = d == 0 ? U : (d == 1 ? V : W);
    const double* ff = field + G.ip3;
    const double *ddx = DDX + G.ipx - 1, *ddy = DDY + G.ipy - 1, *ddz = DDZ + G.ipz - 1;
    const int kk = G.kk, jj = G.jj;
    auto F = [&](int k, int j, int i) -> double {
        return ff[(long long)(i - 1) * kk * jj + (long long)(j - 1) * kk + (k - 1)];
    };
    const int lay = T.iface == 1 || T.iface == 3 || T.iface == 5
                        ? 2
                        : (d == 0 ? G.ii - 2 : (d == 1 ? G.jj - 2 : G.kk - 2));
    double val;
    int di, dj, dk;
    if (d == 0) {
        const int i = lay, j = 3 + 2 * a, k = 3 + 2 * b;
        if (sum) {
            val = F(k, j, i) + F(k, j + 1, i) + F(k + 1, j, i) + F(k + 1, j + 1, i);
        } else {
            const double sua = F(k, j, i) * ddy[j] * ddz[k] + F(k, j + 1, i) * ddy[j + 1] * ddz[k] +
                               F(k + 1, j, i) * ddy[j] * ddz[k + 1] + F(k + 1, j + 1, i) * ddy[j + 1] * ddz[k + 1];
            val = sua / ((ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
        }
        di = T.i0; dj = T.j0 + a; dk = T.k0 + b;
    } else if (d == 1) {
        const int i = 3 + 2 * a, j = lay, k = 3 + 2 * b;
        if (sum) {
            val = F(k, j, i) + F(k, j, i + 1) + F(k + 1, j, i) + F(k + 1, j, i + 1);
        } else {
            const double sua = F(k, j, i) * ddx[i] * ddz[k] + F(k, j, i + 1) * ddx[i + 1] * ddz[k] +
                               F(k + 1, j, i) * ddx[i] * ddz[k + 1] + F(k + 1, j, i + 1) * ddx[i + 1] * ddz[k + 1];
            val = sua / ((ddx[i] + ddx[i + 1]) * (ddz[k] + ddz[k + 1]));
        }
        di = T.i0 + a; dj = T.j0; dk = T.k0 + b;
    } else {
        const int i = 3 + 2 * a, j = 3 + 2 * b, k = lay;
        if (sum) {
            val = F(k, j, i) + F(k, j + 1, i) + F(k, j, i + 1) + F(k, j + 1, i + 1);
        } else {
            const double sua = F(k, j, i) * ddx[i] * ddy[j] + F(k, j + 1, i) * ddx[i] * ddy[j + 1] +
                               F(k, j, i + 1) * ddx[i + 1] * ddy[j] + F(k, j + 1, i + 1) * ddx[i + 1] * ddy[j + 1];
            val = sua / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]));
        }
        di = T.i0 + a; dj = T.j0 + b; dk = T.k0;
    }
    field[C.ip3 + (long long)(di - 1) * C.kk * C.jj + (long long)(dj - 1) * C.kk + (dk - 1)] = val;
}

int upload_list(Ctx* c, const std::vector<int>& h, int** d) {
    if (*d) cudaFree(*d);
    *d = nullptr;
    if (h.empty()) return 0;
    MG_CUDA(cudaMalloc(d, h.size() * sizeof(int)));
    MG_CUDA(copy_on(c->stream, *d, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
    return 0;
}

}  // namespace

int level_init(Ctx* c) {
    std::vector<int> any;
    for (int g = 0; g < c->ngrid; ++g)
        for (int f = 0; f < 6; ++f)
            if (c->grids[g].bc[f] == MGLET_BC_PAR) {
                any.push_back(g);
                break;
            }
    c->npargrids = (int)any.size();
    if (int rc = upload_list(c, any, &c->d_pargrids)) return rc;
    for (int f = 0; f < 6; ++f) {
        c->pgrids[f].clear();
        for (int g = 0; g < c->ngrid; ++g)
            if (c->grids[g].bc[f] == MGLET_BC_PAR) c->pgrids[f].push_back(g);
        if (int rc = upload_list(c, c->pgrids[f], &c->d_pgrids[f])) return rc;
    }
    c->hier.assign(c->ngrid, make_int4(-1, 0, 0, 0));
    MG_CUDA(cudaMalloc(&c->d_hier, (size_t)c->ngrid * sizeof(int4)));
    MG_CUDA(copy_on(c->stream, c->d_hier, c->hier.data(), c->hier.size() * sizeof(int4),
                    cudaMemcpyHostToDevice));
    return 0;
}

int set_hierarchy(Ctx* c, const int32_t* iparent, const int32_t* pos) {
    std::vector<int4> h(c->ngrid);
    for (int g = 0; g < c->ngrid; ++g) {
        const int par = iparent[g];
        if (par < 0 || par > c->ngrid || par == g + 1)
        {
            set_error("set_hierarchy: bad parent");
            return MGLET_ERR_ARG;
        }
        if (par && c->grids[par - 1].level != c->grids[g].level - 1)
        {
            set_error("set_hierarchy: parent not one level coarser");
            return MGLET_ERR_ARG;
        }
        const int ip = pos[3 * g], jp = pos[3 * g + 1], kp = pos[3 * g + 2];
        if (par) {
            // the slabs parent, ftoc and ctof read and write stay inside the parent
            const DevGrid& G = c->grids[g];
            const DevGrid& P = c->grids[par - 1];
            if (ip < 3 || jp < 3 || kp < 3 || ip + G.ii / 2 - 1 > P.ii || jp + G.jj / 2 - 1 > P.jj ||
                kp + G.kk / 2 - 1 > P.kk || (G.ii | G.jj | G.kk) & 1)
            {
                set_error("set_hierarchy: fine grid outside its parent");
                return MGLET_ERR_ARG;
            }
        }
        h[g] = make_int4(par - 1, ip, jp, kp);
    }
    c->hier = h;
    MG_CUDA(copy_on(c->stream, c->d_hier, c->hier.data(), c->hier.size() * sizeof(int4),
                    cudaMemcpyHostToDevice));
    // siblings side by side restrict onto the same coarse face of their
    // parent (U, V, W): the earlier grid of each such pair skips that face
    {
        std::vector<int> skip(c->ngrid, 0);
        std::map<int, std::vector<int>> kids;
        for (int g = 0; g < c->ngrid; ++g)
            if (h[g].x >= 0) kids[h[g].x].push_back(g);
        for (auto& kv : kids)
            for (int a : kv.second)
                for (int b : kv.second) {
                    if (a >= b) continue;
                    const DevGrid& A = c->grids[a];
                    const int pa[3] = {h[a].y, h[a].z, h[a].w}, pb[3] = {h[b].y, h[b].z, h[b].w};
                    const int half[3] = {(A.ii - 4) / 2, (A.jj - 4) / 2, (A.kk - 4) / 2};
                    for (int ax = 0; ax < 3; ++ax) {
                        bool same = true;
                        for (int o = 0; o < 3; ++o)
                            if (o != ax && pa[o] != pb[o]) same = false;
                        if (!same) continue;
                        if (pb[ax] == pa[ax] + half[ax]) skip[a] |= 2 << (2 * ax);   // b above a
                        if (pa[ax] == pb[ax] + half[ax]) skip[a] |= 1 << (2 * ax);   // b below a
                    }
                }
        if (!c->d_ftoc_skip) MG_CUDA(cudaMalloc(&c->d_ftoc_skip, c->ngrid * sizeof(int)));
        MG_CUDA(copy_on(c->stream, c->d_ftoc_skip, skip.data(), c->ngrid * sizeof(int),
                        cudaMemcpyHostToDevice));
    }
    for (auto& kv : c->d_children) cudaFree(kv.second);
    c->d_children.clear();
    c->children.clear();
    for (int g = 0; g < c->ngrid; ++g)
        if (c->hier[g].x >= 0) c->children[c->grids[g].level].push_back(g);
    for (auto& kv : c->children) {
        int* d = nullptr;
        if (int rc = upload_list(c, kv.second, &d)) return rc;
        c->d_children[kv.first] = d;
    }
    // par_ftoc_norm messages (init_par_ftoc, par_ftoc_mod.F90:513-690) and
    // the coarse planes unpack_single (:366-469) writes them to
    for (auto& kv : c->d_pftasks) cudaFree(kv.second);
    c->d_pftasks.clear();
    c->pftasks.clear();
    for (int g = 0; g < c->ngrid; ++g) {
        const int4 H = c->hier[g];
        if (H.x < 0) continue;
        const DevGrid& G = c->grids[g];
        const DevGrid& P = c->grids[H.x];
        for (int iface = 1; iface <= 6; ++iface) {
            if (G.bc[iface - 1] != MGLET_BC_PAR) continue;
            const int d = (iface - 1) / 2;
            const bool odd = iface % 2 == 1;
            const int pos = d == 0 ? H.y : (d == 1 ? H.z : H.w);
            const int nf = d == 0 ? G.ii : (d == 1 ? G.jj : G.kk);
            const int nc = d == 0 ? P.ii : (d == 1 ? P.jj : P.kk);
            const bool one_connect = !(nf > nc);
            int recv1 = iface;
            if (pos == 3 && one_connect) {
                if (!odd) recv1 = -1;
            } else if (pos > 3) {
                if (odd) recv1 = -1;
            }
            auto add = [&](int gc, int ifr) -> int {
                const DevGrid& C = c->grids[gc];
                int lo[3] = {H.y, H.z, H.w};
                int hi[3] = {H.y + (G.ii - 4) / 2 - 1, H.z + (G.jj - 4) / 2 - 1, H.w + (G.kk - 4) / 2 - 1};
                if (ifr < 0) {
                    if (odd) lo[d] = hi[d] = lo[d] - 1;
                    else lo[d] = hi[d];
                } else {
                    const int n = d == 0 ? C.ii : (d == 1 ? C.jj : C.kk);
                    lo[d] = hi[d] = ifr % 2 == 1 ? 2 : n - 2;
                }
                const int dims[3] = {C.ii, C.jj, C.kk};
                for (int q = 0; q < 3; ++q)
                    if (lo[q] < 1 || hi[q] > dims[q]) {
                        set_error("set_hierarchy: a par_ftoc_norm plane lies outside its coarse grid");
                        return MGLET_ERR_ARG;
                    }
                PfTask t;
                t.gf = g; t.gc = gc; t.iface = iface;
                t.i0 = lo[0]; t.j0 = lo[1]; t.k0 = lo[2];
                t.na = d == 0 ? (G.jj - 4) / 2 : (G.ii - 4) / 2;
                t.nb = d == 2 ? (G.jj - 4) / 2 : (G.kk - 4) / 2;
                c->pftasks[G.level].push_back(t);
                return 0;
            };
            if (int rc = add(H.x, recv1)) return rc;
            if (recv1 < 0) continue;
            const int nb = c->nbr[H.x + 1][iface];
            if (nb <= 0) continue;
            if (int rc = add(nb - 1, odd ? iface + 1 : iface - 1)) return rc;
        }
    }
    for (auto& kv : c->pftasks) {
        PfTask* d = nullptr;
        MG_CUDA(cudaMalloc(&d, kv.second.size() * sizeof(PfTask)));
        MG_CUDA(copy_on(c->stream, d, kv.second.data(), kv.second.size() * sizeof(PfTask),
                        cudaMemcpyHostToDevice));
        c->d_pftasks[kv.first] = d;
    }
    for (int f = 0; f < 6; ++f) {
        for (auto& kv : c->d_plist[f]) cudaFree(kv.second);
        c->d_plist[f].clear();
        c->plist[f].clear();
        for (int g : c->pgrids[f])
            if (c->hier[g].x >= 0) c->plist[f][c->grids[g].level].push_back(g);
        for (auto& kv : c->plist[f]) {
            int* d = nullptr;
            if (int rc = upload_list(c, kv.second, &d)) return rc;
            c->d_plist[f][kv.first] = d;
        }
    }
    // the finer levels' G takes its PAR values now that the parents are known
    if (!c->g_user)
        if (int rc = init_viscosity(c)) return rc;
    return 0;
}

double* field_buffer(Ctx* c, const std::string& name) {
    if (name == "U") return c->d_buf[0];
    if (name == "V") return c->d_buf[1];
    if (name == "W") return c->d_buf[2];
    auto it = c->fbuf.find(name);
    if (it != c->fbuf.end()) return it->second;
    double* b = nullptr;
    if (cudaMalloc(&b, (size_t)c->nbuf * sizeof(double)) != cudaSuccess) return nullptr;
    if (zero_on(c->stream, b, (size_t)c->nbuf * sizeof(double)) != cudaSuccess) {
        cudaFree(b);
        return nullptr;
    }
    c->fbuf[name] = b;
    return b;
}

int launch_tstle4_par(Ctx* c, double* uo, double* vo, double* wo, const double* u, const double* v,
                      const double* w, const double* ut, const double* vt, const double* wt) {
    if (!c->npargrids) return 0;
    ProfScope ps_(c, "tstle4_par");
    ParFluxArgs A{};
    A.grids = c->d_grids;
    A.list = c->d_pargrids;
    A.uo = uo; A.vo = vo; A.wo = wo;
    A.u = u; A.v = v; A.w = w; A.ut = ut; A.vt = vt; A.wt = wt;
    A.dx = c->L("DX"); A.dy = c->L("DY"); A.dz = c->L("DZ");
    A.ddx = c->L("DDX"); A.ddy = c->L("DDY"); A.ddz = c->L("DDZ");
    A.rdx = c->L("RDX"); A.rdy = c->L("RDY"); A.rdz = c->L("RDZ");
    A.rddx = c->L("RDDX"); A.rddy = c->L("RDDY"); A.rddz = c->L("RDDZ");
    int pl = 0;
    for (const DevGrid& G : c->grids) pl = std::max(pl, std::max(G.kk * G.jj, std::max(G.kk * G.ii, G.jj * G.ii)));
    const size_t smem = (size_t)2 * pl * sizeof(double);
    if (smem > 227 * 1024) {
        set_error("tstle4_par: a face plane of more than 14528 points does not fit in shared memory");
        return MGLET_ERR_UNSUPPORTED;
    }
    if (smem > 48 * 1024)
        MG_CUDA(cudaFuncSetAttribute(k_tstle4_par, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_tstle4_par<<<c->npargrids, 256, smem, c->stream>>>(A);
    MG_LAUNCHED(c);
    return 0;
}

// init_lesmodel for the model "none" (lesmodel_mod.F90:63-80): G = gmol
// inside, 0 on the ghost layers (zero_ghostlayers), connected with corners;
// on the finer levels the parent's values into the PAR buffers and the bound
// of G.  The coarsest level's wall ghosts keep 0: no viscous flux crosses
// those faces (NOS walls carry the wall function instead).
int init_viscosity(Ctx* c) {
    double* Gf = c->F("G");
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    k_init_g<<<dim3((m + 255) / 256, c->ngrid), 256, 0, c->stream>>>(c->d_grids, Gf, c->prm.gmol);
    MG_LAUNCHED(c);
    if (int rc = connect(c, 0, 2, nullptr, nullptr, nullptr, Gf, nullptr, nullptr, true, false, 0))
        return rc;
    static const char* const none[3] = {nullptr, nullptr, nullptr};
    static const char* const sg[3] = {"G", nullptr, nullptr};
    for (int l = c->minlevel + 1; l <= c->maxlevel; ++l) {
        if (int rc = launch_parent(c, l, none, sg, false)) return rc;
        if (int rc = launch_bound_g(c, l)) return rc;
    }
    return 0;
}

// the bound of G on the grids of ilevel, faces 1..6 one after the other
// (bound_mod.F90:36-76)
int launch_bound_g(Ctx* c, int ilevel) {
    double* buf = field_buffer(c, "G");
    if (!buf) {
        set_error("bound of G: buffer allocation");
        return MGLET_ERR_CUDA;
    }
    int mp = 0;
    for (const DevGrid& g : c->grids) mp = std::max(mp, std::max(g.jj * g.kk, std::max(g.ii * g.kk, g.ii * g.jj)));
    const double geps = -std::numeric_limits<double>::epsilon() * c->prm.gmol;
    for (int f = 1; f <= 6; ++f) {
        k_bound_g<<<dim3((mp + 127) / 128, c->ngrid), 128, 0, c->stream>>>(
            c->d_grids, c->d_bface, f, ilevel, c->F("G"), c->F("BP"), buf, geps);
        MG_LAUNCHED(c);
    }
    return 0;
}

int launch_par_ftoc_norm(Ctx* c, int ilevel, double* u, double* v, double* w, bool sum) {
    ProfScope ps_(c, "par_ftoc_norm");
    auto it = c->d_pftasks.find(ilevel);
    if (it == c->d_pftasks.end()) return 0;
    const std::vector<PfTask>& ts = c->pftasks[ilevel];
    int maxq = 0;
    for (const PfTask& t : ts) maxq = std::max(maxq, t.na * t.nb);
    k_par_ftoc<<<dim3((maxq + 127) / 128, (unsigned)ts.size()), 128, 0, c->stream>>>(
        c->d_grids, it->second, u, v, w, c->L("DDX"), c->L("DDY"), c->L("DDZ"), sum ? 1 : 0);
    MG_LAUNCHED(c);
    return 0;
}

int launch_bound_par(Ctx* c, int iface, int ilevel, double* u, double* v, double* w) {
    const int f = iface - 1;
    if (c->pgrids[f].empty()) return 0;
    int maxq = 0;
    for (int g : c->pgrids[f]) {
        const DevGrid& G = c->grids[g];
        maxq = std::max(maxq, (f / 2 == 2 ? G.jj : G.kk) * (f / 2 == 0 ? G.jj : G.ii));
    }
    ParArgs A{};
    A.grids = c->d_grids;
    A.list = c->d_pgrids[f];
    A.bface = c->d_bface;
    A.ub = c->d_buf[0]; A.vb = c->d_buf[1]; A.wb = c->d_buf[2];
    A.bp = c->F("BP");
    A.ddx = c->L("DDX"); A.ddy = c->L("DDY"); A.ddz = c->L("DDZ");
    A.u = u; A.v = v; A.w = w;
    A.iface = iface;
    A.ilevel = ilevel;
    k_bound_par<<<dim3((maxq + 127) / 128, (unsigned)c->pgrids[f].size()), 128, 0, c->stream>>>(A);
    MG_LAUNCHED(c);
    return 0;
}

int launch_parent(Ctx* c, int ilevel, const char* const v[3], const char* const s[3], bool normal) {
    ProfScope ps_(c, "parent");
    for (int f = 0; f < 6; ++f) {
        auto it = c->d_plist[f].find(ilevel);
        if (it == c->d_plist[f].end()) continue;
        const std::vector<int>& list = c->plist[f][ilevel];
        ParentArgs A{};
        A.grids = c->d_grids;
        A.hier = c->d_hier;
        A.bface = c->d_bface;
        A.list = it->second;
        A.iface = f + 1;
        int nslot = 0;
        const bool ex[3] = {!normal || f < 2, !normal || (f >= 2 && f < 4), !normal || f >= 4};
        for (int q = 0; q < 3; ++q)
            if (v[q] && ex[q]) {
                A.fc[nslot] = c->F(v[q]);
                A.buf[nslot] = field_buffer(c, v[q]);
                if (!A.buf[nslot]) return cuda_fail(cudaErrorMemoryAllocation, "parent buffers");
                A.comp[nslot++] = q + 1;
            }
        for (int q = 0; q < 3; ++q)
            if (s[q]) {
                A.fc[nslot] = c->F(s[q]);
                A.buf[nslot] = field_buffer(c, s[q]);
                if (!A.buf[nslot]) return cuda_fail(cudaErrorMemoryAllocation, "parent buffers");
                A.comp[nslot++] = 0;
            }
        if (!nslot) continue;
        int maxq = 0;
        for (int g : list) {
            const DevGrid& G = c->grids[g];
            maxq = std::max(maxq, (f / 2 == 2 ? G.jj : G.kk) * (f / 2 == 0 ? G.jj : G.ii));
        }
        k_parent<<<dim3((maxq + 127) / 128, (unsigned)list.size(), nslot), 128, 0, c->stream>>>(A);
        MG_LAUNCHED(c);
    }
    return 0;
}

int launch_ftoc(Ctx* c, int ilevel, const double* ff, double* fc, char flag) {
    ProfScope ps_(c, "ftoc");
    auto it = c->d_children.find(ilevel);
    if (it == c->d_children.end()) return 0;
    const std::vector<int>& list = c->children[ilevel];
    FtocArgs A{};
    A.grids = c->d_grids;
    A.hier = c->d_hier;
    A.list = it->second;
    A.ff = ff;
    A.fc = fc;
    A.ddx = c->L("DDX"); A.ddy = c->L("DDY"); A.ddz = c->L("DDZ");
    A.bp = c->F("BP");
    A.skip = c->d_ftoc_skip;
    A.flag = (flag == 'R' || flag == 'S' || flag == 'T') ? 'P' : flag;
    if (c->ibtype == 1 && flag == 'P') A.flag = 'G';       // gc_restrict_t
    if (c->ibtype == 1 && flag == 'R') A.flag = 'H';
    if (c->ibtype == 1 && flag == 'T') {
        // restrict_p weighted by BT instead of BP (gc_restrict_mod.F90:85-89)
        if (!c->f3.count("BT")) {
            set_error("ftoc: the ghost-cell T restriction weighs by BT (set_scalars first)");
            return MGLET_ERR_UNSUPPORTED;
        }
        A.flag = 'G';
        A.bp = c->F("BT");
    }
    int maxq = 0;
    for (int g : list) {
        const DevGrid& G = c->grids[g];
        maxq = std::max(maxq, (G.ii / 2 - 1) * (G.jj / 2 - 1) * (G.kk / 2 - 1));
    }
    k_ftoc<<<dim3((maxq + 127) / 128, (unsigned)list.size()), 128, 0, c->stream>>>(A);
    MG_LAUNCHED(c);
    return 0;
}

int launch_ctof(Ctx* c, int ilevel, double* ff, const double* fc) {
    ProfScope ps_(c, "ctof");
    if (ilevel == c->minlevel) return 0;
    auto it = c->d_children.find(ilevel);
    if (it == c->d_children.end()) return 0;
    const std::vector<int>& list = c->children[ilevel];
    long long maxq = 0;
    for (int g : list) {
        const DevGrid& G = c->grids[g];
        maxq = std::max(maxq, (long long)G.kk * G.jj * G.ii);
    }
    k_ctof<<<dim3((unsigned)((maxq + 255) / 256), (unsigned)list.size()), 256, 0, c->stream>>>(
        c->d_grids, c->d_hier, it->second, ff, fc);
    MG_LAUNCHED(c);
    return 0;
}

int launch_bound_pressure(Ctx* c, int ilevel, double* p, const double* buf, bool withbp) {
    ProfScope ps_(c, "bound_pressure");
    for (int f = 0; f < 6; ++f) {
        if (c->pgrids[f].empty()) continue;
        int maxq = 0;
        for (int g : c->pgrids[f]) {
            const DevGrid& G = c->grids[g];
            const int na = f / 2 == 2 ? G.jj : G.kk, nb = f / 2 == 0 ? G.jj : G.ii;
            maxq = std::max(maxq, ((na - 4) / 2) * ((nb - 4) / 2));
        }
        BpArgs A{};
        A.grids = c->d_grids;
        A.list = c->d_pgrids[f];
        A.bface = c->d_bface;
        A.buf = buf;
        A.bp = withbp ? c->F("BP") : nullptr;
        A.ddx = c->L("DDX"); A.ddy = c->L("DDY"); A.ddz = c->L("DDZ");
        A.dx = c->L("DX"); A.dy = c->L("DY"); A.dz = c->L("DZ");
        A.p = p;
        A.iface = f + 1;
        A.ilevel = ilevel;
        k_bound_pressure<<<dim3((maxq + 127) / 128, (unsigned)c->pgrids[f].size()), 128, 0, c->stream>>>(A);
        MG_LAUNCHED(c);
    }
    return 0;
}

}  // namespace mg
