// gc_create.cu -- construction of the ghost-cell stencil lists (host code).
//
// Restates the reference's stencil construction of the ghost-cell immersed
// boundary, create_flowstencils (src/flow/gc_flowstencils_mod.F90:37-100,
// createstencils_level :164-196) with
//   * fluxcorrection (:199-553): per blocked pressure cell next to open
//     cells, the open face areas through which its divergence is corrected
//     and the flux of the body velocity through its blocked faces;
//   * fluxstencil (:556-752) and calcflux (:838-920): per blocked velocity
//     point next to open ones, an interpolation stencil from the cut cell's
//     plane -- wmcheckneighbor, choosestencil, wmmultimatrix / calcfluxu,
//     wmaddcoefflist and wmindexlistn of src/ib/gc_createstencils_mod.F90,
//     findinterface2 of src/ib/findinterface_mod.F90:14-80;
// in the list formats the runtime consumes (what the reference keeps in
// fxpoli/fxpolr and uxpoli/uxpolr/uxpolrvel etc., and reads back from
// ib_stencils.h5).  Expressions keep the reference's operation order and its
// REAL64-build literal kinds (single-precision 0.9, 0.61 and maccur = 1.0e-4
// widened to double), so the lists do not depend on how they are produced.
// This file is compiled with -ffp-contract=off for the host.
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

struct mglet_flowstencils {
    // per grid, per component 1..4 (index 0..3)
    struct List {
        int ncells = 0;
        std::vector<int64_t> xi;
        std::vector<double> xr, xv;
    };
    std::vector<std::array<List, 4>> g;
};

// per grid the scalar list: 9 integers and 8 reals per cell
struct mglet_scastencils {
    struct List {
        int ncells = 0;
        std::vector<int64_t> xi;
        std::vector<double> xr, xv;
    };
    std::vector<List> g;
};

namespace mg {
namespace {

constexpr double kMaccur = (double)1.0e-4f;    // ibconst_mod.F90:8, default-kind literal

struct GridView {
    int kk, jj, ii;
    int bc[6];
    const double *x, *y, *z, *xs, *ys, *zs, *ddx, *ddy, *ddz;   // 1-based views
    const double *bp, *bu, *bv, *bw, *au, *av, *aw;
    const int32_t* bz;
    int icells;
    const double* nvecs;   // [icells][4], 0-based cell
    const double* ucell;   // [icells][3]
    long long at(int k, int j, int i) const {
        return (long long)(k - 1) + (long long)(j - 1) * kk + (long long)(i - 1) * kk * jj;
    }
    int64_t flat1(int k, int j, int i) const { return 1 + at(k, j, i); }
};

struct Found {
    int found = 0, x1 = 0, x2 = 0, y1 = 0, y2 = 0, z1 = 0, z2 = 0, nr = 0;
};

// findinterface2_a (findinterface_mod.F90:14-64): a blocked point with open
// face neighbours
Found findinterface2(const GridView& G, const double* b, int k, int j, int i) {
    Found f;
    if (b[G.at(k, j, i)] <= 0.5) {
        if (b[G.at(k, j, i + 1)] >= 0.5) { f.nr++; f.found = 1; f.x1 = 1; }
        if (b[G.at(k, j, i - 1)] >= 0.5) { f.nr++; f.found = 1; f.x2 = 1; }
        if (b[G.at(k, j + 1, i)] >= 0.5) { f.nr++; f.found = 1; f.y1 = 1; }
        if (b[G.at(k, j - 1, i)] >= 0.5) { f.nr++; f.found = 1; f.y2 = 1; }
        if (b[G.at(k + 1, j, i)] >= 0.5) { f.nr++; f.found = 1; f.z1 = 1; }
        if (b[G.at(k - 1, j, i)] >= 0.5) { f.nr++; f.found = 1; f.z2 = 1; }
    }
    return f;
}

// Fortran NINT for the 0/1 blocking fields
int nint(double v) { return (int)std::lround(v); }

// wmindexlistn (gc_createstencils_mod.F90:416-453): offsets of a ball of
// radius 3 (without the centre) in i-outer, j, k-inner order
struct Ball {
    std::vector<int> di, dj, dk;
    Ball() {
        const int box = 7, radius = (box - 1) / 2;
        for (int i = 1; i <= box; ++i)
            for (int j = 1; j <= box; ++j)
                for (int k = 1; k <= box; ++k) {
                    const int a = i - ((int)(box / 2.0) + 1);
                    const int b = j - ((int)(box / 2.0) + 1);
                    const int c = k - ((int)(box / 2.0) + 1);
                    if (a != 0 || b != 0 || c != 0) {
                        // (|a|^2+|b|^2+|c|^2)**0.5 <= radius, the REAL power
                        // of an integer sum
                        const double r = std::pow((double)(float)(a * a + b * b + c * c), (double)0.5f);
                        if ((float)r <= (float)radius) {
                            di.push_back(a);
                            dj.push_back(b);
                            dk.push_back(c);
                        }
                    }
                }
    }
};

// wmcheckneighbor (gc_createstencils_mod.F90:15-107): open points of the ball
// inside the region the face conditions allow
void checkneighbor(const GridView& G, const double* b, int k, int j, int i, const Ball& ball,
                   std::vector<int>& is, std::vector<int>& js, std::vector<int>& ks) {
    int ir[6];
    for (int f = 0; f < 6; ++f) {
        const int t = G.bc[f];
        ir[f] = 2;
        if (t == 3 || t == 4 || t == 6) ir[f] = 0;      // OP1, OP2, SLI
        if (t == 8 || t == 7) ir[f] = 1;                // PAR, CON
    }
    is.clear(); js.clear(); ks.clear();
    for (size_t n = 0; n < ball.di.size(); ++n) {
        bool none = false;
        const int it = i + ball.di[n], jt = j + ball.dj[n], kt = k + ball.dk[n];
        if (it < 3 - ir[0] || it > G.ii - 2 + ir[1]) none = true;
        if (jt < 3 - ir[2] || jt > G.jj - 2 + ir[3]) none = true;
        if (kt < 3 - ir[4] || kt > G.kk - 2 + ir[5]) none = true;
        if (!none && nint(b[G.at(kt, jt, it)]) == 1) {
            is.push_back(it);
            js.push_back(jt);
            ks.push_back(kt);
        }
    }
}

// choosestencil (gc_createstencils_mod.F90:110-174): the face neighbours, and
// with only one of them the next point beyond it; one point alone is no
// stencil.  Returns velpts, the chosen points first in is/js/ks.
int choosestencil(int k, int j, int i, std::vector<int>& is, std::vector<int>& js,
                  std::vector<int>& ks) {
    const int nstc = (int)is.size();
    std::vector<int> it(nstc, 0), jt(nstc, 0), kt(nstc, 0);
    int velpts = 0;
    for (int n = 0; n < nstc; ++n) {
        const int id = std::abs(is[n] - i), jd = std::abs(js[n] - j), kd = std::abs(ks[n] - k);
        if (id + jd + kd == 1) {
            it[velpts] = is[n]; jt[velpts] = js[n]; kt[velpts] = ks[n];
            velpts++;
        }
    }
    if (velpts == 1) {
        const int ig = (it[0] - i) * 2 + i, jg = (jt[0] - j) * 2 + j, kg = (kt[0] - k) * 2 + k;
        for (int n = 0; n < nstc; ++n)
            if (ig == is[n] && jg == js[n] && kg == ks[n]) {
                it[velpts] = is[n]; jt[velpts] = js[n]; kt[velpts] = ks[n];
                velpts++;
            }
    }
    if (velpts == 1) velpts = 0;
    is = it; js = jt; ks = kt;
    return velpts;
}

struct Coeffs {
    double c[20], cv[20];
    double a = 0.0, av = 0.0;
};

// calcfluxu (gc_createstencils_mod.F90:241-384) in its own argument names:
// the face of point (k, j, i) normal to x, the plane a x + b y + c z = dpl,
// the body velocity avel; 20 x 20 midpoint sub-faces.  Returns found.
int calcfluxu(int k, int j, int i, const double* x, const double* y, const double* z,
              const double* xstag, const double* ystag, const double* zstag, double a, double b,
              double c, double dpl, double avel, int velpts, const int* istc, const int* jstc,
              const int* kstc, Coeffs& co) {
    (void)x;
    const int parts = 20;
    double dpoint = a * xstag[i] + b * ystag[j] + c * zstag[k] - dpl;
    double dall = 0.0;
    double dist[20], ce[20];
    for (int n = 0; n < velpts; ++n) {
        dist[n] = a * xstag[istc[n]] + b * ystag[jstc[n]] + c * zstag[kstc[n]] - dpl;
        if (dist[n] < std::fabs(dpoint) * (double)0.9f) dist[n] = 0.0;
        dall = dall + dist[n] * dist[n];
    }
    if (std::fabs(dall) <= 2.2250738585072014e-308) return 0;    // TINY(dall)
    double cesum = 0.0;
    for (int n = 0; n < velpts; ++n) {
        ce[n] = dist[n] / dall;
        cesum = cesum + ce[n];
    }
    const double dy = y[j] - y[j - 1];
    const double dz = z[k] - z[k - 1];
    const double ddy = dy / (double)parts;
    const double ddz = dz / (double)parts;
    const double ys = y[j - 1] - ddy / 2.0;
    const double zs = z[k - 1] - ddz / 2.0;
    int carea2 = 0;
    const double xm = xstag[i];
    const double dt = -dpl + a * xm;
    for (int jt = 1; jt <= parts; ++jt) {
        const double ym = ys + ddy * (double)jt;
        for (int kt = 1; kt <= parts; ++kt) {
            const double zm = zs + ddz * (double)kt;
            const double dir = dt + b * ym + c * zm;
            if (dir > 0.0) {
                dpoint = a * xm + b * ym + c * zm - dpl;
                for (int n = 0; n < velpts; ++n) co.c[n] = co.c[n] + dpoint * ce[n];
                co.a = co.a + 1.0 - dpoint * cesum;
            } else {
                carea2 = carea2 + 1;
            }
        }
    }
    const double area = ddy * ddz;
    for (int n = 0; n < velpts; ++n) co.c[n] = co.c[n] * area / (dy * dz);
    co.a = co.a * avel * area / (dy * dz);
    co.a = co.a + avel * ((double)carea2 * area) / (dy * dz);
    dpoint = a * xstag[i] + b * ystag[j] + c * zstag[k] - dpl;
    for (int n = 0; n < velpts; ++n) co.cv[n] = dpoint * ce[n];
    co.av = avel * (1.0 - dpoint * cesum);
    double sum = 0.0;
    for (int n = 0; n < velpts; ++n) sum = sum + co.c[n];
    if (sum > (double)0.61f) return -1;
    return 1;
}

struct Lists {
    std::vector<int64_t> xi;
    std::vector<double> xr, xv;
    int n = 0;
};

// wmdocoefflist (gc_flowstencils_mod.F90:755-812)
void docoefflist(const GridView& G, int k, int j, int i, double ac, double acv, int velpts,
                 const int* is, const int* js, const int* ks, const Coeffs* co, Lists& L) {
    L.xi.push_back(G.flat1(k, j, i));
    L.xi.push_back(velpts);
    for (int n = 0; n < velpts; ++n) {
        L.xi.push_back(G.flat1(ks[n], js[n], is[n]));
        L.xr.push_back(co->c[n]);
        L.xv.push_back(co->cv[n]);
    }
    L.xr.push_back(ac);
    L.xv.push_back(acv);
}

// wmaddcoefflist (gc_createstencils_mod.F90:387-413): the second cut cell's
// stencil averaged into the entry just written
void addcoefflist(int velpts, const Coeffs& co, Lists& L) {
    size_t p = L.xr.size() - (velpts + 1);
    for (int n = 0; n < velpts; ++n, ++p) {
        L.xr[p] = 0.5 * L.xr[p] + 0.5 * co.c[n];
        L.xv[p] = 0.5 * L.xv[p] + 0.5 * co.cv[n];
    }
    L.xr[p] = 0.5 * L.xr[p] + 0.5 * co.a;
    L.xv[p] = 0.5 * L.xv[p] + 0.5 * co.av;
}

// wmmultimatrix (gc_createstencils_mod.F90:177-238): calcfluxu with the
// coordinates permuted to the component's face direction
int multimatrix(const GridView& G, int compon, int k, int j, int i, int kt, int jt, int it,
                const std::vector<int>& is, const std::vector<int>& js, const std::vector<int>& ks,
                int velpts, Coeffs& co) {
    const int cell = -G.bz[G.at(kt, jt, it)] - 1;
    const double* nv = G.nvecs + 4LL * cell;
    const double* uc = G.ucell + 3LL * cell;
    const double a = nv[0], b = nv[1], c = nv[2], dpl = nv[3];
    for (int n = 0; n < 20; ++n) co.c[n] = co.cv[n] = 0.0;
    co.a = co.av = 0.0;
    switch (compon) {
        case 1:
            return calcfluxu(k, j, i, G.x, G.ys, G.zs, G.xs, G.y, G.z, a, b, c, dpl, uc[0], velpts,
                             is.data(), js.data(), ks.data(), co);
        case 2:
            return calcfluxu(k, i, j, G.y, G.xs, G.zs, G.ys, G.x, G.z, b, a, c, dpl, uc[1], velpts,
                             js.data(), is.data(), ks.data(), co);
        default:
            return calcfluxu(i, j, k, G.z, G.ys, G.xs, G.zs, G.y, G.x, c, b, a, dpl, uc[2], velpts,
                             ks.data(), js.data(), is.data(), co);
    }
}

// calcflux (gc_flowstencils_mod.F90:838-920); found in/out as there
void calcflux(const GridView& G, const double* b, int compon, int k, int j, int i, int kt, int jt,
              int it, const Ball& ball, int& found, int foundone, Lists& L) {
    std::vector<int> is, js, ks;
    checkneighbor(G, b, k, j, i, ball, is, js, ks);
    const int velpts = choosestencil(k, j, i, is, js, ks);
    if (velpts > 6) { found = -2; return; }
    if (velpts == 0) { found = -3; return; }
    Coeffs co;
    found = multimatrix(G, compon, k, j, i, kt, jt, it, is, js, ks, velpts, co);
    for (int m = 0; m < velpts; ++m)
        if (std::fabs(co.cv[m]) > 12.0) found = -4;
    if (found == 1) {
        if (foundone == 0)
            docoefflist(G, k, j, i, co.a, co.av, velpts, is.data(), js.data(), ks.data(), &co, L);
        else if (foundone == 1)
            addcoefflist(velpts, co, L);
    }
}

// fluxstencil (gc_flowstencils_mod.F90:556-752), b the component's blocking
void fluxstencil(const GridView& G, const double* b, int compon, const Ball& ball, Lists& L) {
    const int kb = compon == 3 ? 2 : 3, jb = compon == 2 ? 2 : 3, ib = compon == 1 ? 2 : 3;
    for (int i = ib; i <= G.ii - 2; ++i)
        for (int j = jb; j <= G.jj - 2; ++j)
            for (int k = kb; k <= G.kk - 2; ++k) {
                int found = findinterface2(G, b, k, j, i).found;
                if (found != 1) continue;
                int it[2] = {i, i}, jt[2] = {j, j}, kt[2] = {k, k};
                int calc = 0;
                const int di = compon == 1, dj = compon == 2, dk = compon == 3;
                if (G.bz[G.at(k, j, i)] < 0) calc++;
                if (G.bz[G.at(k + dk, j + dj, i + di)] < 0) {
                    calc++;
                    it[calc - 1] = i + di;
                    jt[calc - 1] = j + dj;
                    kt[calc - 1] = k + dk;
                }
                if (calc == 0) {
                    docoefflist(G, k, j, i, 0.0, 0.0, 0, nullptr, nullptr, nullptr, nullptr, L);
                    L.n++;
                    continue;
                }
                int foundone = 0;
                for (int add = 0; add < calc; ++add) {
                    calcflux(G, b, compon, k, j, i, kt[add], jt[add], it[add], ball, found, foundone, L);
                    if (found == 1) foundone = 1;
                }
                if (foundone != 1) {
                    // rescue stencil: the body velocity of the first cut cell
                    const int cell = -G.bz[G.at(kt[0], jt[0], it[0])] - 1;
                    const double avel = G.ucell[3LL * cell + compon - 1];
                    docoefflist(G, k, j, i, avel, avel, 0, nullptr, nullptr, nullptr, nullptr, L);
                }
                L.n++;
            }
}

// fluxcorrection (gc_flowstencils_mod.F90:199-553)
void fluxcorrection(const GridView& G, Lists& L) {
    const int nfro = G.bc[0], nbac = G.bc[1], nrgt = G.bc[2], nlft = G.bc[3], nbot = G.bc[4],
              ntop = G.bc[5];
    int kmax = G.kk - 2, jmax = G.jj - 2, imax = G.ii - 2;
    if (nbac == 7) imax = G.ii - 1;
    if (nlft == 7) jmax = G.jj - 1;
    if (ntop == 7) kmax = G.kk - 1;
    auto wall = [](int t) { return t == 2 || t == 5 || t == 6; };
    for (int i = 3; i <= imax; ++i)
        for (int j = 3; j <= jmax; ++j)
            for (int k = 3; k <= kmax; ++k) {
                const Found f = findinterface2(G, G.bp, k, j, i);
                if (f.found != 1) continue;
                const double dx = G.ddx[i], dy = G.ddy[j], dz = G.ddz[k];
                const double cx2 = findinterface2(G, G.bu, k, j, i - 1).found;
                const double cx1 = findinterface2(G, G.bu, k, j, i).found;
                const double cy2 = findinterface2(G, G.bv, k, j - 1, i).found;
                const double cy1 = findinterface2(G, G.bv, k, j, i).found;
                const double cz2 = findinterface2(G, G.bw, k - 1, j, i).found;
                const double cz1 = findinterface2(G, G.bw, k, j, i).found;
                double xvel = 0.0, yvel = 0.0, zvel = 0.0;
                const int bzc = G.bz[G.at(k, j, i)];
                auto nb = [&](int kq, int jq, int iq) { return G.bz[G.at(kq, jq, iq)]; };
                auto addvel = [&](int cell) {
                    const double* u = G.ucell + 3LL * (-cell - 1);
                    xvel = xvel + u[0];
                    yvel = yvel + u[1];
                    zvel = zvel + u[2];
                };
                if (bzc < 0) {
                    // (bzc >= -icells: checked for the whole grid beforehand)
                    const double* u = G.ucell + 3LL * (-bzc - 1);
                    xvel = u[0]; yvel = u[1]; zvel = u[2];
                } else {
                    int ngeo = 0;
                    const int tx1 = nb(k, j, i + 1), tx2 = nb(k, j, i - 1), ty1 = nb(k, j + 1, i),
                              ty2 = nb(k, j - 1, i), tz1 = nb(k + 1, j, i), tz2 = nb(k - 1, j, i);
                    if (f.x1 == 1 && tx1 < 0) ngeo++;
                    if (f.x2 == 1 && tx2 < 0) ngeo++;
                    if (f.y1 == 1 && ty1 < 0) ngeo++;
                    if (f.y2 == 1 && ty2 < 0) ngeo++;
                    if (f.z1 == 1 && tz1 < 0) ngeo++;
                    if (f.z2 == 1 && tz2 < 0) ngeo++;
                    if (ngeo == 0) {
                        if (f.x1 == 0 && tx1 < 0) ngeo--;
                        if (f.x2 == 0 && tx2 < 0) ngeo--;
                        if (f.y1 == 0 && ty1 < 0) ngeo--;
                        if (f.y2 == 0 && ty2 < 0) ngeo--;
                        if (f.z1 == 0 && tz1 < 0) ngeo--;
                        if (f.z2 == 0 && tz2 < 0) ngeo--;
                    }
                    if (ngeo > 0) {
                        if (f.x1 == 1 && tx1 < 0) addvel(tx1);
                        if (f.x2 == 1 && tx2 < 0) addvel(tx2);
                        if (f.y1 == 1 && ty1 < 0) addvel(ty1);
                        if (f.y2 == 1 && ty2 < 0) addvel(ty2);
                        if (f.z1 == 1 && tz1 < 0) addvel(tz1);
                        if (f.z2 == 1 && tz2 < 0) addvel(tz2);
                        xvel = xvel / (double)ngeo;
                        yvel = yvel / (double)ngeo;
                        zvel = zvel / (double)ngeo;
                    } else if (ngeo < 0) {
                        if (f.x1 == 0 && tx1 < 0) addvel(tx1);
                        if (f.x2 == 0 && tx2 < 0) addvel(tx2);
                        if (f.y1 == 0 && ty1 < 0) addvel(ty1);
                        if (f.y2 == 0 && ty2 < 0) addvel(ty2);
                        if (f.z1 == 0 && tz1 < 0) addvel(tz1);
                        if (f.z2 == 0 && tz2 < 0) addvel(tz2);
                        xvel = -xvel / (double)ngeo;
                        yvel = -yvel / (double)ngeo;
                        zvel = -zvel / (double)ngeo;
                    }
                }
                const double acoeff = (1.0 - cx1) * xvel * dy * dz - (1.0 - cx2) * xvel * dy * dz +
                                      (1.0 - cy1) * yvel * dx * dz - (1.0 - cy2) * yvel * dx * dz +
                                      (1.0 - cz1) * zvel * dx * dy - (1.0 - cz2) * zvel * dx * dy;
                double ax1 = f.x1, ax2 = f.x2, ay1 = f.y1, ay2 = f.y2, az1 = f.z1, az2 = f.z2;
                if (i == 3 && wall(nfro)) ax2 = 0.0;
                if (i == G.ii - 2 && wall(nbac)) ax1 = 0.0;
                if (j == 3 && wall(nrgt)) ay2 = 0.0;
                if (j == G.jj - 2 && wall(nlft)) ay1 = 0.0;
                if (k == 3 && wall(nbot)) az2 = 0.0;
                if (k == G.kk - 2 && wall(ntop)) az1 = 0.0;
                const double sarea = ax1 * G.au[G.at(k, j, i)] + ax2 * G.au[G.at(k, j, i - 1)] +
                                     ay1 * G.av[G.at(k, j, i)] + ay2 * G.av[G.at(k, j - 1, i)] +
                                     az1 * G.aw[G.at(k, j, i)] + az2 * G.aw[G.at(k - 1, j, i)];
                const double r3 = (dx + dy + dz) / 3.0;
                const double refarea = r3 * r3;
                if (sarea > refarea * kMaccur) {
                    ax1 = ax1 * G.au[G.at(k, j, i)];
                    ax2 = ax2 * G.au[G.at(k, j, i - 1)];
                    ay1 = ay1 * G.av[G.at(k, j, i)];
                    ay2 = ay2 * G.av[G.at(k, j - 1, i)];
                    az1 = az1 * G.aw[G.at(k, j, i)];
                    az2 = az2 * G.aw[G.at(k - 1, j, i)];
                }
                L.n++;
                L.xi.push_back(f.nr);
                L.xi.push_back(G.flat1(k, j, i));
                for (double v : {ax1, ax2, ay1, ay2, az1, az2, acoeff}) L.xr.push_back(v);
            }
}

// ---- scalar stencils (src/scalar/gc_scastencils_mod.F90:127-946) ---------
// Per treated cell one standard-sized record: 9 integers {cell, body, N, N
// stencil cells, -1 for the unused of the six} and 8 reals {areabyvol, N
// coefficients, -HUGE for the unused, the additive constant}, for the
// cell-value ('C', xpolr) and the point-value ('P', xpolrvel) forms.
constexpr int kScaNperi = 6;

struct ScaLists {
    int n = 0;
    std::vector<int64_t> xi;
    std::vector<double> xr, xv;
    void record(int64_t cell, int body, int nst, const int64_t* st, double areabyvol, const double* c,
                const double* cv, double ac, double acv) {
        xi.push_back(cell);
        xi.push_back(body);
        xi.push_back(nst);
        xr.push_back(areabyvol);
        xv.push_back(areabyvol);
        for (int q = 0; q < kScaNperi; ++q) {
            const bool used = q < nst;
            xi.push_back(used ? st[q] : -1);
            xr.push_back(used ? c[q] : -DBL_MAX);
            xv.push_back(used ? cv[q] : -DBL_MAX);
        }
        xr.push_back(ac);
        xv.push_back(acv);
        ++n;
    }
};

// the cut cell idx (1-based within the grid) of a negative bzelltyp
struct ScaCut {
    const double* nvecs;     // [icells][4]
    const double* area;      // [icells]
    const int32_t* body;     // [icells]
};

// calcfluxtsca (:525-782): from the cut cell's plane a x + b y + c z = dpl,
// the cell-value stencil (the mean over the fluid part of the cell, by a
// 20^3 midpoint integration) and the point-value stencil (linear in the
// distance to the plane); 1 on success, -11 without a usable distance,
// -12 when the cell-value weights exceed 0.61, -99 on a non-finite
// coefficient (an error in the reference).
int calcfluxtsca(const GridView& G, const ScaCut& cut, int k, int j, int i, int kt, int jt, int it,
                 const std::vector<int>& is, const std::vector<int>& js, const std::vector<int>& ks,
                 int velpts, double* co, double& ac, double* cv, double& acv) {
    const double* nv = cut.nvecs + 4 * (long long)(-G.bz[G.at(kt, jt, it)] - 1);
    const double a = nv[0], b = nv[1], c = nv[2], dpl = nv[3];
    for (int n = 0; n < kScaNperi; ++n) co[n] = cv[n] = 0.0;
    ac = acv = 0.0;
    double dpoint = a * G.x[i] + b * G.y[j] + c * G.z[k] - dpl;
    double dall = 0.0, dist[kScaNperi] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int n = 0; n < velpts; ++n) {
        dist[n] = a * G.x[is[n]] + b * G.y[js[n]] + c * G.z[ks[n]] - dpl;
        if (dist[n] < std::fabs(dpoint) * (double)0.2f) dist[n] = 0.0;
        dall = dall + dist[n] * dist[n];
    }
    if (std::fabs(dall) < DBL_MIN) return -11;
    double ce[kScaNperi], cesum = 0.0;
    for (int n = 0; n < velpts; ++n) {
        ce[n] = dist[n] / dall;
        cesum = cesum + ce[n];
    }
    const int parts = 20;
    const double ddi = G.ddx[i] / parts, ddj = G.ddy[j] / parts, ddk = G.ddz[k] / parts;
    const double xs = G.xs[i - 1] - ddi / 2.0, ys = G.ys[j - 1] - ddj / 2.0, zs = G.zs[k - 1] - ddk / 2.0;
    int cvol1 = 0;
    const double dvol = ddi * ddj * ddk;
    for (int i2 = 1; i2 <= parts; ++i2) {
        const double xm = xs + ddi * (double)i2;
        for (int j2 = 1; j2 <= parts; ++j2) {
            const double ym = ys + ddj * (double)j2;
            for (int k2 = 1; k2 <= parts; ++k2) {
                const double zm = zs + ddk * (double)k2;
                const double dir = (a * xm + b * ym + c * zm) - dpl;
                if (dir > 0.0) {
                    for (int n = 0; n < velpts; ++n) co[n] = co[n] + dir * ce[n];
                    ac = ac + (1.0 - dir * cesum);
                    ++cvol1;
                }
            }
        }
    }
    if (cvol1 > 0) {
        for (int n = 0; n < velpts; ++n) co[n] = co[n] * dvol / ((double)cvol1 * dvol);
        ac = ac * dvol / ((double)cvol1 * dvol);
    } else {
        for (int n = 0; n < velpts; ++n) co[n] = 0.0;
        ac = 0.0;
    }
    dpoint = a * G.x[i] + b * G.y[j] + c * G.z[k] - dpl;
    for (int n = 0; n < velpts; ++n) cv[n] = dpoint * ce[n];
    acv = 1.0 - dpoint * cesum;
    int found = 1;
    double sum = 0.0;
    for (int n = 0; n < velpts; ++n) sum = sum + co[n];
    if (sum > (double)0.61f) found = -12;
    bool bad = !std::isfinite(acv) || !std::isfinite(ac);
    for (int n = 0; n < velpts; ++n) bad = bad || !std::isfinite(cv[n]) || !std::isfinite(co[n]);
    return bad ? -99 : found;
}

// tscastencilcoeff (:447-522): the open neighbours, the chosen stencil and
// its coefficients; the full record on success.  Returns the reference's
// found (<= 0: the caller writes the rescue record), -99 on an error.
int tscastencilcoeff(const GridView& G, const ScaCut& cut, const Ball& ball, int k, int j, int i, int kt,
                     int jt, int it, double areabyvol, int body, ScaLists& L) {
    std::vector<int> is, js, ks;
    checkneighbor(G, G.bp, k, j, i, ball, is, js, ks);
    const int velpts = choosestencil(k, j, i, is, js, ks);
    if (velpts > kScaNperi) return -2;
    if (velpts == 0) return -3;
    double co[kScaNperi], cv[kScaNperi], ac, acv;
    const int found = calcfluxtsca(G, cut, k, j, i, kt, jt, it, is, js, ks, velpts, co, ac, cv, acv);
    if (found == -99) return -99;
    for (int n = 0; n < velpts; ++n)
        if (std::fabs(cv[n]) > 12.0) return -4;
    if (found == 1) {
        int64_t st[kScaNperi];
        for (int n = 0; n < velpts; ++n) st[n] = G.flat1(ks[n], js[n], is[n]);
        L.record(G.flat1(k, j, i), body, velpts, st, areabyvol, co, cv, ac, acv);
    }
    return found;
}

// tscastencil (:127-363): every blocked interior cell with an open face
// neighbour (findinterface2) gets a stencil from the cut cell with the
// boundary information -- itself, else the face neighbour with the largest
// body id -- or the rescue record (no stencil points, constant 1: the
// cell takes the body's value); an open cut cell gets the area record (its
// interface area per volume only, for the flux condition).
int tscastencil(const GridView& G, const ScaCut& cut, const Ball& ball, ScaLists& L) {
    const int64_t none[1] = {0};
    const double zero[1] = {0.0};
    for (int i = 3; i <= G.ii - 2; ++i)
        for (int j = 3; j <= G.jj - 2; ++j)
            for (int k = 3; k <= G.kk - 2; ++k) {
                const Found f = findinterface2(G, G.bp, k, j, i);
                const int32_t bz = G.bz[G.at(k, j, i)];
                const double vol = G.ddx[i] * G.ddy[j] * G.ddz[k];
                if (!f.found) {
                    if (bz < 0 && G.bp[G.at(k, j, i)] > 0.5) {
                        // tscastencilcoeffarea (:366-444): the cell itself, weight 1
                        const double areabyvol = cut.area[-bz - 1] / vol;
                        const int64_t self[1] = {G.flat1(k, j, i)};
                        const double one[1] = {1.0};
                        L.record(G.flat1(k, j, i), cut.body[-bz - 1], 1, self, areabyvol, one, one, 0.0, 0.0);
                    }
                    continue;
                }
                int found2 = 0, kt = 0, jt = 0, it = 0, body = 0;
                if (bz < 0) {
                    it = i; jt = j; kt = k;
                    found2 = 1;
                } else {
                    const int flag[6] = {f.x1, f.x2, f.y1, f.y2, f.z1, f.z2};
                    const int off[6][3] = {{0, 0, 1}, {0, 0, -1}, {0, 1, 0}, {0, -1, 0}, {1, 0, 0}, {-1, 0, 0}};
                    for (int q = 0; q < 6; ++q) {
                        const int kq = k + off[q][0], jq = j + off[q][1], iq = i + off[q][2];
                        const int32_t bq = G.bz[G.at(kq, jq, iq)];
                        if (flag[q] == 1 && bq < 0 && cut.body[-bq - 1] > body) {
                            body = cut.body[-bq - 1];
                            it = iq; jt = jq; kt = kq;
                        }
                    }
                    if (body > 0) found2 = 1;
                }
                if (found2 == 1) {
                    const int32_t bt = G.bz[G.at(kt, jt, it)];
                    const double areabyvol = (k == kt && j == jt && i == it) ? cut.area[-bt - 1] / vol : 0.0;
                    body = cut.body[-bt - 1];
                    const int found3 = tscastencilcoeff(G, cut, ball, k, j, i, kt, jt, it, areabyvol, body, L);
                    if (found3 == -99) return MGLET_ERR_ARG;
                    // tscastencilcoeffrescue (:872-946): no points, constant 1
                    if (found3 <= 0) L.record(G.flat1(k, j, i), body, 0, none, areabyvol, zero, zero, 1.0, 1.0);
                } else {
                    L.record(G.flat1(k, j, i), 0, 0, none, 0.0, zero, zero, 1.0, 1.0);
                }
            }
    return 0;
}

}  // namespace
}  // namespace mg

extern "C" int mglet_create_scastencils(const mglet_grid_desc* d, const mglet_sca_geometry* geo,
                                        mglet_scastencils** out) {
    using namespace mg;
    if (!d || !geo || !out || d->ngrid <= 0 || !d->mgdims || !d->bctype || !d->x || !d->dx || !d->ddx ||
        !geo->bp || !geo->bzelltyp || !geo->icells) {
        set_error("create_scastencils: null argument");
        return MGLET_ERR_ARG;
    }
    long long ncut = 0;
    for (int g = 0; g < d->ngrid; ++g) {
        if (geo->icells[g] < 0) {
            set_error("create_scastencils: negative icells");
            return MGLET_ERR_ARG;
        }
        ncut += geo->icells[g];
    }
    if (ncut > 0 && (!geo->nvecs || !geo->arealist || !geo->bodyid)) {
        set_error("create_scastencils: nvecs, arealist and bodyid are needed for intersected cells");
        return MGLET_ERR_ARG;
    }
    static const Ball ball;
    auto* S = new mglet_scastencils();
    S->g.resize(d->ngrid);
    long long ip3 = 0, ipx = 0, ipy = 0, ipz = 0, ipc = 0;
    std::vector<double> xs, ys, zs;
    for (int g = 0; g < d->ngrid; ++g) {
        GridView G{};
        G.kk = d->mgdims[3 * g];
        G.jj = d->mgdims[3 * g + 1];
        G.ii = d->mgdims[3 * g + 2];
        for (int f = 0; f < 6; ++f) G.bc[f] = d->bctype[6 * g + f];
        xs.assign(G.ii + 1, 0.0);
        ys.assign(G.jj + 1, 0.0);
        zs.assign(G.kk + 1, 0.0);
        for (int i = 1; i <= G.ii; ++i) xs[i] = d->x[ipx + i - 1] + 0.5 * d->dx[ipx + i - 1];
        for (int j = 1; j <= G.jj; ++j) ys[j] = d->y[ipy + j - 1] + 0.5 * d->dy[ipy + j - 1];
        for (int k = 1; k <= G.kk; ++k) zs[k] = d->z[ipz + k - 1] + 0.5 * d->dz[ipz + k - 1];
        G.x = d->x + ipx - 1; G.y = d->y + ipy - 1; G.z = d->z + ipz - 1;
        G.xs = xs.data(); G.ys = ys.data(); G.zs = zs.data();
        G.ddx = d->ddx + ipx - 1; G.ddy = d->ddy + ipy - 1; G.ddz = d->ddz + ipz - 1;
        G.bp = geo->bp + ip3;
        G.bz = geo->bzelltyp + ip3;
        G.icells = geo->icells[g];
        const long long npts = (long long)G.kk * G.jj * G.ii;
        for (long long q = 0; q < npts; ++q)
            if (G.bz[q] < -G.icells) {
                delete S;
                set_error("create_scastencils: bzelltyp refers past the grid's intersected cells");
                return MGLET_ERR_ARG;
            }
        ScaCut cut{geo->nvecs ? geo->nvecs + 4 * ipc : nullptr, geo->arealist ? geo->arealist + ipc : nullptr,
                   geo->bodyid ? geo->bodyid + ipc : nullptr};
        ScaLists L;
        if (int rc = tscastencil(G, cut, ball, L)) {
            delete S;
            set_error("create_scastencils: a non-finite stencil coefficient");
            return rc;
        }
        auto& o = S->g[g];
        o.ncells = L.n;
        o.xi = std::move(L.xi);
        o.xr = std::move(L.xr);
        o.xv = std::move(L.xv);
        ip3 += npts;
        ipx += G.ii; ipy += G.jj; ipz += G.kk;
        ipc += G.icells;
    }
    *out = S;
    return 0;
}

extern "C" int mglet_scastencils_size(const mglet_scastencils* s, int32_t igrid, int32_t* ncells) {
    if (!s || igrid < 1 || igrid > (int)s->g.size()) {
        mg::set_error("scastencils_size: bad handle or grid");
        return MGLET_ERR_ARG;
    }
    if (ncells) *ncells = s->g[igrid - 1].ncells;
    return 0;
}

extern "C" int mglet_scastencils_copy(const mglet_scastencils* s, int32_t igrid, int64_t* xpoli,
                                      double* xpolr, double* xpolrvel) {
    if (!s || igrid < 1 || igrid > (int)s->g.size()) {
        mg::set_error("scastencils_copy: bad handle or grid");
        return MGLET_ERR_ARG;
    }
    const auto& L = s->g[igrid - 1];
    if (xpoli && !L.xi.empty()) std::memcpy(xpoli, L.xi.data(), L.xi.size() * sizeof(int64_t));
    if (xpolr && !L.xr.empty()) std::memcpy(xpolr, L.xr.data(), L.xr.size() * sizeof(double));
    if (xpolrvel && !L.xv.empty()) std::memcpy(xpolrvel, L.xv.data(), L.xv.size() * sizeof(double));
    return 0;
}

extern "C" int mglet_scastencils_free(mglet_scastencils* s) {
    delete s;
    return 0;
}

extern "C" int mglet_create_flowstencils(const mglet_grid_desc* d, const mglet_ib_geometry* geo,
                                         mglet_flowstencils** out) {
    using namespace mg;
    if (!d || !geo || !out || d->ngrid <= 0 || !d->mgdims || !d->bctype || !d->x || !d->dx ||
        !d->ddx || !geo->bp || !geo->bu || !geo->bv || !geo->bw || !geo->areau || !geo->areav ||
        !geo->areaw || !geo->bzelltyp || !geo->icells) {
        set_error("create_flowstencils: null argument");
        return MGLET_ERR_ARG;
    }
    const int ng = d->ngrid;
    long long ncut = 0;
    for (int g = 0; g < ng; ++g) {
        if (geo->icells[g] < 0) {
            set_error("create_flowstencils: negative icells");
            return MGLET_ERR_ARG;
        }
        ncut += geo->icells[g];
    }
    if (ncut > 0 && (!geo->nvecs || !geo->ucell)) {
        set_error("create_flowstencils: nvecs and ucell are needed for intersected cells");
        return MGLET_ERR_ARG;
    }
    static const Ball ball;
    auto* S = new mglet_flowstencils();
    S->g.resize(ng);
    long long ip3 = 0, ipx = 0, ipy = 0, ipz = 0, ipc = 0;
    std::vector<double> xs, ys, zs;
    for (int g = 0; g < ng; ++g) {
        GridView G;
        G.kk = d->mgdims[3 * g];
        G.jj = d->mgdims[3 * g + 1];
        G.ii = d->mgdims[3 * g + 2];
        for (int f = 0; f < 6; ++f) G.bc[f] = d->bctype[6 * g + f];
        // calc_stag (corefields_mod.F90:176-192)
        xs.assign(G.ii + 1, 0.0);
        ys.assign(G.jj + 1, 0.0);
        zs.assign(G.kk + 1, 0.0);
        for (int i = 1; i <= G.ii; ++i) xs[i] = d->x[ipx + i - 1] + 0.5 * d->dx[ipx + i - 1];
        for (int j = 1; j <= G.jj; ++j) ys[j] = d->y[ipy + j - 1] + 0.5 * d->dy[ipy + j - 1];
        for (int k = 1; k <= G.kk; ++k) zs[k] = d->z[ipz + k - 1] + 0.5 * d->dz[ipz + k - 1];
        G.x = d->x + ipx - 1; G.y = d->y + ipy - 1; G.z = d->z + ipz - 1;
        G.xs = xs.data(); G.ys = ys.data(); G.zs = zs.data();
        G.ddx = d->ddx + ipx - 1; G.ddy = d->ddy + ipy - 1; G.ddz = d->ddz + ipz - 1;
        G.bp = geo->bp + ip3; G.bu = geo->bu + ip3; G.bv = geo->bv + ip3; G.bw = geo->bw + ip3;
        G.au = geo->areau + ip3; G.av = geo->areav + ip3; G.aw = geo->areaw + ip3;
        G.bz = geo->bzelltyp + ip3;
        G.icells = geo->icells[g];
        G.nvecs = geo->nvecs ? geo->nvecs + 4 * ipc : nullptr;
        G.ucell = geo->ucell ? geo->ucell + 3 * ipc : nullptr;
        const long long npts = (long long)G.kk * G.jj * G.ii;
        for (long long q = 0; q < npts; ++q)
            if (G.bz[q] < -G.icells) {
                delete S;
                set_error("create_flowstencils: bzelltyp refers past the grid's intersected cells");
                return MGLET_ERR_ARG;
            }
        Lists L[4];
        fluxcorrection(G, L[3]);
        fluxstencil(G, G.bu, 1, ball, L[0]);
        fluxstencil(G, G.bv, 2, ball, L[1]);
        fluxstencil(G, G.bw, 3, ball, L[2]);
        for (int c = 0; c < 4; ++c) {
            auto& o = S->g[g][c];
            o.ncells = L[c].n;
            o.xi = std::move(L[c].xi);
            o.xr = std::move(L[c].xr);
            o.xv = std::move(L[c].xv);
        }
        ip3 += npts;
        ipx += G.ii; ipy += G.jj; ipz += G.kk;
        ipc += G.icells;
    }
    *out = S;
    return 0;
}

extern "C" int mglet_flowstencils_size(const mglet_flowstencils* s, int32_t igrid, int32_t comp,
                                       int32_t* ncells, int64_t* nxi, int64_t* nxr) {
    if (!s || igrid < 1 || igrid > (int)s->g.size() || comp < 1 || comp > 4) {
        mg::set_error("flowstencils_size: bad handle, grid or component");
        return MGLET_ERR_ARG;
    }
    const auto& L = s->g[igrid - 1][comp - 1];
    if (ncells) *ncells = L.ncells;
    if (nxi) *nxi = (int64_t)L.xi.size();
    if (nxr) *nxr = (int64_t)L.xr.size();
    return 0;
}

extern "C" int mglet_flowstencils_copy(const mglet_flowstencils* s, int32_t igrid, int32_t comp,
                                       int64_t* xpoli, double* xpolr, double* xpolrvel) {
    if (!s || igrid < 1 || igrid > (int)s->g.size() || comp < 1 || comp > 4) {
        mg::set_error("flowstencils_copy: bad handle, grid or component");
        return MGLET_ERR_ARG;
    }
    const auto& L = s->g[igrid - 1][comp - 1];
    if (xpoli && !L.xi.empty()) std::memcpy(xpoli, L.xi.data(), L.xi.size() * sizeof(int64_t));
    if (xpolr && !L.xr.empty()) std::memcpy(xpolr, L.xr.data(), L.xr.size() * sizeof(double));
    if (xpolrvel && !L.xv.empty()) std::memcpy(xpolrvel, L.xv.data(), L.xv.size() * sizeof(double));
    return 0;
}

extern "C" int mglet_flowstencils_free(mglet_flowstencils* s) {
    delete s;
    return 0;
}
