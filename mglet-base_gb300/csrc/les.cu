// les.cu -- the LES models of lesmodel_mod.F90 (plain FP64 form): the
// effective viscosity G = rho delta^2 D_m + gmol of efvisc_gc (:200-365)
// with the Smagorinsky (:368-390), WALE (:393-487) or sigma (:490-517)
// operator D_m, one thread per interior cell; the filter width delta = cbrt(cell volume) is
// taken once on the host with the C library's cbrt, the routine the
// reference calls (simdfunctions_mod.F90:165-180), and kept as the field
// LESD.  After efvisc: per level parent, bound and connect of G, setginbody
// (ghost-cell IB only; with BP = 1 it leaves G unchanged) and the corner
// connect tstle4 reads (lesmodel_gc :108-197).  Built without FMA
// contraction, so that G of Smagorinsky and WALE matches the CPU
// restatement bit for bit (sigma to the ulps of CUDA's pow, acos, cos).

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "internal.h"
#include "mixed.h"

namespace mg {
namespace {

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

struct LesArgs {
    const DevGrid* grids;
    const double *u, *v, *w, *bp, *delta;
    double* g;
    const double *dx, *dy, *dz, *ddx, *ddy, *ddz, *rddx, *rddy, *rddz;
    double gmol, rho, cm, tol;
    double cpo6, cpo11, cpo12;   // gradp2 (wernerwengle_mod.F90:36-61)
    double pi;                   // 4 atan(1), taken on the host
    int model;
};

__device__ __forceinline__ double sabs(const double* a) {
    return sqrt(a[0] * a[0] + a[4] * a[4] + a[8] * a[8] + 0.5 * ((a[3] + a[1]) * (a[3] + a[1])) +
                0.5 * ((a[6] + a[2]) * (a[6] + a[2])) + 0.5 * ((a[7] + a[5]) * (a[7] + a[5])));
}

__device__ double wale(double cm, double tol, const double* gr) {
    const double dudx = gr[0], dudy = gr[1], dudz = gr[2], dvdx = gr[3], dvdy = gr[4], dvdz = gr[5];
    const double dwdx = gr[6], dwdy = gr[7], dwdz = gr[8];
    const double third = (double)(1.0f / 3.0f);   // (1.0/3.0) of default-kind literals
    const double tr = dudx * dudx + dudy * dvdx + dudz * dwdx + dvdx * dudy + dvdy * dvdy + dvdz * dwdy +
                      dwdx * dudz + dwdy * dvdz + dwdz * dwdz;
    const double s00 = 0.5 * (dudx * dudx + dudy * dvdx + dudz * dwdx + dudx * dudx + dudy * dvdx + dudz * dwdx) -
                       third * tr;
    const double s01 = 0.5 * (dudx * dudy + dudy * dvdy + dudz * dwdy + dvdx * dudx + dvdy * dvdx + dvdz * dwdx);
    const double s02 = 0.5 * (dudx * dudz + dudy * dvdz + dudz * dwdz + dwdx * dudx + dwdy * dvdx + dwdz * dwdx);
    const double s11 = 0.5 * (dvdx * dudy + dvdy * dvdy + dvdz * dwdy + dvdx * dudy + dvdy * dvdy + dvdz * dwdy) -
                       third * tr;
    const double s12 = 0.5 * (dvdx * dudz + dvdy * dvdz + dvdz * dwdz + dwdx * dudy + dwdy * dvdy + dwdz * dwdy);
    const double s22 = 0.5 * (dwdx * dudz + dwdy * dvdz + dwdz * dwdz + dwdx * dudz + dwdy * dvdz + dwdz * dwdz) -
                       third * tr;
    const double sd = sqrt(s00 * s00 + 2 * (s01 * s01) + 2 * (s02 * s02) + s11 * s11 + 2 * (s12 * s12) + s22 * s22);
    const double sa = sabs(gr);
    const double root = sqrt(sd);
    if (root < tol * sa) return 0.0;
    const double x = root == 0.0 ? 0.0 : sa / root;
    const double x2 = x * x, x3 = x2 * x;
    return cm * cm * root / (x3 * x2 + 1.0);
}

// sigma (lesmodel_mod.F90:490-517) with the tensor products of
// tensormath_mod.F90 and the analytic eigenvalues of eig_b (:221-268); pow,
// acos and cos are CUDA's, within a few ulp of the C library's the
// reference calls
__device__ double sigma(double cm, double pi, const double* gr) {
    double g[3][3];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) g[c][r] = gr[3 * c + r];
    double G[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double a = 0.0;
            for (int k = 0; k < 3; ++k) a = a + g[k][i] * g[k][j];
            G[i][j] = a;
        }
#define AT(r, c) G[(c) - 1][(r) - 1]
    const double q11 = AT(1, 1) * AT(1, 1) + AT(2, 1) * AT(1, 2) + AT(3, 1) * AT(1, 3);
    const double q22 = AT(1, 2) * AT(2, 1) + AT(2, 2) * AT(2, 2) + AT(3, 2) * AT(2, 3);
    const double q33 = AT(1, 3) * AT(3, 1) + AT(2, 3) * AT(3, 2) + AT(3, 3) * AT(3, 3);
    const double i1 = AT(1, 1) + AT(2, 2) + AT(3, 3);
    const double i2 = 0.5 * (i1 * i1 - (q11 + q22 + q33));
    const double i3 = AT(1, 1) * (AT(2, 2) * AT(3, 3) - AT(3, 2) * AT(2, 3)) -
                      AT(2, 1) * (AT(1, 2) * AT(3, 3) - AT(3, 2) * AT(1, 3)) +
                      AT(3, 1) * (AT(1, 2) * AT(2, 3) - AT(2, 2) * AT(1, 3));
#undef AT
    double a1 = i1 * i1 / 9.0 - i2 / 3.0;
    const double a2 = i1 * i1 * i1 / 27.0 - (i1 * i2) / 6.0 + i3 / 2.0;
    a1 = a1 < 0.0 ? 0.0 : a1;
    const double den = pow(a1, 3.0 / 2.0);
    double arg = den == 0.0 ? 0.0 : a2 / den;
    arg = arg > 1.0 ? 1.0 : (arg < -1.0 ? -1.0 : arg);
    const double a3 = (1.0 / 3.0) * acos(arg);
    double e1 = i1 / 3.0 + 2.0 * sqrt(a1) * cos(a3);
    double e2 = i1 / 3.0 - 2.0 * sqrt(a1) * cos(pi / 3.0 + a3);
    double e3 = i1 / 3.0 - 2.0 * sqrt(a1) * cos(pi / 3.0 - a3);
    e1 = e1 < 0.0 ? 0.0 : e1;
    e2 = e2 < 0.0 ? 0.0 : e2;
    e3 = e3 < 0.0 ? 0.0 : e3;
    const double s1 = sqrt(e1), s2 = sqrt(e2), s3 = sqrt(e3);
    const double num = s3 * (s1 - s2) * (s2 - s3), d1 = s1 * s1;
    return cm * cm * (d1 == 0.0 ? 0.0 : num / d1);
}

__device__ __forceinline__ double gradp2(const LesArgs& A, double uquer, double dds) {
    const double uquern = fabs(uquer);
    const double vz = copysign(1.0, uquer);
    const double rdds = 1.0 / dds;
    if (uquern >= A.cpo6 * rdds) return rdds * (A.cpo12 * uquern + A.cpo11 * rdds) * vz;
    return 2.0 * uquern / dds * vz;
}

__global__ void k_efvisc(LesArgs A) {
    const DevGrid G = A.grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj * nk) return;
    const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
    const long long o = G.ip3;
    const double *u = A.u + o, *v = A.v + o, *w = A.w + o;
    const double *dx = A.dx + G.ipx - 1, *dy = A.dy + G.ipy - 1, *dz = A.dz + G.ipz - 1;
    const double *ddx = A.ddx + G.ipx - 1, *ddy = A.ddy + G.ipy - 1, *ddz = A.ddz + G.ipz - 1;
    const double *rddx = A.rddx + G.ipx - 1, *rddy = A.rddy + G.ipy - 1, *rddz = A.rddz + G.ipz - 1;
#define F(a, k, j, i) a[IX(k, j, i)]
    double gr[9];
    const double dxf = 0.25 * dx[i - 1] * rddx[i];
    gr[0] = (F(u, k, j, i) - F(u, k, j, i - 1)) * rddx[i];
    gr[1] = ((F(u, k, j + 1, i) - F(u, k, j - 1, i)) * dxf + (F(u, k, j + 1, i - 1) - F(u, k, j - 1, i - 1)) * (0.5 - dxf)) * rddy[j];
    gr[2] = ((F(u, k + 1, j, i) - F(u, k - 1, j, i)) * dxf + (F(u, k + 1, j, i - 1) - F(u, k - 1, j, i - 1)) * (0.5 - dxf)) * rddz[k];
    const double dyf = 0.25 * dy[j - 1] * rddy[j];
    gr[3] = ((F(v, k, j, i + 1) - F(v, k, j, i - 1)) * dyf + (F(v, k, j - 1, i + 1) - F(v, k, j - 1, i - 1)) * (0.5 - dyf)) * rddx[i];
    gr[4] = (F(v, k, j, i) - F(v, k, j - 1, i)) * rddy[j];
    gr[5] = ((F(v, k + 1, j, i) - F(v, k - 1, j, i)) * dyf + (F(v, k + 1, j - 1, i) - F(v, k - 1, j - 1, i)) * (0.5 - dyf)) * rddz[k];
    const double dzf = 0.25 * dz[k - 1] * rddz[k];
    gr[6] = ((F(w, k, j, i + 1) - F(w, k, j, i - 1)) * dzf + (F(w, k - 1, j, i + 1) - F(w, k - 1, j, i - 1)) * (0.5 - dzf)) * rddx[i];
    gr[7] = ((F(w, k, j + 1, i) - F(w, k, j - 1, i)) * dzf + (F(w, k - 1, j + 1, i) - F(w, k - 1, j - 1, i)) * (0.5 - dzf)) * rddy[j];
    gr[8] = (F(w, k, j, i) - F(w, k - 1, j, i)) * rddz[k];
    const double delta = A.delta[o + IX(k, j, i)] * A.bp[o + IX(k, j, i)];
    // the NOS corrections (:261-330), in the reference's order
    const int nfro = G.bc[0], nbac = G.bc[1], nrgt = G.bc[2], nlft = G.bc[3], nbot = G.bc[4], ntop = G.bc[5];
    if (nfro == 5 || nbac == 5 || nrgt == 5 || nlft == 5 || nbot == 5 || ntop == 5) {
        const double dyf2 = 0.5 * dy[j - 1] * rddy[j], dzf2 = 0.5 * dz[k - 1] * rddz[k];
        const double dxf2 = 0.5 * dx[i - 1] * rddx[i];
        const double vm = dyf2 * F(v, k, j, i) + (1.0 - dyf2) * F(v, k, j - 1, i);
        const double wm = dzf2 * F(w, k, j, i) + (1.0 - dzf2) * F(w, k - 1, j, i);
        const double um = dxf2 * F(u, k, j, i) + (1.0 - dxf2) * F(u, k, j, i - 1);
        if (nfro == 5 && i == 3) { gr[3] = gradp2(A, vm, ddx[i]); gr[6] = gradp2(A, wm, ddx[i]); }
        if (nbac == 5 && i == ii - 2) { gr[3] = -gradp2(A, vm, ddx[i]); gr[6] = -gradp2(A, wm, ddx[i]); }
        if (nrgt == 5 && j == 3) { gr[1] = gradp2(A, um, ddy[j]); gr[7] = gradp2(A, wm, ddy[j]); }
        if (nlft == 5 && j == jj - 2) { gr[1] = -gradp2(A, um, ddy[j]); gr[7] = -gradp2(A, wm, ddy[j]); }
        if (nbot == 5 && k == 3) { gr[2] = gradp2(A, um, ddz[k]); gr[5] = gradp2(A, vm, ddz[k]); }
        if (ntop == 5 && k == kk - 2) { gr[2] = -gradp2(A, um, ddz[k]); gr[5] = -gradp2(A, vm, ddz[k]); }
    }
#undef F
    const double dm = A.model == 1 ? A.cm * A.cm * sqrt(2.0) * sabs(gr)
                                   : (A.model == 2 ? wale(A.cm, A.tol, gr) : sigma(A.cm, A.pi, gr));
    A.g[o + IX(k, j, i)] = A.rho * (delta * delta) * dm + A.gmol;
}

// setginbody (lesmodel_mod.F90:543-570): in place and in loop order, one
// thread per grid walking its cells as the reference does
__global__ void k_setginbody(const DevGrid* __restrict__ grids, double* Gf, const double* __restrict__ BPF,
                             int ngrid) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= ngrid) return;
    const DevGrid G = grids[gi];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    double* g = Gf + G.ip3;
    const double* bp = BPF + G.ip3;
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                double nn = bp[IX(k, j, i + 1)] + bp[IX(k, j, i - 1)] + bp[IX(k, j + 1, i)] + bp[IX(k, j - 1, i)] +
                            bp[IX(k + 1, j, i)] + bp[IX(k - 1, j, i)];
                nn = nn < 1.0 ? 1.0 : nn;
                const double gbpn = (g[IX(k, j, i + 1)] * bp[IX(k, j, i + 1)] + g[IX(k, j, i - 1)] * bp[IX(k, j, i - 1)] +
                                     g[IX(k, j + 1, i)] * bp[IX(k, j + 1, i)] + g[IX(k, j - 1, i)] * bp[IX(k, j - 1, i)] +
                                     g[IX(k + 1, j, i)] * bp[IX(k + 1, j, i)] + g[IX(k - 1, j, i)] * bp[IX(k - 1, j, i)]) /
                                    nn;
                g[IX(k, j, i)] = bp[IX(k, j, i)] * g[IX(k, j, i)] + (1.0 - bp[IX(k, j, i)]) * gbpn;
            }
}

#undef IX

}  // namespace

int lesmodel(Ctx* c) {
    if (c->ilesmodel == 0) return 0;
    ProfScope ps_(c, "lesmodel");
    LesArgs A{};
    A.grids = c->d_grids;
    A.u = c->F("U"); A.v = c->F("V"); A.w = c->F("W"); A.bp = c->F("BP"); A.delta = c->F("LESD");
    A.g = c->F("G");
    A.dx = c->L("DX"); A.dy = c->L("DY"); A.dz = c->L("DZ");
    A.ddx = c->L("DDX"); A.ddy = c->L("DDY"); A.ddz = c->L("DDZ");
    A.rddx = c->L("RDDX"); A.rddy = c->L("RDDY"); A.rddz = c->L("RDDZ");
    A.gmol = c->prm.gmol;
    A.rho = c->prm.rho;
    A.cm = c->cm;
    A.model = c->ilesmodel;
    A.tol = 1.0 / std::pow(std::numeric_limits<double>::max(), 1.0 / 6.0);
    A.pi = 4.0 * std::atan(1.0);
    // init_wernerwengle (wernerwengle_mod.F90:13-28)
    const double cwa = 8.3, cwb = 1.0 / 7.0, cpo1 = 1.0 - cwb, cpo2 = 1.0 + cwb;
    A.cpo6 = 0.5 * A.gmol / A.rho * std::pow(cwa, 2.0 / cpo1);
    A.cpo11 = 2.0 * A.cpo6 * cwb * cpo1 / std::pow(2.0, cwb);
    A.cpo12 = cwb * cpo2 / std::pow(2.0, cwb - 1.0);
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, (g.kk - 4) * (g.jj - 4) * (g.ii - 4));
    k_efvisc<<<dim3((m + 255) / 256, c->ngrid), 256, 0, c->stream>>>(A);
    MG_LAUNCHED(c);
    static const char* const none[3] = {nullptr, nullptr, nullptr};
    static const char* const sg[3] = {"G", nullptr, nullptr};
    double* Gf = c->F("G");
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        if (int rc = launch_parent(c, l, none, sg, false)) return rc;
        if (int rc = launch_bound_g(c, l)) return rc;
        if (int rc = connect(c, l, 1, nullptr, nullptr, nullptr, Gf, nullptr, nullptr, false, false, 0))
            return rc;
    }
    if (c->ibtype == 1) {
        k_setginbody<<<(c->ngrid + 63) / 64, 64, 0, c->stream>>>(c->d_grids, Gf, c->F("BP"), c->ngrid);
        MG_LAUNCHED(c);
    }
    return connect(c, 0, 1, nullptr, nullptr, nullptr, Gf, nullptr, nullptr, true, false, 0);
}

// the LES model of the stage (init_lesmodel, lesmodel_mod.F90:34-84):
// 0 none, 1 smagorinsky, 2 wale; cm < 0 takes the model's default (the
// default-kind literals 0.1 and 0.5)
int set_lesmodel(Ctx* c, int model, double cm) {
    if (model != 0 && model != 1 && model != 2 && model != 5) {
        set_error("set_lesmodel: model 0 (none), 1 (smagorinsky), 2 (wale) or 5 (sigma)");
        return MGLET_ERR_ARG;
    }
    c->ilesmodel = model;
    // the mixed form's fluxes read G at every point from now on, and the
    // captured stage is rebuilt with (or without) the LES model's steps
    if (c->prm.form == MGLET_FORM_MIXED) mixed_g_field(c);
    c->cm = cm < 0.0 ? (model == 1 ? (double)0.1f : (model == 2 ? 0.5 : (double)1.35f)) : cm;
    if (model == 0) return init_viscosity(c);
    if (!c->f3.count("LESD")) {
        if (int rc = alloc_field3(c, "LESD")) return rc;
        std::vector<double> hx(c->idimx), hy(c->idimy), hz(c->idimz), d(c->idim3d, 0.0);
        MG_CUDA(copy_on(c->stream, hx.data(), c->L("DDX"), hx.size() * sizeof(double), cudaMemcpyDeviceToHost));
        MG_CUDA(copy_on(c->stream, hy.data(), c->L("DDY"), hy.size() * sizeof(double), cudaMemcpyDeviceToHost));
        MG_CUDA(copy_on(c->stream, hz.data(), c->L("DDZ"), hz.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (const DevGrid& G : c->grids)
            for (int i = 1; i <= G.ii; ++i)
                for (int j = 1; j <= G.jj; ++j)
                    for (int k = 1; k <= G.kk; ++k)
                        d[G.ip3 + (long long)(i - 1) * G.kk * G.jj + (long long)(j - 1) * G.kk + (k - 1)] =
                            std::cbrt(hx[G.ipx + i - 1] * hy[G.ipy + j - 1] * hz[G.ipz + k - 1]);
        MG_CUDA(copy_on(c->stream, c->F("LESD"), d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    return lesmodel(c);
}

}  // namespace mg
