// mixed_flux.cu -- momentum right-hand side and RK update of the mixed form.
//
// Same discretisation as tstle4 (src/flow/tstle4_mod.F90:139-529: skew-
// symmetric convection with interpolated mass fluxes, viscous fluxes with
// the harmonic face viscosity, pressure gradient) followed by rkstep
// (src/core/rungekutta_mod.F90:315-333), fused into one pass per grid, with
// the arithmetic reorganised for GB300:
//
//  * u, v, w, p stay FP64 in HBM.  Each value is split once, with integer
//    operations only, into an FP32 pair (hi, lo) with x = hi + lo to about
//    2^-48 relative.  Every stencil difference is then formed in FP32 as
//    (hi_a - hi_b) + (lo_a - lo_b): the hi difference of neighbouring values
//    is exact, so the differences carry ~FP32 relative accuracy *of the
//    difference*, and the convective term is written around the centre value
//    (c * div(mass flux) + 1/2 sum f * delta) so that nothing cancels in FP32.
//    The FP64 units of this part issue ~2 instructions/clk/SM; this form
//    needs only the 3 FP64 adds of the RK update per cell.
//  * the 2N-storage register DU is kept in FP32 (it only ever carries
//    dt * rhs); u = u + dtfu * du is the one FP64 operation per component.
//  * the grid is swept plane by plane in i with 3-plane windows of (hi, lo)
//    in shared memory; every thread owns one (k, j) column and keeps the raw
//    FP64 value of its own points for the update, so u is updated exactly.
//
// Requires a viscosity field without an LES model (G = gmol inside every
// grid): away from faces without a neighbour the diffusive harmonic means
// collapse to one host-computed constant.  Grids with FIX, OP1, NOS, SLI or
// PAR faces take a second instantiation that reads G on their outermost
// interior layer, drops the wall-normal flux points tstle4 does not compute
// and adds the Werner-Wengle wall shear of NOS faces; on grids with a PAR
// face it writes the fluxes to UO, VO, WO instead, for tstle4_par and the
// separate RK update.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <string>

#include "internal.h"

namespace mg {
namespace {

// x (FP64, normal or zero, |x| < 2^127) -> (hi, lo) FP32 with
// hi = x truncated to 24 significant bits, lo = rest (29 bits) rounded to 24.
__device__ __forceinline__ float2 split64(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF);
    const unsigned long long m = b & 0x000FFFFFFFFFFFFFULL;
    const int fe = e - 1023 + 127;
    if (e == 0 || fe <= 0) return make_float2(__uint_as_float(sign), __uint_as_float(sign));
    const float hi = __uint_as_float(sign | ((unsigned int)fe << 23) | (unsigned int)(m >> 29));
    const unsigned int rem = (unsigned int)(m & 0x1FFFFFFFu);            // 29 bits
    // weight of rem's lsb: 2^(e-1023-52), i.e. biased float exponent fe-52
    const int le = fe - 52;
    float lo = 0.f;
    if (rem != 0 && le > 0) {
        const float scale = __uint_as_float((unsigned int)le << 23);
        lo = __uint2float_rn(rem) * scale;
        lo = __uint_as_float(__float_as_uint(lo) | sign);
    }
    return make_float2(hi, lo);
}

__device__ __forceinline__ float dif(float2 a, float2 b) { return (a.x - b.x) + (a.y - b.y); }
__device__ __forceinline__ float val(float2 a) { return a.x + a.y; }

struct FluxArgs {
    const DevGrid* grids;
    const double *U0, *V0, *W0, *P0;   // read
    double *U, *V, *W;                 // written (interior)
    float *DU, *DV, *DW;               // FP32 RK registers
    // FP32 spacing tables per axis, concatenated like the FP64 arrays:
    // [0] d, [1] dd, [2] rd, [3] rdd, [4] d(i)/dd(i+1), [5] d(i-1)/dd(i)
    const float *sx, *sy, *sz;
    long long nx, ny, nz;     // stride between the 6 tables of an axis
    float g, gh;                       // uniform face viscosities (ge=gw, gn.. harmonic sum)
    float rrho;
    float gpx, gpy, gpz;
    const double* sprm;                // [0] frhs, [1] dt*fu (device)
    // grids with faces that have no neighbour (walls, inflow, outflow):
    // the viscosity field read next to those faces, the FP64 cell widths
    // and width**(-1/7) of the wall function, the Werner-Wengle constants
    const double* G;
    const double *ddx, *ddy, *ddz, *wwx, *wwy, *wwz;
    // grids with a PAR face: their fluxes go to UO, VO, WO (tstle4_par and
    // the RK update follow in separate kernels)
    double *UO, *VO, *WO;
    double wrho, wgmol, cpo4, cpo5, cpo6, cpo8;
    // ghost-cell IB: per grid 1 where the transported velocities are the
    // point values PWU, PWV, PWW (PU0, PV0, PW0), loaded into windows of
    // their own (pw: the launch has those windows)
    const unsigned char* pwflag;
    const double *PU0, *PV0, *PW0;
    int pw;
    // per grid {1, h2} where G is one value on the box 2..n-1: the uniform
    // face viscosities hold there too
    const double* guni;
    int gall;                          // G is a field (LES or uploaded): every point of a grid
                                       // whose G is not one value reads it
    int iles;                          // an LES model is on: tstle4_diff's cross term
    int* err;                          // set when a bulk-copy wait gives up
    int skip_plane;                    // test switch: this plane's copy is not issued (0: none)
    int nslab;                         // j-slabs (CTAs) per grid
};

// j- and k-dependent spacing factors of one thread's (k, j) column
struct Col {
    float dy_j, ddy_j, rdy_j, rdy_jm, rddy_j, rddy_jp, ry1, ry0;
    float dz_k, ddz_k, rdz_k, rdz_km, rddz_k, rddz_kp, rz1, rz0;
};

__device__ __forceinline__ Col column(const float* Y, long long ny, int j, const float* Z,
                                      long long nz, int k) {
    Col c;
    c.dy_j = Y[j]; c.ddy_j = Y[ny + j]; c.rdy_j = Y[2 * ny + j]; c.rdy_jm = Y[2 * ny + j - 1];
    c.rddy_j = Y[3 * ny + j]; c.rddy_jp = Y[3 * ny + j + 1];
    c.ry1 = Y[4 * ny + j]; c.ry0 = Y[5 * ny + j];
    c.dz_k = Z[k]; c.ddz_k = Z[nz + k]; c.rdz_k = Z[2 * nz + k]; c.rdz_km = Z[2 * nz + k - 1];
    c.rddz_k = Z[3 * nz + k]; c.rddz_kp = Z[3 * nz + k + 1];
    c.rz1 = Z[4 * nz + k]; c.rz0 = Z[5 * nz + k];
    return c;
}

// Face viscosities of one component (east, west, north, south, top, bottom)
struct Visc {
    float e, w, n, s, t, b;
};
struct Visc3 {
    Visc u, v, w;
};

#define DX(i) X[(i)]
#define DDX(i) X[nx + (i)]
#define RDX(i) X[2 * nx + (i)]
#define RDDX(i) X[3 * nx + (i)]
#define RX1(i) X[4 * nx + (i)]
#define RX0(i) X[5 * nx + (i)]

// uo, vo, wo of the thread's point (window position q) on plane i from the
// three-plane windows of (hi, lo) pairs (u, v, w: slots (i-1)%3, i%3,
// (i+1)%3; p: slots i%2, (i+1)%2)
// kW: the face viscosities come from vs (grids with boundary faces); else
// every face has the uniform a.g / a.gh.  gfl is the grid's gradpflag.
// kPW: the transported velocities are the point values in the windows xu,
// xv, xw (ghost-cell IB), the transporting ones U, V, W in su, sv, sw; else
// both are su, sv, sw and xu.. are not read.
template <bool kW, bool kPW = false>
__device__ __forceinline__ void flux_point(const FluxArgs& a, const float* X, long long nx,
                                           const Col& cl, const float2* su, const float2* sv,
                                           const float2* sw, const float2* sp, int plane, int pk,
                                           int q, int i, float gfl, const Visc3& vs, float& uo,
                                           float& vo, float& wo, const float2* xu = nullptr,
                                           const float2* xv = nullptr, const float2* xw = nullptr) {
    const float g = a.g, gh = a.gh;
    const float dy_j = cl.dy_j, ddy_j = cl.ddy_j, rdy_j = cl.rdy_j, rdy_jm = cl.rdy_jm;
    const float rddy_j = cl.rddy_j, rddy_jp = cl.rddy_jp, ry1 = cl.ry1, ry0 = cl.ry0;
    const float dz_k = cl.dz_k, ddz_k = cl.ddz_k, rdz_k = cl.rdz_k, rdz_km = cl.rdz_km;
    const float rddz_k = cl.rddz_k, rddz_kp = cl.rddz_kp, rz1 = cl.rz1, rz0 = cl.rz0;
    const int sm1 = (i - 1) % 3, s0 = i % 3, sp1 = (i + 1) % 3;
    const int p0 = i % 2, p1 = (i + 1) % 2;
        const float2* u_m = su + sm1 * plane;
        const float2* u_0 = su + s0 * plane;
        const float2* u_p = su + sp1 * plane;
        const float2* v_m = sv + sm1 * plane;
        const float2* v_0 = sv + s0 * plane;
        const float2* v_p = sv + sp1 * plane;
        const float2* w_m = sw + sm1 * plane;
        const float2* w_0 = sw + s0 * plane;
        const float2* w_p = sw + sp1 * plane;
        const float2* p_0 = sp + p0 * plane;
        const float2* p_p = sp + p1 * plane;
        const int qs = q - pk, qn = q + pk, qb = q - 1, qt = q + 1;   // j-1, j+1, k-1, k+1
        const float fdx_i = DX(i), fddx = DDX(i), rdx_i = RDX(i), rdx_im = RDX(i - 1);
        const float rddx_i = RDDX(i), rddx_ip = RDDX(i + 1), rx1 = RX1(i), rx0 = RX0(i);
        const float fdy_j = dy_j, fddy = ddy_j, fdz_k = dz_k, fddz = ddz_k;
        // the transported velocities (the point values under the ghost-cell
        // IB), which the LES cross term differentiates
        const float2* tu_m = kPW ? xu + sm1 * plane : u_m;
        const float2* tu_0 = kPW ? xu + s0 * plane : u_0;
        const float2* tv_0 = kPW ? xv + s0 * plane : v_0;
        const float2* tv_p = kPW ? xv + sp1 * plane : v_p;
        const float2* tw_0 = kPW ? xw + s0 * plane : w_0;
        const float2* tw_p = kPW ? xw + sp1 * plane : w_p;
        const bool cross = kW && a.iles;
        // ---------------- U at (k, j, i+1/2)
        {
            // transporting U along x (mass fluxes fe, fw), transported u
            const float2 ct = u_0[q];
            const float tE = dif(u_p[q], ct), tW = dif(u_m[q], ct);
            float2 c = ct;
            float dE = tE, dW = tW, dN, dS, dT, dB;
            if constexpr (kPW) {
                const float2 *x_m = xu + sm1 * plane, *x_0 = xu + s0 * plane, *x_p = xu + sp1 * plane;
                c = x_0[q];
                dE = dif(x_p[q], c); dW = dif(x_m[q], c);
                dN = dif(x_0[qn], c); dS = dif(x_0[qs], c);
                dT = dif(x_0[qt], c); dB = dif(x_0[qb], c);
            } else {
                dN = dif(u_0[qn], c); dS = dif(u_0[qs], c);
                dT = dif(u_0[qt], c); dB = dif(u_0[qb], c);
            }
            const float cf = val(c);
            const float ax = fddy * fddz, ay = fdx_i * fddz, az = fdx_i * fddy;
            const float fe = ax * (val(ct) + 0.5f * tE * rx1);
            const float fw = ax * (val(u_m[q]) - 0.5f * tW * rx0);
            const float fn = 0.5f * ay * (val(v_0[q]) + val(v_p[q]));
            const float fs = 0.5f * ay * (val(v_0[qs]) + val(v_p[qs]));
            const float ft = 0.5f * az * (val(w_0[q]) + val(w_p[q]));
            const float fb = 0.5f * az * (val(w_0[qb]) + val(w_p[qb]));
            const float divf = ax * (-tW + 0.5f * tE * rx1 + 0.5f * tW * rx0) +
                               0.5f * ay * (dif(v_0[q], v_0[qs]) + dif(v_p[q], v_p[qs])) +
                               0.5f * az * (dif(w_0[q], w_0[qb]) + dif(w_p[q], w_p[qb]));
            const float sig = cf * divf + 0.5f * (fe * dE - fw * dW + fn * dN - fs * dS +
                                                  ft * dT - fb * dB);
            const float vol = rdx_i * rddy_j * rddz_k;
            const float conv = -sig * vol;
            const float qd = kW ? -ax * (vs.u.e * rddx_ip * dE + vs.u.w * rddx_i * dW) -
                                      ay * (vs.u.n * rdy_j * dN + vs.u.s * rdy_jm * dS) -
                                      az * (vs.u.t * rdz_k * dT + vs.u.b * rdz_km * dB)
                                : -g * ax * (rddx_ip * dE + rddx_i * dW) -
                                      gh * ay * (rdy_j * dN + rdy_jm * dS) -
                                      gh * az * (rdz_k * dT + rdz_km * dB);
            // the LES cross term of tstle4_diff (src/flow/tstle4_mod.F90:268-458)
            float qc = 0.f;
            if (cross)
                qc = (vs.u.e * dE * rddx_ip + vs.u.w * dW * rddx_i) * ax +
                     (vs.u.n * dif(tv_p[q], tv_0[q]) - vs.u.s * dif(tv_p[qs], tv_0[qs])) * fddz +
                     (vs.u.t * dif(tw_p[q], tw_0[q]) - vs.u.b * dif(tw_p[qb], tw_0[qb])) * fddy;
            const float fak = a.rrho * vol;
            const float gp = (dif(p_p[q], p_0[q]) + a.gpx * gfl * fdx_i) * (a.rrho / fdx_i);
            uo = conv - fak * qd - gp;
            if (cross) uo += fak * qc;
        }
        // ---------------- V at (k, j+1/2, i)
        {
            // transporting V along y (mass fluxes fn, fs), transported v
            const float2 ct = v_0[q];
            const float tN = dif(v_0[qn], ct), tS = dif(v_0[qs], ct);
            float2 c = ct;
            float dE, dW, dN = tN, dS = tS, dT, dB;
            if constexpr (kPW) {
                const float2 *x_m = xv + sm1 * plane, *x_0 = xv + s0 * plane, *x_p = xv + sp1 * plane;
                c = x_0[q];
                dE = dif(x_p[q], c); dW = dif(x_m[q], c);
                dN = dif(x_0[qn], c); dS = dif(x_0[qs], c);
                dT = dif(x_0[qt], c); dB = dif(x_0[qb], c);
            } else {
                dE = dif(v_p[q], c); dW = dif(v_m[q], c);
                dT = dif(v_0[qt], c); dB = dif(v_0[qb], c);
            }
            const float cf = val(c);
            const float ax = fdy_j * fddz, ay = fddx * fddz, az = fddx * fdy_j;
            const float fe = 0.5f * ax * (val(u_0[q]) + val(u_0[qn]));
            const float fw = 0.5f * ax * (val(u_m[q]) + val(u_m[qn]));
            const float fn = ay * (val(ct) + 0.5f * tN * ry1);
            const float fs = ay * (val(v_0[qs]) - 0.5f * tS * ry0);
            const float ft = 0.5f * az * (val(w_0[q]) + val(w_0[qn]));
            const float fb = 0.5f * az * (val(w_0[qb]) + val(w_0[qb + pk]));
            const float divf = 0.5f * ax * (dif(u_0[q], u_m[q]) + dif(u_0[qn], u_m[qn])) +
                               ay * (-tS + 0.5f * tN * ry1 + 0.5f * tS * ry0) +
                               0.5f * az * (dif(w_0[q], w_0[qb]) + dif(w_0[qn], w_0[qb + pk]));
            const float sig = cf * divf + 0.5f * (fe * dE - fw * dW + fn * dN - fs * dS +
                                                  ft * dT - fb * dB);
            const float vol = rddx_i * rdy_j * rddz_k;
            const float conv = -sig * vol;
            const float qd = kW ? -ax * (vs.v.e * rdx_i * dE + vs.v.w * rdx_im * dW) -
                                      ay * (vs.v.n * rddy_jp * dN + vs.v.s * rddy_j * dS) -
                                      az * (vs.v.t * rdz_k * dT + vs.v.b * rdz_km * dB)
                                : -gh * ax * (rdx_i * dE + rdx_im * dW) -
                                      g * ay * (rddy_jp * dN + rddy_j * dS) -
                                      gh * az * (rdz_k * dT + rdz_km * dB);
            float qc = 0.f;
            if (cross)
                qc = (vs.v.e * dif(tu_0[qn], tu_0[q]) - vs.v.w * dif(tu_m[qn], tu_m[q])) * fddz +
                     (vs.v.n * dN * rddy_jp + vs.v.s * dS * rddy_j) * ay +
                     (vs.v.t * dif(tw_0[qn], tw_0[q]) - vs.v.b * dif(tw_0[qb + pk], tw_0[qb])) * fddx;
            const float fak = a.rrho * vol;
            const float gp = (dif(p_0[qn], p_0[q]) + a.gpy * gfl * fdy_j) * (a.rrho / fdy_j);
            vo = conv - fak * qd - gp;
            if (cross) vo += fak * qc;
        }
        // ---------------- W at (k+1/2, j, i)
        {
            // transporting W along z (mass fluxes ft, fb), transported w
            const float2 ct = w_0[q];
            const float tT = dif(w_0[qt], ct), tB = dif(w_0[qb], ct);
            float2 c = ct;
            float dE, dW, dN, dS, dT = tT, dB = tB;
            if constexpr (kPW) {
                const float2 *x_m = xw + sm1 * plane, *x_0 = xw + s0 * plane, *x_p = xw + sp1 * plane;
                c = x_0[q];
                dE = dif(x_p[q], c); dW = dif(x_m[q], c);
                dN = dif(x_0[qn], c); dS = dif(x_0[qs], c);
                dT = dif(x_0[qt], c); dB = dif(x_0[qb], c);
            } else {
                dE = dif(w_p[q], c); dW = dif(w_m[q], c);
                dN = dif(w_0[qn], c); dS = dif(w_0[qs], c);
            }
            const float cf = val(c);
            const float ax = fddy * fdz_k, ay = fddx * fdz_k, az = fddx * fddy;
            const float fe = 0.5f * ax * (val(u_0[q]) + val(u_0[qt]));
            const float fw = 0.5f * ax * (val(u_m[q]) + val(u_m[qt]));
            const float fn = 0.5f * ay * (val(v_0[q]) + val(v_0[qt]));
            const float fs = 0.5f * ay * (val(v_0[qs]) + val(v_0[qs + 1]));
            const float ft = az * (val(ct) + 0.5f * tT * rz1);
            const float fb = az * (val(w_0[qb]) - 0.5f * tB * rz0);
            const float divf = 0.5f * ax * (dif(u_0[q], u_m[q]) + dif(u_0[qt], u_m[qt])) +
                               0.5f * ay * (dif(v_0[q], v_0[qs]) + dif(v_0[qt], v_0[qs + 1])) +
                               az * (-tB + 0.5f * tT * rz1 + 0.5f * tB * rz0);
            const float sig = cf * divf + 0.5f * (fe * dE - fw * dW + fn * dN - fs * dS +
                                                  ft * dT - fb * dB);
            const float vol = rddx_i * rddy_j * rdz_k;
            const float conv = -sig * vol;
            const float qd = kW ? -ax * (vs.w.e * rdx_i * dE + vs.w.w * rdx_im * dW) -
                                      ay * (vs.w.n * rdy_j * dN + vs.w.s * rdy_jm * dS) -
                                      az * (vs.w.t * rddz_kp * dT + vs.w.b * rddz_k * dB)
                                : -gh * ax * (rdx_i * dE + rdx_im * dW) -
                                      gh * ay * (rdy_j * dN + rdy_jm * dS) -
                                      g * az * (rddz_kp * dT + rddz_k * dB);
            float qc = 0.f;
            if (cross)
                qc = (vs.w.e * dif(tu_0[qt], tu_0[q]) - vs.w.w * dif(tu_m[qt], tu_m[q])) * fddy +
                     (vs.w.n * dif(tv_0[qt], tv_0[q]) - vs.w.s * dif(tv_0[qs + 1], tv_0[qs])) * fddx +
                     (vs.w.t * dT * rddz_kp + vs.w.b * dB * rddz_k) * az;
            const float fak = a.rrho * vol;
            const float gp = (dif(p_0[qt], p_0[q]) + a.gpz * gfl * fdz_k) * (a.rrho / fdz_k);
            wo = conv - fak * qd - gp;
            if (cross) wo += fak * qc;
        }
}

// ---- grids with faces that have no neighbour --------------------------------
// harmonic face mean of tstle4_diff: g*g'/MAX(g+g', gmol), in FP32 like
// the rest of the fluxes
__device__ __forceinline__ float fhm(float x, float y, float gmol) {
    const float s = x + y;
    return x * y / (s < gmol ? gmol : s);
}

__device__ __forceinline__ Visc3 visc_uniform(const FluxArgs& a) {
    const float g = a.g, h = a.gh;
    return Visc3{{g, g, h, h, h, h}, {h, h, g, g, h, h}, {h, h, h, h, g, g}};
}

// The face viscosities of tstle4_diff (src/flow/tstle4_mod.F90:268-458) at
// the point (k, j, i) of one grid, from its viscosity field gg: next to a face
// without a neighbour the ghost values of G enter the means (zero on the
// walls of the coarsest level, so no viscous flux crosses them).
__device__ Visc3 visc_field(const double* gg, int kk, int jj, int k, int j, int i, float gm) {
    auto G = [&](int kq, int jq, int iq) -> float {
        return (float)gg[(long long)(iq - 1) * kk * jj + (long long)(jq - 1) * kk + (kq - 1)];
    };
    Visc3 v;
    v.u.e = G(k, j, i + 1);
    v.u.w = G(k, j, i);
    v.u.n = fhm(G(k, j, i), G(k, j + 1, i), gm) + fhm(G(k, j, i + 1), G(k, j + 1, i + 1), gm);
    v.u.s = fhm(G(k, j - 1, i), G(k, j, i), gm) + fhm(G(k, j - 1, i + 1), G(k, j, i + 1), gm);
    v.u.t = fhm(G(k, j, i), G(k + 1, j, i), gm) + fhm(G(k, j, i + 1), G(k + 1, j, i + 1), gm);
    v.u.b = fhm(G(k - 1, j, i), G(k, j, i), gm) + fhm(G(k - 1, j, i + 1), G(k, j, i + 1), gm);
    v.v.e = fhm(G(k, j, i), G(k, j, i + 1), gm) + fhm(G(k, j + 1, i), G(k, j + 1, i + 1), gm);
    v.v.w = fhm(G(k, j, i - 1), G(k, j, i), gm) + fhm(G(k, j + 1, i - 1), G(k, j + 1, i), gm);
    v.v.n = G(k, j + 1, i);
    v.v.s = G(k, j, i);
    v.v.t = fhm(G(k, j, i), G(k + 1, j, i), gm) + fhm(G(k, j + 1, i), G(k + 1, j + 1, i), gm);
    v.v.b = fhm(G(k - 1, j, i), G(k, j, i), gm) + fhm(G(k - 1, j + 1, i), G(k, j + 1, i), gm);
    v.w.e = fhm(G(k, j, i), G(k, j, i + 1), gm) + fhm(G(k + 1, j, i), G(k + 1, j, i + 1), gm);
    v.w.w = fhm(G(k, j, i - 1), G(k, j, i), gm) + fhm(G(k + 1, j, i - 1), G(k + 1, j, i), gm);
    v.w.n = fhm(G(k, j, i), G(k, j + 1, i), gm) + fhm(G(k + 1, j, i), G(k + 1, j + 1, i), gm);
    v.w.s = fhm(G(k, j - 1, i), G(k, j, i), gm) + fhm(G(k + 1, j - 1, i), G(k + 1, j, i), gm);
    v.w.t = G(k + 1, j, i);
    v.w.b = G(k, j, i);
    return v;
}

// Does the grid have a face without a neighbour (anything but CON)?
__device__ __forceinline__ bool has_open_face(const DevGrid& G) {
    bool w = false;
    for (int f = 0; f < 6; ++f) w |= G.bc[f] != MGLET_BC_CON;
    return w;
}
__device__ __forceinline__ bool has_par_face(const DevGrid& G) {
    bool w = false;
    for (int f = 0; f < 6; ++f) w |= G.bc[f] == MGLET_BC_PAR;
    return w;
}

// The face viscosities of the point on a grid whose G is not one value (wv):
// from G at every point when G is a field (LES, or a G the caller set), else
// on the outermost interior layer only (a wall's zero ghosts); the uniform
// ones otherwise.
__device__ __forceinline__ Visc3 visc_at(const FluxArgs& a, const DevGrid& G, bool wv, int k, int j,
                                         int i) {
    const bool shell = i == 3 || i == G.ii - 2 || j == 3 || j == G.jj - 2 || k == 3 || k == G.kk - 2;
    if (wv && (a.gall || shell)) return visc_field(a.G + G.ip3, G.kk, G.jj, k, j, i, (float)a.wgmol);
    return visc_uniform(a);
}

// tauwin (src/flow/wernerwengle_mod.F90:64-87) / dds as swcle3d applies it
// (src/flow/tstle4_mod.F90:1832-1844); ddsb = dds**(-1/7); FP64.
__device__ double wall_shear(const FluxArgs& a, double dds, double ddsb, double u) {
    const double vz = copysign(1.0, u);
    const double uq = fabs(u);
    double tau;
    if (uq >= a.cpo6 / dds)
        tau = vz * a.wrho * pow(ddsb * (a.cpo4 * uq + a.cpo5 / dds), a.cpo8);
    else
        tau = vz * 2.0 * a.wgmol * uq / dds;
    return tau / a.wrho / dds;
}

// What tstle4 does differently next to faces without a neighbour, for the
// point (k, j, i) with own values u, v, w (src/flow/tstle4_mod.F90:13-120):
// the velocity normal to a wall, inflow or CO1 face on its last interior
// position is not a flux point (only CON and OP1 faces extend the ranges),
// and on NOS faces swcle3d (tstle4_mod.F90:1756-1829) subtracts the
// Werner-Wengle wall shear from the tangential components next to the wall.
__device__ void boundary_terms(const FluxArgs& a, const DevGrid& G, int k, int j, int i, double u,
                               double v, double w, float& uo, float& vo, float& wo) {
    const int* bc = G.bc;
    auto ext = [](int t) { return t == MGLET_BC_CON || t == MGLET_BC_OP1; };
    if (i == G.ii - 2 && !ext(bc[1])) uo = 0.f;
    if (j == G.jj - 2 && !ext(bc[3])) vo = 0.f;
    if (k == G.kk - 2 && !ext(bc[5])) wo = 0.f;
    const double *ddx = a.ddx + G.ipx - 1, *ddy = a.ddy + G.ipy - 1, *ddz = a.ddz + G.ipz - 1;
    const double *wwx = a.wwx + G.ipx - 1, *wwy = a.wwy + G.ipy - 1, *wwz = a.wwz + G.ipz - 1;
    const bool xl = bc[0] == MGLET_BC_NOS && i == 3, xh = bc[1] == MGLET_BC_NOS && i == G.ii - 2;
    const bool yl = bc[2] == MGLET_BC_NOS && j == 3, yh = bc[3] == MGLET_BC_NOS && j == G.jj - 2;
    const bool zl = bc[4] == MGLET_BC_NOS && k == 3, zh = bc[5] == MGLET_BC_NOS && k == G.kk - 2;
    if (!(xl || xh || yl || yh || zl || zh)) return;
    double su = 0.0, sv = 0.0, sw = 0.0;
    if (xl || xh) {
        sv += wall_shear(a, ddx[i], wwx[i], v);
        sw += wall_shear(a, ddx[i], wwx[i], w);
    }
    if (yl || yh) {
        su += wall_shear(a, ddy[j], wwy[j], u);
        sw += wall_shear(a, ddy[j], wwy[j], w);
    }
    if (zl || zh) {
        su += wall_shear(a, ddz[k], wwz[k], u);
        sv += wall_shear(a, ddz[k], wwz[k], v);
    }
    uo -= (float)su;
    vo -= (float)sv;
    wo -= (float)sw;
}

// One CTA per j-slab of a grid, one thread per interior (k, j) of the slab,
// marching i.
template <bool kW>
__global__ void __launch_bounds__(576, 2) k_mx_flux(FluxArgs a) {
    extern __shared__ float2 sm[];
    const DevGrid G = a.grids[blockIdx.x / a.nslab];
    const int slab = blockIdx.x % a.nslab;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int js = (jj - 4 + a.nslab - 1) / a.nslab;
    const int j0 = 3 + slab * js;                     // first interior j of the slab
    const int nj = min(js, jj - 1 - j0);              // interior j of the slab: j0 .. j0+nj-1
    // plane window: k = 2..kk-1, j = j0-1..j0+nj
    const int pk = kk - 2, pj = nj + 2, plane = pk * pj;
    float2* su = sm;                  // [3][plane]
    float2* sv = su + 3 * plane;
    float2* sw = sv + 3 * plane;
    float2* sp = sw + 3 * plane;      // [2][plane]
    // point-value windows (ghost-cell IB), [3][plane] each, when the launch has them
    float2* xu = sp + 2 * plane;
    float2* xv = xu + 3 * plane;
    float2* xw = xv + 3 * plane;
    const bool pwg = kW && a.pw && a.pwflag && a.pwflag[blockIdx.x / a.nslab];
    const long long o = G.ip3;
    const int kj = kk * jj;
    const int nk = kk - 4;
    const int t = threadIdx.x;
    const bool on = t < nk * nj;
    const int k = on ? t % nk + 3 : 3, j = on ? t / nk + j0 : j0;
    const int nring = plane - nk * nj;
    // window-local index of (k, j): (k-2) + (j-j0+1)*pk
    auto pl = [pk, j0](int kq, int jq) { return (kq - 2) + (jq - j0 + 1) * pk; };
    // ring point r (0..nring-1) -> (k, j) on the border of the window
    auto ring = [&](int r, int& kq, int& jq) {
        if (r < pk) { kq = 2 + r; jq = j0 - 1; return; }
        r -= pk;
        if (r < pk) { kq = 2 + r; jq = j0 + nj; return; }
        r -= pk;
        jq = j0 + r / 2;
        kq = (r & 1) ? kk - 1 : 2;
    };
    const double *U0 = a.U0 + o, *V0 = a.V0 + o, *W0 = a.W0 + o, *P0 = a.P0 + o;
    // 1-based views of the FP32 spacing tables of this grid
    const float* X = a.sx + G.ipx - 1;
    const float* Y = a.sy + G.ipy - 1;
    const float* Z = a.sz + G.ipz - 1;
    const long long nx = a.nx, ny = a.ny, nz = a.nz;
    // j- and k-dependent factors are fixed per thread
    const Col cl = column(Y, ny, j, Z, nz, k);

    // own raw FP64 values of planes i (cur) and i+1, i+2 (pipeline)
    double ucur = 0, vcur = 0, wcur = 0, unx = 0, vnx = 0, wnx = 0;

    auto load_plane = [&](int i, int slot3, int slot2, bool with_p, double& uo_, double& vo_,
                          double& wo_) {
        // interior point of this thread
        if (on) {
            const long long c = (long long)(i - 1) * kj + (long long)(j - 1) * kk + (k - 1);
            const double u = U0[c], v = V0[c], w = W0[c];
            uo_ = u; vo_ = v; wo_ = w;
            const int q = pl(k, j);
            su[slot3 * plane + q] = split64(u);
            sv[slot3 * plane + q] = split64(v);
            sw[slot3 * plane + q] = split64(w);
            if (with_p) sp[slot2 * plane + q] = split64(P0[c]);
            if (pwg) {
                xu[slot3 * plane + q] = split64(a.PU0[o + c]);
                xv[slot3 * plane + q] = split64(a.PV0[o + c]);
                xw[slot3 * plane + q] = split64(a.PW0[o + c]);
            }
        }
        for (int r = t; r < nring; r += blockDim.x) {
            int kq, jq;
            ring(r, kq, jq);
            const long long c = (long long)(i - 1) * kj + (long long)(jq - 1) * kk + (kq - 1);
            const int q = pl(kq, jq);
            su[slot3 * plane + q] = split64(U0[c]);
            sv[slot3 * plane + q] = split64(V0[c]);
            sw[slot3 * plane + q] = split64(W0[c]);
            if (with_p) sp[slot2 * plane + q] = split64(P0[c]);
            if (pwg) {
                xu[slot3 * plane + q] = split64(a.PU0[o + c]);
                xv[slot3 * plane + q] = split64(a.PV0[o + c]);
                xw[slot3 * plane + q] = split64(a.PW0[o + c]);
            }
        }
    };

    double dummy0, dummy1, dummy2;
    load_plane(2, 2 % 3, 0, false, dummy0, dummy1, dummy2);
    load_plane(3, 3 % 3, 3 % 2, true, ucur, vcur, wcur);
    load_plane(4, 4 % 3, 4 % 2, true, unx, vnx, wnx);
    __syncthreads();

    const int q = pl(k, j);
    const float gfl = (float)G.gradpflag;
    const bool wg = kW && has_open_face(G);
    const bool pgrid = kW && has_par_face(G);
    const bool wv = (wg || (kW && a.gall)) && !(a.guni && a.guni[2 * (blockIdx.x / a.nslab)] != 0.0);
    for (int i = 3; i <= ii - 2; ++i) {
        float uo = 0.f, vo = 0.f, wo = 0.f;
        if (on) {
            if constexpr (kW) {
                const Visc3 vs = visc_at(a, G, wv, k, j, i);
                if (pwg)
                    flux_point<true, true>(a, X, nx, cl, su, sv, sw, sp, plane, pk, q, i, gfl, vs, uo, vo,
                                           wo, xu, xv, xw);
                else
                    flux_point<true>(a, X, nx, cl, su, sv, sw, sp, plane, pk, q, i, gfl, vs, uo, vo, wo);
                if (wg) boundary_terms(a, G, k, j, i, ucur, vcur, wcur, uo, vo, wo);
            } else {
                const Visc3 vs{};
                flux_point<false>(a, X, nx, cl, su, sv, sw, sp, plane, pk, q, i, gfl, vs, uo, vo, wo);
            }
        }
        // issue the global loads of plane i+2 before the RK update and the barrier
        double unx2 = 0, vnx2 = 0, wnx2 = 0;
        __syncthreads();   // every thread is done with slot (i-1)%3 and p slot i%2
        if (i + 2 <= ii - 1) load_plane(i + 2, (i + 2) % 3, (i + 2) % 2, true, unx2, vnx2, wnx2);
        if (on) {
            const long long c = o + (long long)(i - 1) * kj + (long long)(j - 1) * kk + (k - 1);
            if (kW && pgrid) {
                a.UO[c] = (double)uo; a.VO[c] = (double)vo; a.WO[c] = (double)wo;
            } else {
                const float frhs = (float)a.sprm[0];
                const float du = frhs * a.DU[c] + uo;
                const float dv = frhs * a.DV[c] + vo;
                const float dw = frhs * a.DW[c] + wo;
                a.DU[c] = du; a.DV[c] = dv; a.DW[c] = dw;
                const float fdt = (float)a.sprm[1];
                a.U[c] = ucur + (double)(fdt * du);
                a.V[c] = vcur + (double)(fdt * dv);
                a.W[c] = wcur + (double)(fdt * dw);
            }
        }
        ucur = unx; vcur = vnx; wcur = wnx;
        unx = unx2; vnx = vnx2; wnx = wnx2;
        __syncthreads();
    }
}

// ---- the same kernel with the planes staged by TMA -------------------------
// A wait for a bulk copy gives up after this many SM clock cycles (about one
// second); a healthy wait lasts microseconds.
constexpr long long kFluxWait = 2000000000LL;

__device__ __forceinline__ unsigned fsm_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void fbar_init(unsigned long long* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fsm_u32(b)));
}

__device__ __forceinline__ void fbar_expect(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fsm_u32(b)), "r"(bytes)
                 : "memory");
}

// bounded wait for the phase of the given parity; false on timeout
__device__ __forceinline__ bool fbar_wait(unsigned long long* b, unsigned parity) {
    const long long t0 = clock64();
    while (true) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(fsm_u32(b)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kFluxWait) return false;
    }
}

// one (kk x jj) plane of a field, tensor coordinates (0, 0, z)
__device__ __forceinline__ void tma_plane(double* dst, const CUtensorMap* m, int z,
                                          unsigned long long* b) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(fsm_u32(dst)),
        "l"((unsigned long long)m), "r"(0), "r"(0), "r"(z), "r"(fsm_u32(b))
        : "memory");
}

// One CTA per grid (grids whose k x j interior fits one CTA), marching i.
// Thread 0 issues TMA tensor copies of whole planes of U, V, W and P (each
// a contiguous kk x jj slab of the grid) into two staging slots, two planes
// ahead, completing on one mbarrier per slot; after a plane arrives every
// thread splits its points of it (its own column and the window border)
// into the (hi, lo) windows, as the plain-load kernel does from global
// memory.  Same windows, same arithmetic (flux_point), same bits.
template <bool kW>
__global__ void __launch_bounds__(576, 2)
    k_mx_flux_tma(FluxArgs a, const __grid_constant__ CUtensorMap mu,
                  const __grid_constant__ CUtensorMap mv, const __grid_constant__ CUtensorMap mw,
                  const __grid_constant__ CUtensorMap mp) {
    extern __shared__ __align__(128) unsigned char fraw[];
    unsigned char* fsm = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<unsigned long long>(fraw) + 127) & ~127ULL);
    const int gid = blockIdx.x;
    const DevGrid G = a.grids[gid];
    const int kk = G.kk, jj = G.jj, ii = G.ii, kj = kk * jj;
    const int nk = kk - 4, nj = jj - 4, j0 = 3;
    const int pk = kk - 2, pj = nj + 2, plane = pk * pj;
    double* stage = reinterpret_cast<double*>(fsm);                 // [2][4][kj]
    float2* su = reinterpret_cast<float2*>(fsm + (size_t)8 * kj * 8);
    float2* sv = su + 3 * plane;
    float2* sw = sv + 3 * plane;
    float2* sp = sw + 3 * plane;
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(sp + 2 * plane);
    const int t = threadIdx.x;
    const bool on = t < nk * nj;
    const int k = on ? t % nk + 3 : 3, j = on ? t / nk + j0 : j0;
    const int nring = plane - nk * nj;
    auto pl = [pk, j0](int kq, int jq) { return (kq - 2) + (jq - j0 + 1) * pk; };
    auto ring = [&](int r, int& kq, int& jq) {
        if (r < pk) { kq = 2 + r; jq = j0 - 1; return; }
        r -= pk;
        if (r < pk) { kq = 2 + r; jq = j0 + nj; return; }
        r -= pk;
        jq = j0 + r / 2;
        kq = (r & 1) ? kk - 1 : 2;
    };
    const long long o = G.ip3;
    const float* X = a.sx + G.ipx - 1;
    const float* Y = a.sy + G.ipy - 1;
    const float* Z = a.sz + G.ipz - 1;
    const long long nx = a.nx, ny = a.ny, nz = a.nz;
    const Col cl = column(Y, ny, j, Z, nz, k);
    const int zbase = gid * ii;        // plane i of this grid is tensor z = zbase + i - 1
    const unsigned bytes = (unsigned)(4 * kj * 8);
    int last[2] = {0, 0};               // thread 0: plane last issued per slot
    if (t == 0) {
        fbar_init(&bar[0]);
        fbar_init(&bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int pln) {
        const int s = pln & 1;
        if (pln == a.skip_plane) {   // test switch: the wait for this plane runs out
            last[s] = 0;
            return;
        }
        double* d = stage + (size_t)s * 4 * kj;
        fbar_expect(&bar[s], bytes);
        tma_plane(d, &mu, zbase + pln - 1, &bar[s]);
        tma_plane(d + kj, &mv, zbase + pln - 1, &bar[s]);
        tma_plane(d + 2 * kj, &mw, zbase + pln - 1, &bar[s]);
        tma_plane(d + 3 * kj, &mp, zbase + pln - 1, &bar[s]);
        last[s] = pln;
    };
    // every thread waits for plane pln (slot pln & 1, its (pln-2)/2-th use)
    auto arrived = [&](int pln) -> bool {
        const bool ok = fbar_wait(&bar[pln & 1], (unsigned)(((pln - 2) >> 1) & 1));
        return __syncthreads_and(ok) != 0;
    };
    auto fail = [&]() {
        if (t == 0) {
            atomicExch(a.err, 1);
            // let the copies still in flight land before the CTA leaves
            for (int s = 0; s < 2; ++s)
                if (last[s]) fbar_wait(&bar[s], (unsigned)(((last[s] - 2) >> 1) & 1));
        }
    };
    auto convert = [&](int pln, int slot3, int slot2, double& uo_, double& vo_, double& wo_) {
        const double* Su = stage + (size_t)(pln & 1) * 4 * kj;
        const double *Sv = Su + kj, *Sw = Sv + kj, *Sp = Sw + kj;
        if (on) {
            const int c = (j - 1) * kk + (k - 1);
            const double u = Su[c], v = Sv[c], w = Sw[c];
            uo_ = u; vo_ = v; wo_ = w;
            const int q = pl(k, j);
            su[slot3 * plane + q] = split64(u);
            sv[slot3 * plane + q] = split64(v);
            sw[slot3 * plane + q] = split64(w);
            if (slot2 >= 0) sp[slot2 * plane + q] = split64(Sp[c]);
        }
        for (int r = t; r < nring; r += blockDim.x) {
            int kq, jq;
            ring(r, kq, jq);
            const int c = (jq - 1) * kk + (kq - 1);
            const int q = pl(kq, jq);
            su[slot3 * plane + q] = split64(Su[c]);
            sv[slot3 * plane + q] = split64(Sv[c]);
            sw[slot3 * plane + q] = split64(Sw[c]);
            if (slot2 >= 0) sp[slot2 * plane + q] = split64(Sp[c]);
        }
    };
    double ucur = 0, vcur = 0, wcur = 0, unx = 0, vnx = 0, wnx = 0, d0, d1, d2;
    if (t == 0) {
        issue(2);
        issue(3);
    }
    if (!arrived(2)) { fail(); return; }
    convert(2, 2 % 3, -1, d0, d1, d2);
    __syncthreads();
    if (t == 0) issue(4);
    if (!arrived(3)) { fail(); return; }
    convert(3, 3 % 3, 3 % 2, ucur, vcur, wcur);
    __syncthreads();
    if (t == 0 && 5 <= ii - 1) issue(5);
    if (!arrived(4)) { fail(); return; }
    convert(4, 4 % 3, 4 % 2, unx, vnx, wnx);
    __syncthreads();
    if (t == 0 && 6 <= ii - 1) issue(6);

    const int q = pl(k, j);
    const float gfl = (float)G.gradpflag;
    const bool wg = kW && has_open_face(G);
    const bool pgrid = kW && has_par_face(G);
    const bool wv = (wg || (kW && a.gall)) && !(a.guni && a.guni[2 * gid] != 0.0);
    for (int i = 3; i <= ii - 2; ++i) {
        float uo = 0.f, vo = 0.f, wo = 0.f;
        if (on) {
            if constexpr (kW) {
                const Visc3 vs = visc_at(a, G, wv, k, j, i);
                flux_point<true>(a, X, nx, cl, su, sv, sw, sp, plane, pk, q, i, gfl, vs, uo, vo, wo);
                if (wg) boundary_terms(a, G, k, j, i, ucur, vcur, wcur, uo, vo, wo);
            } else {
                const Visc3 vs{};
                flux_point<false>(a, X, nx, cl, su, sv, sw, sp, plane, pk, q, i, gfl, vs, uo, vo, wo);
            }
        }
        double unx2 = 0, vnx2 = 0, wnx2 = 0;
        __syncthreads();   // every thread is done with slot (i-1)%3 and p slot i%2
        if (i + 2 <= ii - 1) {
            if (!arrived(i + 2)) { fail(); return; }
            convert(i + 2, (i + 2) % 3, (i + 2) % 2, unx2, vnx2, wnx2);
        }
        if (on) {
            const long long c = o + (long long)(i - 1) * kj + (long long)(j - 1) * kk + (k - 1);
            if (kW && pgrid) {
                a.UO[c] = (double)uo; a.VO[c] = (double)vo; a.WO[c] = (double)wo;
            } else {
                const float frhs = (float)a.sprm[0];
                const float du = frhs * a.DU[c] + uo;
                const float dv = frhs * a.DV[c] + vo;
                const float dw = frhs * a.DW[c] + wo;
                a.DU[c] = du; a.DV[c] = dv; a.DW[c] = dw;
                const float fdt = (float)a.sprm[1];
                a.U[c] = ucur + (double)(fdt * du);
                a.V[c] = vcur + (double)(fdt * dv);
                a.W[c] = wcur + (double)(fdt * dw);
            }
        }
        ucur = unx; vcur = vnx; wcur = wnx;
        unx = unx2; vnx = vnx2; wnx = wnx2;
        __syncthreads();   // staging slot (i+2)&1 consumed
        if (t == 0 && i + 4 <= ii - 1) issue(i + 4);
    }
}

}  // namespace

// j-slabs per grid: the fewest for which a slab has at most 576 (k, j) columns
static int flux_slabs(const DevGrid& G0) {
    const int nk = G0.kk - 4, nj = G0.jj - 4;
    for (int s = 1; s <= nj; ++s)
        if (nk * ((nj + s - 1) / s) <= 576) return s;
    return 0;
}

// 11 planes of (hi, lo) windows (U, V, W: 3 each; P: 2), 20 with the point
// values' windows of the ghost-cell IB
static size_t flux_smem(const DevGrid& G0, bool pw = false) {
    const int nslab = flux_slabs(G0);
    const int js = (G0.jj - 4 + nslab - 1) / nslab;
    return (size_t)(pw ? 20 : 11) * (G0.kk - 2) * (js + 2) * sizeof(float2);
}

// Per context: the tensor maps of U, V, W, P for the TMA variant and the
// variant in use (0 plane loads, 1 TMA staging, -1 untuned default).
struct FluxState {
    CUtensorMap map[4];
    bool tma = false;
    bool walls = false;     // some grid has a face that is not CON: the boundary path
    bool gfield = false;    // G is a field: the boundary instantiation, G at every point
    // ghost-cell IB: per-grid flags of the grids whose transported velocities
    // are the point values (the plane-load kernel then carries their windows)
    const unsigned char* d_pw = nullptr;
    int variant = -1;
    double ms[2] = {0.0, 0.0};
};
static std::map<const Ctx*, FluxState> g_flux;

static size_t flux_tma_smem(const DevGrid& G0) {
    const size_t kj = (size_t)G0.kk * G0.jj, plane = (size_t)(G0.kk - 2) * (G0.jj - 2);
    return 128 + 8 * kj * sizeof(double) + 11 * plane * sizeof(float2) + 16;
}

// 3-D tensor map over one field: (k, j, i + ii * grid), boxes of one plane
static int encode_plane_map(Ctx* c, const double* base, CUtensorMap* m) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            set_error("mixed form: cuTensorMapEncodeTiled is not available");
            return MGLET_ERR_CUDA;
        }
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const DevGrid& G0 = c->grids[0];
    const cuuint64_t dims[3] = {(cuuint64_t)G0.kk, (cuuint64_t)G0.jj,
                                (cuuint64_t)G0.ii * (cuuint64_t)c->ngrid};
    const cuuint64_t strides[2] = {(cuuint64_t)G0.kk * sizeof(double),
                                   (cuuint64_t)G0.kk * G0.jj * sizeof(double)};
    const cuuint32_t box[3] = {(cuuint32_t)G0.kk, (cuuint32_t)G0.jj, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(base), dims,
                              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("mixed form: cuTensorMapEncodeTiled failed");
        return MGLET_ERR_CUDA;
    }
    return 0;
}

// Checks the launch limits of the flux kernel for this grid shape and opts
// in to the dynamic shared memory it needs; where a grid's k x j interior
// fits one CTA and its planes meet the TMA rules (16-byte rows, boxes of at
// most 256 points per side), also builds the TMA variant's tensor maps.
int mx_flux_prepare(Ctx* c) {
    const DevGrid& G0 = c->grids[0];
    if (G0.kk - 4 > 576) {
        set_error("mixed form: the flux kernel takes at most 576 cells in k per grid");
        return MGLET_ERR_UNSUPPORTED;
    }
    const size_t smem = flux_smem(G0);
    if (smem > 200 * 1024) {
        set_error("mixed form: grid planes too large for the flux kernel's shared memory");
        return MGLET_ERR_UNSUPPORTED;
    }
    MG_CUDA(cudaFuncSetAttribute(k_mx_flux<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MG_CUDA(cudaFuncSetAttribute(k_mx_flux<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    FluxState& fs = g_flux[c];
    fs = FluxState();
    for (const DevGrid& g : c->grids)
        for (int f = 0; f < 6; ++f) fs.walls |= g.bc[f] != MGLET_BC_CON;
    const size_t tsm = flux_tma_smem(G0);
    if (flux_slabs(G0) == 1 && (G0.kk * sizeof(double)) % 16 == 0 && G0.kk <= 256 &&
        G0.jj <= 256 && tsm <= 113 * 1024) {
        const char* names[4] = {"U", "V", "W", "P"};
        for (int f = 0; f < 4; ++f)
            if (int rc = encode_plane_map(c, c->F(names[f]), &fs.map[f])) return rc;
        MG_CUDA(cudaFuncSetAttribute(k_mx_flux_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tsm));
        MG_CUDA(cudaFuncSetAttribute(k_mx_flux_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tsm));
        fs.tma = true;
    }
    return 0;
}

void mx_flux_release(Ctx* c) { g_flux.erase(c); }

void mx_flux_set_gfield(Ctx* c) { g_flux[c].gfield = true; }

static int launch_variant(Ctx* c, int v, const FluxArgs& a, int threads) {
    const DevGrid& G0 = c->grids[0];
    FluxState& fs = g_flux[c];
    const size_t tsm = flux_tma_smem(G0), psm = flux_smem(G0, fs.d_pw != nullptr);
    const unsigned nb = (unsigned)(c->ngrid * a.nslab);
    const bool kw = fs.walls || fs.gfield;
    if (v == 1 && fs.tma && !fs.d_pw) {
        if (kw)
            k_mx_flux_tma<true><<<c->ngrid, threads, tsm, c->stream>>>(a, fs.map[0], fs.map[1],
                                                                      fs.map[2], fs.map[3]);
        else
            k_mx_flux_tma<false><<<c->ngrid, threads, tsm, c->stream>>>(a, fs.map[0], fs.map[1],
                                                                       fs.map[2], fs.map[3]);
    } else if (kw) {
        k_mx_flux<true><<<nb, threads, psm, c->stream>>>(a);
    } else {
        k_mx_flux<false><<<nb, threads, psm, c->stream>>>(a);
    }
    MG_LAUNCHED(c);
    return 0;
}

static FluxArgs flux_args(Ctx* c, float* du, float* dv, float* dw, const float* sx, const float* sy,
                          const float* sz, const double* sprm, int* err, int* threads) {
    const DevGrid& G0 = c->grids[0];
    const int nslab = flux_slabs(G0);
    const int js = (G0.jj - 4 + nslab - 1) / nslab;
    *threads = ((G0.kk - 4) * js + 31) / 32 * 32;
    FluxArgs a{};
    a.nslab = nslab;
    a.grids = c->d_grids;
    a.U0 = c->F("U"); a.V0 = c->F("V"); a.W0 = c->F("W"); a.P0 = c->F("P");
    a.U = c->F("U"); a.V = c->F("V"); a.W = c->F("W");
    a.DU = du; a.DV = dv; a.DW = dw;
    a.sx = sx; a.sy = sy; a.sz = sz;
    a.nx = c->idimx; a.ny = c->idimy; a.nz = c->idimz;
    const double gm = c->prm.gmol;
    const double h0 = gm * gm / std::max(gm + gm, gm);
    a.g = (float)gm;
    a.gh = (float)(h0 + h0);
    a.rrho = (float)(1.0 / c->prm.rho);
    a.gpx = (float)c->prm.gradp[0]; a.gpy = (float)c->prm.gradp[1]; a.gpz = (float)c->prm.gradp[2];
    a.sprm = sprm;
    a.err = err;
    a.skip_plane = 0;
    // boundary path: G, FP64 widths and the Werner-Wengle constants
    // (wernerwengle_mod.F90:13-28 init_wernerwengle)
    a.G = c->F("G");
    a.UO = c->F("UO"); a.VO = c->F("VO"); a.WO = c->F("WO");
    a.pwflag = g_flux[c].d_pw;
    a.pw = a.pwflag ? 1 : 0;
    a.PU0 = c->f3.count("PWU") ? c->F("PWU") : nullptr;
    a.PV0 = c->f3.count("PWV") ? c->F("PWV") : nullptr;
    a.PW0 = c->f3.count("PWW") ? c->F("PWW") : nullptr;
    a.guni = c->d_guni;
    a.gall = g_flux[c].gfield ? 1 : 0;
    a.iles = c->ilesmodel != 0 ? 1 : 0;
    a.ddx = c->L("DDX"); a.ddy = c->L("DDY"); a.ddz = c->L("DDZ");
    a.wwx = c->L("WWX"); a.wwy = c->L("WWY"); a.wwz = c->L("WWZ");
    const double rho = c->prm.rho, cwa = 8.3, cwb = 1.0 / 7.0;
    const double cpo1 = 1.0 - cwb, cpo2 = 1.0 + cwb;
    a.wrho = rho;
    a.wgmol = gm;
    a.cpo4 = cpo2 / cwa * std::pow(gm / rho, cwb);
    a.cpo5 = 0.5 * cpo1 * std::pow(cwa, cpo2 / cpo1) * std::pow(gm / rho, cpo2);
    a.cpo6 = 0.5 * gm / rho * std::pow(cwa, 2.0 / cpo1);
    a.cpo8 = 2.0 / cpo2;
    return a;
}

// Times both variants on the current fields and keeps the faster; the
// fields are still zero when the context is created, so the timing
// launches leave them unchanged (zero fluxes, zero increments).
int mx_flux_tune(Ctx* c, float* du, float* dv, float* dw, const float* sx, const float* sy,
                 const float* sz, const double* sprm, int* err) {
    FluxState& fs = g_flux[c];
    if (!fs.tma) return 0;
    int threads;
    const FluxArgs a = flux_args(c, du, dv, dw, sx, sy, sz, sprm, err, &threads);
    cudaEvent_t e0, e1;
    MG_CUDA(cudaEventCreate(&e0));
    MG_CUDA(cudaEventCreate(&e1));
    for (int v = 0; v < 2; ++v) {
        if (int rc = launch_variant(c, v, a, threads)) return rc;
        cudaEventRecord(e0, c->stream);
        for (int r = 0; r < 3; ++r)
            if (int rc = launch_variant(c, v, a, threads)) return rc;
        cudaEventRecord(e1, c->stream);
        MG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        fs.ms[v] = ms / 3.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    fs.variant = fs.ms[1] < fs.ms[0] ? 1 : 0;
    return 0;
}

int mx_flux_force(Ctx* c, int v) {
    FluxState& fs = g_flux[c];
    if (v < -1 || v > 1) {
        set_error("force_variant: mx_flux variants are 0 (plane loads) and 1 (TMA staging)");
        return MGLET_ERR_ARG;
    }
    if (v == 1 && !fs.tma) {
        set_error("force_variant: the TMA flux variant needs grids that fit one CTA");
        return MGLET_ERR_UNSUPPORTED;
    }
    fs.variant = v;
    return 0;
}

std::string mx_flux_tuning(Ctx* c) {
    const FluxState& fs = g_flux[c];
    char b[160];
    const int v = fs.variant < 0 ? 0 : fs.variant;
    std::snprintf(b, sizeof b, "mx_flux: %s%s (plane loads %.4f ms, TMA %.4f ms)",
                  v == 1 ? "TMA tensor staging" : "plane loads", fs.variant < 0 ? " [default]" : "",
                  fs.ms[0], fs.ms[1]);
    return b;
}

int launch_mx_flux(Ctx* c, float* du, float* dv, float* dw, const float* sx, const float* sy,
                   const float* sz, const double* sprm, int* err, bool skip) {
    ProfScope ps_(c, "mx_flux");
    int threads;
    FluxArgs a = flux_args(c, du, dv, dw, sx, sy, sz, sprm, err, &threads);
    const FluxState& fs = g_flux[c];
    // the boundary instantiation reads G only on grids where it is not one value
    if (fs.walls || fs.gfield)
        if (int rc = launch_g_uniform(c)) return rc;
    if (skip && fs.tma) {
        a.skip_plane = 4;
        return launch_variant(c, 1, a, threads);
    }
    return launch_variant(c, fs.variant == 1 ? 1 : 0, a, threads);
}

bool mx_flux_has_tma(Ctx* c) { return g_flux[c].tma; }

// Ghost-cell IB: device flags (per grid, 1 = the transported velocities are
// the point values PWU, PWV, PWW); the boundary instantiation of the
// plane-load kernel, which carries the point values' windows, is used from
// then on.
int mx_flux_set_pw(Ctx* c, const unsigned char* d_pw) {
    FluxState& fs = g_flux[c];
    fs.d_pw = d_pw;
    if (!d_pw) return 0;
    fs.walls = true;
    const size_t smem = flux_smem(c->grids[0], true);
    if (smem > 227 * 1024) {
        set_error("mixed form: grid planes too large for the ghost-cell flux windows");
        return MGLET_ERR_UNSUPPORTED;
    }
    MG_CUDA(cudaFuncSetAttribute(k_mx_flux<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return 0;
}

}  // namespace mg
