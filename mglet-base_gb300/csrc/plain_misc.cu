// plain_misc.cu -- halo box copies and itinfo diagnostics.
//
//   connect_self_single  src/core/connect/connect2_mod.F90:947-995
//   compcflmax           src/flow/timeintegration_mod.F90:306-370
//   compdivmax           src/flow/timeintegration_mod.F90:376-414
//   enerfg               src/flow/timeintegration_mod.F90:417-452
//
// With one rank every connection of the reference is a self connection:
// a 3-D box copy from the sending grid's interior into the receiving
// grid's ghost layers.  The host turns the connection table into a task
// list once per (level, layers, corners, normal, forward, field set); the
// copy kernel takes one task per CTA.
#include <algorithm>

#include "internal.h"

namespace mg {
namespace {

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

struct FieldSlots {
    double* f[6];
};

__global__ void k_connect(const BoxCopy* __restrict__ tasks, FieldSlots fs) {
    const BoxCopy t = tasks[blockIdx.x];
    double* a = fs.f[t.slot];
    const int nkj = t.nk * t.nj;
    for (int q = threadIdx.x; q < t.npts; q += blockDim.x) {
        const int k = q % t.nk, j = (q / t.nk) % t.nj, i = q / nkj;
        a[t.dst + (long long)i * t.djj + (long long)j * t.dkk + k] =
            a[t.src + (long long)i * t.sjj + (long long)j * t.skk + k];
    }
}

struct FieldSlots32 {
    float* f[6];
};

__global__ void k_connect32(const BoxCopy* __restrict__ tasks, FieldSlots32 fs,
                            const int* __restrict__ skip) {
    if (skip && *skip) return;
    const BoxCopy t = tasks[blockIdx.x];
    float* a = fs.f[t.slot];
    const int nkj = t.nk * t.nj;
    for (int q = threadIdx.x; q < t.npts; q += blockDim.x) {
        const int k = q % t.nk, j = (q / t.nk) % t.nj, i = q / nkj;
        a[t.dst + (long long)i * t.djj + (long long)j * t.dkk + k] =
            a[t.src + (long long)i * t.sjj + (long long)j * t.skk + k];
    }
}

// Per-grid partial diagnostics: red[4g+0] = cflmax*0.25*dt, [4g+1] = divmax,
// [4g+2] = esum, [4g+3] = vsum.
__global__ void __launch_bounds__(256) k_itinfo(const DevGrid* __restrict__ grids,
                                                const double* __restrict__ U, const double* __restrict__ V,
                                                const double* __restrict__ W, const double* __restrict__ BP,
                                                const double* __restrict__ SDIV,
                                                const double* __restrict__ DX, const double* __restrict__ DY,
                                                const double* __restrict__ DZ, const double* __restrict__ DDX,
                                                const double* __restrict__ DDY, const double* __restrict__ DDZ,
                                                const double* __restrict__ RDDX, const double* __restrict__ RDDY,
                                                const double* __restrict__ RDDZ, double dt,
                                                double* __restrict__ red) {
    __shared__ double sh[4][32];
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const long long o = G.ip3;
    const double *u = U + o, *v = V + o, *w = W + o, *bp = BP + o, *sdiv = SDIV + o;
    const double *dx = DX + G.ipx - 1, *dy = DY + G.ipy - 1, *dz = DZ + G.ipz - 1;
    const double *ddx = DDX + G.ipx - 1, *ddy = DDY + G.ipy - 1, *ddz = DDZ + G.ipz - 1;
    const double *rddx = RDDX + G.ipx - 1, *rddy = RDDY + G.ipy - 1, *rddz = RDDZ + G.ipz - 1;
    double cm = 0.0, dm = 0.0, es = 0.0, vs = 0.0;
#define A(a, k, j, i) a[IX(k, j, i)]
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        double cflu = fabs(2.0 * A(u, k, j, i - 1) + (A(u, k, j, i) - A(u, k, j, i - 1)) * dx[i - 1] / ddx[i]) / ddx[i] +
                      fabs(2.0 * A(u, k, j, i) + (A(u, k, j, i + 1) - A(u, k, j, i)) * dx[i] / ddx[i + 1]) / ddx[i] +
                      fabs(A(v, k, j, i) + A(v, k, j, i + 1)) / ddy[j] +
                      fabs(A(v, k, j - 1, i) + A(v, k, j - 1, i + 1)) / ddy[j] +
                      fabs(A(w, k, j, i) + A(w, k, j, i + 1)) / ddz[k] +
                      fabs(A(w, k - 1, j, i) + A(w, k - 1, j, i + 1)) / ddz[k];
        cflu = cflu * A(bp, k, j, i) * A(bp, k, j, i + 1);
        double cflv = fabs(A(u, k, j, i) + A(u, k, j + 1, i)) / ddx[i] +
                      fabs(A(u, k, j, i - 1) + A(u, k, j + 1, i - 1)) / ddx[i] +
                      fabs(2.0 * A(v, k, j - 1, i) + (A(v, k, j, i) - A(v, k, j - 1, i)) * dy[j - 1] / ddy[j]) / ddy[j] +
                      fabs(2.0 * A(v, k, j, i) + (A(v, k, j + 1, i) - A(v, k, j, i)) * dy[j] / ddy[j + 1]) / ddy[j] +
                      fabs(A(w, k, j, i) + A(w, k, j + 1, i)) / ddz[k] +
                      fabs(A(w, k - 1, j, i) + A(w, k - 1, j + 1, i)) / ddz[k];
        cflv = cflv * A(bp, k, j, i) * A(bp, k, j + 1, i);
        double cflw = fabs(A(u, k, j, i) + A(u, k + 1, j, i)) / ddx[i] +
                      fabs(A(u, k, j, i - 1) + A(u, k + 1, j, i - 1)) / ddx[i] +
                      fabs(A(v, k, j, i) + A(v, k + 1, j, i)) / ddy[j] +
                      fabs(A(v, k, j - 1, i) + A(v, k + 1, j - 1, i)) / ddy[j] +
                      fabs(2.0 * A(w, k - 1, j, i) + (A(w, k, j, i) - A(w, k - 1, j, i)) * dz[k - 1] / ddz[k]) / ddz[k] +
                      fabs(2.0 * A(w, k, j, i) + (A(w, k + 1, j, i) - A(w, k, j, i)) * dz[k] / ddz[k + 1]) / ddz[k];
        cflw = cflw * A(bp, k, j, i) * A(bp, k + 1, j, i);
        double m = fmax(cflu, fmax(cflv, cflw));
        // NaN must propagate to the exploded check
        cm = (m > cm || m != m) ? m : cm;
        double div = A(sdiv, k, j, i) + (A(u, k, j, i) - A(u, k, j, i - 1)) * rddx[i] +
                     (A(v, k, j, i) - A(v, k, j - 1, i)) * rddy[j] +
                     (A(w, k, j, i) - A(w, k - 1, j, i)) * rddz[k];
        div = fabs(A(bp, k, j, i) * div);
        dm = (div > dm || div != div) ? div : dm;
        double up = A(u, k, j, i - 1) + (A(u, k, j, i) - A(u, k, j, i - 1)) * 0.5 * dx[i - 1] / ddx[i];
        double vp = A(v, k, j - 1, i) + (A(v, k, j, i) - A(v, k, j - 1, i)) * 0.5 * dy[j - 1] / ddy[j];
        double wp = A(w, k - 1, j, i) + (A(w, k, j, i) - A(w, k - 1, j, i)) * 0.5 * dz[k - 1] / ddz[k];
        double vol = ddx[i] * ddy[j] * ddz[k];
        es = es + vol * 0.5 * (up * up + vp * vp + wp * wp);
        vs = vs + vol;
    }
#undef A
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int off = 16; off > 0; off >>= 1) {
        double a = __shfl_xor_sync(0xffffffffu, cm, off);
        cm = (a > cm || a != a) ? a : cm;
        double b = __shfl_xor_sync(0xffffffffu, dm, off);
        dm = (b > dm || b != b) ? b : dm;
        es += __shfl_xor_sync(0xffffffffu, es, off);
        vs += __shfl_xor_sync(0xffffffffu, vs, off);
    }
    if (lane == 0) { sh[0][wid] = cm; sh[1][wid] = dm; sh[2][wid] = es; sh[3][wid] = vs; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
            cm = (sh[0][q] > cm || sh[0][q] != sh[0][q]) ? sh[0][q] : cm;
            dm = (sh[1][q] > dm || sh[1][q] != sh[1][q]) ? sh[1][q] : dm;
            es += sh[2][q];
            vs += sh[3][q];
        }
        red[4 * blockIdx.x + 0] = cm * 0.25 * dt;
        red[4 * blockIdx.x + 1] = dm;
        red[4 * blockIdx.x + 2] = es;
        red[4 * blockIdx.x + 3] = vs;
    }
}

}  // namespace

int launch_connect(Ctx* c, const ConnectPlan& plan, double* const fields[6]) {
    ProfScope ps_(c, "connect");
    if (plan.ntasks == 0) return 0;
    FieldSlots fs;
    for (int q = 0; q < 6; ++q) fs.f[q] = fields[q];
    k_connect<<<plan.ntasks, 128, 0, c->stream>>>(plan.d_tasks, fs);
    MG_LAUNCHED(c);
    return 0;
}

int launch_connect32(Ctx* c, const ConnectPlan& plan, float* const fields[6], const int* skip) {
    ProfScope ps_(c, "connect32");
    if (plan.ntasks == 0) return 0;
    FieldSlots32 fs;
    for (int q = 0; q < 6; ++q) fs.f[q] = fields[q];
    k_connect32<<<plan.ntasks, 128, 0, c->stream>>>(plan.d_tasks, fs, skip);
    MG_LAUNCHED(c);
    return 0;
}

int launch_itinfo(Ctx* c, double dt) {
    ProfScope ps_(c, "itinfo");
    k_itinfo<<<c->ngrid, 256, 0, c->stream>>>(c->d_grids, c->F("U"), c->F("V"), c->F("W"),
                                              c->F("BP"), c->F("SDIV"), c->L("DX"), c->L("DY"),
                                              c->L("DZ"), c->L("DDX"), c->L("DDY"), c->L("DDZ"),
                                              c->L("RDDX"), c->L("RDDY"), c->L("RDDZ"), dt,
                                              c->d_gridred);
    MG_LAUNCHED(c);
    return 0;
}

}  // namespace mg
