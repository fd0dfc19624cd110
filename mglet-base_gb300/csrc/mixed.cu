// mixed.cu -- the batched mixed-precision form of the RK stage.
//
// Same algorithm and data flow as the reference's mgpoisl
// (src/flow/pressuresolver_mod.F90:160-357): an FP64 defect-correction outer
// loop (laplacephi + rescal + maxabscal + accumulate_pcorr) around ninner SIP
// iterations per level (mgpoisit/sip, :361-465) with the lagged halo
// exchanges conn(res) and conn(dp) between them.  What changes:
//
//  * the inner iterations run in FP32: hilf, res and an FP32 copy of the
//    outer residual rhs, and FP32 SIP/Poisson coefficients.  The FP64 outer
//    loop measures the true residual of the accumulated correction, so the
//    converged pressure is an FP64 solution (the reference's own loop
//    structure, only the inner precision drops);
//  * grids with identical spacing, boundary types and BP share one
//    coefficient set ("coefficient class"); on a uniform periodic tiling all
//    4096 grids read the same 0.7 MB of FP32 coefficients from L2 instead
//    of 7 x 719 MB of FP64 fields from HBM;
//  * the SIP sweeps use a column wavefront: one CTA per grid, one thread per
//    (j, i) column.  At step t the thread works on k = t - (i-3) - (j-3) + 3,
//    so all active threads lie on the hyperplane i+j+k = t+9 -- the
//    reference's wavefront (sip_hyperplane_mod.F90:450-569).  res(k-1)
//    stays in a register, res(j-1) and res(i-1) come from a double-buffered
//    shared-memory plane written one step earlier;
//  * convergence is decided on the device: the outer-loop kernels check a
//    device flag and return at once after convergence, so a whole stage is
//    one CUDA graph with no host round trip (the reference's MPI_Allreduce
//    + host test per outer iteration).
//
// Compiled with FMA contraction on (the parity form lives in plain_*.cu).
#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <vector>

#include "mixed.h"

namespace mg {

int launch_mx_flux(Ctx* c, float* du, float* dv, float* dw, const float* sx, const float* sy,
                   const float* sz, double frhs, double dtfu);
int mx_flux_prepare(Ctx* c);

struct MixedState {
    int nclass = 0;
    std::vector<int> gcls;          // coefficient class of each grid
    int* d_gcls = nullptr;
    long long cls_stride = 0;       // points per class slab (kk*jj*ii of the shape)
    // FP32 class coefficients, natural layout per class slab
    float *lw = nullptr, *ls = nullptr, *lb = nullptr, *lpr = nullptr;
    float *ue = nullptr, *un = nullptr, *ut = nullptr, *ap32 = nullptr;
    double* ap64 = nullptr;
    // FP32 inner-solver fields (natural layout with ghosts, like field_t%arr)
    float *h32 = nullptr, *r32 = nullptr, *rhs32 = nullptr;
    // FP32 2N-storage registers DU, DV, DW of the RK scheme
    float *du32 = nullptr, *dv32 = nullptr, *dw32 = nullptr;
    // FP32 spacing tables per axis: d, dd, rd, rdd, d(i)/dd(i+1), d(i-1)/dd(i)
    float *sx = nullptr, *sy = nullptr, *sz = nullptr;
    bool g_uniform = true;
    // device control block: [0] converged flag, [1] outer iterations done
    int* d_ctl = nullptr;
    double* d_maxrhs = nullptr;
    int* h_ctl = nullptr;           // pinned mirror
    double* h_maxrhs = nullptr;
    int maxcols = 0;
    // graph cache: (irk, dt, frhs, fu, dtrk bit patterns) -> executable graph
    // of the whole stage, and the number of kernels inside it
    using GraphKey = std::array<unsigned long long, 5>;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::map<GraphKey, long long> graph_launches;
};

namespace {

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

// ---------------------------------------------------------------------------
// Coefficient classes: copy the representative grid's FP64 SIP coefficients
// (hyperplane order for "sip", natural order for "classic") to FP32 natural
// layout, and its GSAP to the FP32/FP64 class slabs.
__global__ void k_extract(const DevGrid* __restrict__ grids, const int* __restrict__ reps,
                          const int* const* __restrict__ idxs, int planeorder, long long stride,
                          const double* __restrict__ lw, const double* __restrict__ ls,
                          const double* __restrict__ lb, const double* __restrict__ lpr,
                          const double* __restrict__ ue, const double* __restrict__ un,
                          const double* __restrict__ ut, const double* __restrict__ ap,
                          float* olw, float* ols, float* olb, float* olpr, float* oue, float* oun,
                          float* out, float* oap, double* oap64) {
    const int cls = blockIdx.y;
    const DevGrid G = grids[reps[cls]];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int npts = (kk - 4) * (jj - 4) * (ii - 4);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    const int id = idxs[G.cls][q];                // natural local index of plane entry q
    const long long src = G.ip3 + (planeorder ? q : id);
    const long long dst = cls * stride + id;
    olw[dst] = (float)lw[src]; ols[dst] = (float)ls[src]; olb[dst] = (float)lb[src];
    olpr[dst] = (float)lpr[src]; oue[dst] = (float)ue[src]; oun[dst] = (float)un[src];
    out[dst] = (float)ut[src];
    oap[dst] = (float)ap[G.ip3 + id];
    oap64[dst] = ap[G.ip3 + id];
}

struct Coef1 {
    const double *aw, *ae, *as, *an, *ab, *at;
};

// ---------------------------------------------------------------------------
// mixed divcal: FP64 divergence (noib_mod.F90:304-354) into rhs, plus its
// FP32 copy for the inner iterations.
__global__ void k_mx_divcal(const DevGrid* __restrict__ grids, double* __restrict__ RHS,
                            float* __restrict__ RHS32, const double* __restrict__ U,
                            const double* __restrict__ V, const double* __restrict__ W,
                            const double* __restrict__ RDDX, const double* __restrict__ RDDY,
                            const double* __restrict__ RDDZ, double fak) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj * nk) return;
    const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
    const long long o = G.ip3;
    const long long c = IX(k, j, i);
    const double *u = U + o, *v = V + o, *w = W + o;
    const double d = fak * ((u[c] - u[IX(k, j, i - 1)]) * RDDX[G.ipx + i - 1] +
                            (v[c] - v[IX(k, j - 1, i)]) * RDDY[G.ipy + j - 1] +
                            (w[c] - w[IX(k - 1, j, i)]) * RDDZ[G.ipz + k - 1]);
    RHS[o + c] = d;
    RHS32[o + c] = (float)d;
}

// ---------------------------------------------------------------------------
// Forward sweep: res = -A hilf (laplacephi_grid, bp = 1) then
// res = (rhs + res) lpr - lb res(k-1) - ls res(j-1) - lw res(i-1), on the
// column wavefront.  Ghost values of hilf and res come from conn.
template <int MAXC>
__global__ void __launch_bounds__(1024) k_mx_fwd(const DevGrid* __restrict__ grids,
                                                 const int* __restrict__ gcls, long long cstride,
                                                 const float* __restrict__ H,
                                                 const float* __restrict__ RHS, float* R,
                                                 const float* __restrict__ LW, const float* __restrict__ LS,
                                                 const float* __restrict__ LB, const float* __restrict__ LPR,
                                                 const float* __restrict__ AP, Coef1 cf,
                                                 const int* __restrict__ conv) {
    if (*conv) return;
    __shared__ float xb[2][MAXC];
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int col = threadIdx.x;
    const bool on = col < ni * nj;
    const int jo = on ? col % nj : 0, io = on ? col / nj : 0;   // 0-based column
    const int j = jo + 3, i = io + 3;
    const long long o = G.ip3;
    const long long co = (long long)gcls[blockIdx.x] * cstride;
    const float *h = H + o, *rhs = RHS + o;
    float* res = R + o;
    const float *lw = LW + co, *ls = LS + co, *lb = LB + co, *lpr = LPR + co, *ap = AP + co;
    const float aw = (float)cf.aw[G.ipx + i - 1], ae = (float)cf.ae[G.ipx + i - 1];
    const float as = (float)cf.as[G.ipy + j - 1], an = (float)cf.an[G.ipy + j - 1];
    const int kj = kk * jj;
    float rprev = 0.f;
    const int nsteps = ni + nj + nk - 2;
    for (int t = 0; t < nsteps; ++t) {
        const int kx = t - io - jo;
        if (on && kx >= 0 && kx < nk) {
            const int k = kx + 3;
            const long long c = IX(k, j, i);
            const float ab = (float)cf.ab[G.ipz + k - 1], at = (float)cf.at[G.ipz + k - 1];
            float lap = -aw * h[c - kj] - ae * h[c + kj] - as * h[c - kk] - an * h[c + kk] -
                        ab * h[c - 1] - at * h[c + 1] - ap[c] * h[c];
            const float rkm = (k == 3) ? res[c - 1] : rprev;
            const float rjm = (j == 3) ? res[c - kk] : xb[(t + 1) & 1][col - 1];
            const float rim = (i == 3) ? res[c - kj] : xb[(t + 1) & 1][col - nj];
            float r = (rhs[c] + lap) * lpr[c];
            r = r - lb[c] * rkm - ls[c] * rjm - lw[c] * rim;
            res[c] = r;
            xb[t & 1][col] = r;
            rprev = r;
        }
        __syncthreads();
    }
}

// Backward sweep: res = res - ut res(k+1) - un res(j+1) - ue res(i+1) in
// reverse wavefront order, then hilf += res.
template <int MAXC>
__global__ void __launch_bounds__(1024) k_mx_bwd(const DevGrid* __restrict__ grids,
                                                 const int* __restrict__ gcls, long long cstride,
                                                 float* H, const float* __restrict__ R,
                                                 const float* __restrict__ UE, const float* __restrict__ UN,
                                                 const float* __restrict__ UT,
                                                 const int* __restrict__ conv) {
    if (*conv) return;
    __shared__ float xb[2][MAXC];
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int col = threadIdx.x;
    const bool on = col < ni * nj;
    const int jo = on ? col % nj : 0, io = on ? col / nj : 0;
    const int j = jo + 3, i = io + 3;
    const int jr = nj - 1 - jo, ir = ni - 1 - io;   // distance from the high faces
    const long long o = G.ip3;
    const long long co = (long long)gcls[blockIdx.x] * cstride;
    float* h = H + o;
    const float* res = R + o;
    const float *ue = UE + co, *un = UN + co, *ut = UT + co;
    const int kj = kk * jj;
    float rprev = 0.f;
    const int nsteps = ni + nj + nk - 2;
    for (int t = 0; t < nsteps; ++t) {
        const int kr = t - ir - jr;
        if (on && kr >= 0 && kr < nk) {
            const int k = kk - 2 - kr;
            const long long c = IX(k, j, i);
            const float rkp = (k == kk - 2) ? res[c + 1] : rprev;
            const float rjp = (j == jj - 2) ? res[c + kk] : xb[(t + 1) & 1][col + 1];
            const float rip = (i == ii - 2) ? res[c + kj] : xb[(t + 1) & 1][col + nj];
            float r = res[c] - ut[c] * rkp - un[c] * rjp - ue[c] * rip;
            h[c] = h[c] + r;
            xb[t & 1][col] = r;
            rprev = r;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ double block_max_d(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    __syncthreads();
    return v;
}

// Outer step in FP64: res = -A hilf (laplacephi), rhs += res (rescal),
// max|rhs| per grid (maxabscal_grid), dp += hilf (accumulate_pcorr),
// rhs32 = rhs, hilf = 0.
__global__ void __launch_bounds__(512) k_mx_outer(const DevGrid* __restrict__ grids,
                                                  const int* __restrict__ gcls, long long cstride,
                                                  float* H, double* __restrict__ RHS,
                                                  float* __restrict__ RHS32, double* __restrict__ DP,
                                                  const double* __restrict__ AP64, Coef1 cf,
                                                  double* __restrict__ gridmax,
                                                  const int* __restrict__ conv) {
    if (*conv) return;
    __shared__ double sh[32];
    const DevGrid G = grids[blockIdx.x];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const long long o = G.ip3;
    const long long co = (long long)gcls[blockIdx.x] * cstride;
    float* h = H + o;
    const double* ap = AP64 + co;
    const int kj = kk * jj;
    double m = 0.0;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        const long long c = IX(k, j, i);
        const double hc = h[c];
        const double lap = -cf.aw[G.ipx + i - 1] * (double)h[c - kj] -
                           cf.ae[G.ipx + i - 1] * (double)h[c + kj] -
                           cf.as[G.ipy + j - 1] * (double)h[c - kk] -
                           cf.an[G.ipy + j - 1] * (double)h[c + kk] -
                           cf.ab[G.ipz + k - 1] * (double)h[c - 1] -
                           cf.at[G.ipz + k - 1] * (double)h[c + 1] - ap[c] * hc;
        const double r = RHS[o + c] + lap;
        RHS[o + c] = r;
        RHS32[o + c] = (float)r;
        DP[o + c] = DP[o + c] + hc;
        m = fmax(fabs(r), m);
    }
    m = block_max_d(m, sh);
    if (threadIdx.x == 0) gridmax[blockIdx.x] = m;
    // all reads of this grid's hilf (interior and ghosts) are done
    const int npt = kk * jj * ii;
    for (int t = threadIdx.x; t < npt; t += blockDim.x) h[t] = 0.f;
}

// maxabscal over grids + the outer-loop stopping test of mgpoisl
// (pressuresolver_mod.F90:275,294-301), on the device.
__global__ void k_mx_conv(const DevGrid* __restrict__ grids, int ngrid, int maxlevel,
                          const double* __restrict__ gridmax, int* ctl, double* maxrhs,
                          double prefak, double epcorr, int nouter_min) {
    if (ctl[0]) return;
    __shared__ double sh[32];
    double m = 0.0;
    for (int g = threadIdx.x; g < ngrid; g += blockDim.x)
        m = fmax(fabs(gridmax[g] * ldexp(1.0, maxlevel - grids[g].level)), m);
    m = block_max_d(m, sh);
    if (threadIdx.x == 0) {
        const int done = ctl[1] + 1;
        ctl[1] = done;
        maxrhs[0] = m;
        if (done >= nouter_min && m / prefak < epcorr) ctl[0] = 1;
    }
}

// mgpcorr on the interior only (the ghost layers it also touches in the
// reference are overwritten by the closing connect), FP64.
__global__ void k_mx_mgpcorr(const DevGrid* __restrict__ grids, double* U, double* V, double* W,
                             double* P, const double* __restrict__ DP, const double* __restrict__ RDX,
                             const double* __restrict__ RDY, const double* __restrict__ RDZ,
                             double rfak) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj * nk) return;
    const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
    const long long o = G.ip3;
    const double* dp = DP + o;
    const long long c = IX(k, j, i);
    const double d = dp[c];
    P[o + c] = P[o + c] + d;
    U[o + c] = U[o + c] + (d - dp[c + (long long)kk * jj]) * RDX[G.ipx + i - 1] * rfak;
    V[o + c] = V[o + c] + (d - dp[c + kk]) * RDY[G.ipy + j - 1] * rfak;
    W[o + c] = W[o + c] + (d - dp[c + 1]) * RDZ[G.ipz + k - 1] * rfak;
}

int interior_max(const Ctx* c) {
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, (g.kk - 4) * (g.jj - 4) * (g.ii - 4));
    return m;
}

Coef1 coef1(Ctx* c) {
    return Coef1{c->L("GSAW"), c->L("GSAE"), c->L("GSAS"), c->L("GSAN"), c->L("GSAB"), c->L("GSAT")};
}

int enqueue_mgpoisl(Ctx* c, double dt) {
    MixedState* m = c->mx;
    const double prefak = c->prm.rho / dt;
    double* U = c->F("U"); double* V = c->F("V"); double* W = c->F("W"); double* P = c->F("P");
    double* dp = c->F("DP"); double* rhs = c->F("RHS");
    const size_t b8 = (size_t)c->idim3d * sizeof(double), b4 = (size_t)c->idim3d * sizeof(float);
    MG_CUDA(cudaMemsetAsync(dp, 0, b8, c->stream));
    MG_CUDA(cudaMemsetAsync(rhs, 0, b8, c->stream));
    MG_CUDA(cudaMemsetAsync(m->h32, 0, b4, c->stream));
    MG_CUDA(cudaMemsetAsync(m->r32, 0, b4, c->stream));
    MG_CUDA(cudaMemsetAsync(m->d_ctl, 0, 2 * sizeof(int), c->stream));
    {
        ProfScope ps_(c, "mx_divcal");
        dim3 grid((interior_max(c) + 255) / 256, c->ngrid);
        k_mx_divcal<<<grid, 256, 0, c->stream>>>(c->d_grids, rhs, m->rhs32, U, V, W, c->L("RDDX"),
                                                 c->L("RDDY"), c->L("RDDZ"), prefak);
        MG_LAUNCHED(c);
    }
    const ConnectPlan *p_all, *p_hi;
    if (int rc = get_plan(c, 0, 1, 1 << 3, false, false, 0, &p_all)) return rc;
    if (int rc = get_plan(c, 0, 1, 1 << 3, false, false, -1, &p_hi)) return rc;
    float* slot_r[6] = {nullptr, nullptr, nullptr, m->r32, nullptr, nullptr};
    float* slot_h[6] = {nullptr, nullptr, nullptr, m->h32, nullptr, nullptr};
    const int* conv = m->d_ctl;
    const Coef1 cf = coef1(c);
    const int threads = ((m->maxcols + 31) / 32) * 32;
    for (int ipcount = 1; ipcount <= c->prm.nouter; ++ipcount) {
        for (int iloop = 1; iloop <= c->prm.ninner; ++iloop) {
            {
                ProfScope ps_(c, "mx_sip_fwd");
                if (m->maxcols <= 576)
                    k_mx_fwd<576><<<c->ngrid, threads, 0, c->stream>>>(
                        c->d_grids, m->d_gcls, m->cls_stride, m->h32, m->rhs32, m->r32, m->lw, m->ls,
                        m->lb, m->lpr, m->ap32, cf, conv);
                else
                    k_mx_fwd<1024><<<c->ngrid, threads, 0, c->stream>>>(
                        c->d_grids, m->d_gcls, m->cls_stride, m->h32, m->rhs32, m->r32, m->lw, m->ls,
                        m->lb, m->lpr, m->ap32, cf, conv);
                MG_LAUNCHED(c);
            }
            if (int rc = launch_connect32(c, iloop < c->prm.ninner ? *p_all : *p_hi, slot_r, conv))
                return rc;
            {
                ProfScope ps_(c, "mx_sip_bwd");
                if (m->maxcols <= 576)
                    k_mx_bwd<576><<<c->ngrid, threads, 0, c->stream>>>(
                        c->d_grids, m->d_gcls, m->cls_stride, m->h32, m->r32, m->ue, m->un, m->ut, conv);
                else
                    k_mx_bwd<1024><<<c->ngrid, threads, 0, c->stream>>>(
                        c->d_grids, m->d_gcls, m->cls_stride, m->h32, m->r32, m->ue, m->un, m->ut, conv);
                MG_LAUNCHED(c);
            }
            if (int rc = launch_connect32(c, *p_all, slot_h, conv)) return rc;
        }
        {
            ProfScope ps_(c, "mx_outer");
            k_mx_outer<<<c->ngrid, 512, 0, c->stream>>>(c->d_grids, m->d_gcls, m->cls_stride, m->h32,
                                                        rhs, m->rhs32, dp, m->ap64, cf, c->d_gridred,
                                                        conv);
            MG_LAUNCHED(c);
            k_mx_conv<<<1, 1024, 0, c->stream>>>(c->d_grids, c->ngrid, c->maxlevel, c->d_gridred,
                                                 m->d_ctl, m->d_maxrhs, prefak, c->prm.epcorr,
                                                 c->prm.nouter_min);
            MG_LAUNCHED(c);
        }
    }
    // dp ghosts (the reference accumulates the connected hilf ghosts into dp)
    if (int rc = connect(c, 0, 1, nullptr, nullptr, nullptr, dp, nullptr, nullptr, false, false, 0))
        return rc;
    {
        ProfScope ps_(c, "mx_mgpcorr");
        dim3 grid((interior_max(c) + 255) / 256, c->ngrid);
        k_mx_mgpcorr<<<grid, 256, 0, c->stream>>>(c->d_grids, U, V, W, P, dp, c->L("RDX"),
                                                  c->L("RDY"), c->L("RDZ"), dt / c->prm.rho);
        MG_LAUNCHED(c);
    }
    if (int rc = connect(c, 0, 2, U, V, W, P, nullptr, nullptr, true, false, 0)) return rc;
    MG_CUDA(cudaMemcpyAsync(m->h_ctl, m->d_ctl, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaMemcpyAsync(m->h_maxrhs, m->d_maxrhs, sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    return 0;
}

int enqueue_stage(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk) {
    double frhs, fu, dtrk, dtrki;
    if (int rc = rk_coeffs(rk, irk, &frhs, &fu, &dtrk, &dtrki)) return rc;
    double *U = c->F("U"), *V = c->F("V"), *W = c->F("W"), *P = c->F("P"), *G = c->F("G");
    double *UO = c->F("UO"), *VO = c->F("VO"), *WO = c->F("WO");
    MixedState* m = c->mx;
    (void)P; (void)G; (void)UO; (void)VO; (void)WO;
    if (!m->g_uniform) {
        set_error("mixed form: needs a uniform viscosity field G = gmol (no LES model)");
        return MGLET_ERR_UNSUPPORTED;
    }
    if (int rc = launch_mx_flux(c, m->du32, m->dv32, m->dw32, m->sx, m->sy, m->sz, frhs, dt * fu))
        return rc;
    if (int rc = connect(c, 0, 1, U, V, W, nullptr, nullptr, nullptr, false, true, 1)) return rc;
    return enqueue_mgpoisl(c, dtrk * dt);
}

void fill_stats(Ctx* c, double dt, mglet_stage_stats* st) {
    MixedState* m = c->mx;
    st->nouter_done = m->h_ctl[1];
    st->ipc = m->h_ctl[1] * c->prm.ninner;
    st->maxrhs = m->h_maxrhs[0];
    st->prefak = c->prm.rho / dt;
}

}  // namespace

int mixed_init(Ctx* c) {
    if (c->minlevel != c->maxlevel) {
        set_error("mixed form: one grid level only");
        return MGLET_ERR_UNSUPPORTED;
    }
    MixedState* m = new MixedState();
    c->mx = m;
    // coefficient classes: same dims, BC types and spacing arrays
    std::vector<std::vector<double>> sp(9);
    const char* names[9] = {"DX", "DY", "DZ", "DDX", "DDY", "DDZ", "X", "Y", "Z"};
    const long long lens[3] = {c->idimx, c->idimy, c->idimz};
    for (int q = 0; q < 6; ++q) {
        sp[q].resize(lens[q % 3]);
        MG_CUDA(cudaMemcpy(sp[q].data(), c->L(names[q]), lens[q % 3] * sizeof(double),
                           cudaMemcpyDeviceToHost));
    }
    std::vector<int> reps;
    m->gcls.assign(c->ngrid, -1);
    std::map<std::vector<double>, int> seen;
    for (int g = 0; g < c->ngrid; ++g) {
        const DevGrid& G = c->grids[g];
        std::vector<double> key = {(double)G.kk, (double)G.jj, (double)G.ii};
        for (int f = 0; f < 6; ++f) key.push_back(G.bc[f]);
        const int off[3] = {G.ipx, G.ipy, G.ipz};
        const int len[3] = {G.ii, G.jj, G.kk};
        for (int q = 0; q < 6; ++q)
            key.insert(key.end(), sp[q].begin() + off[q % 3], sp[q].begin() + off[q % 3] + len[q % 3]);
        auto it = seen.find(key);
        if (it == seen.end()) {
            it = seen.emplace(key, (int)reps.size()).first;
            reps.push_back(g);
        }
        m->gcls[g] = it->second;
        m->maxcols = std::max(m->maxcols, (G.ii - 4) * (G.jj - 4));
    }
    if (m->maxcols > 1024) {
        set_error("mixed form: more than 1024 (j, i) columns per grid");
        return MGLET_ERR_UNSUPPORTED;
    }
    if (!c->uniform) {
        set_error("mixed form: all grids must have the same dimensions");
        return MGLET_ERR_UNSUPPORTED;
    }
    if (int rc = mx_flux_prepare(c)) return rc;
    // FP32 spacing tables
    {
        const long long n3[3] = {c->idimx, c->idimy, c->idimz};
        float** dst[3] = {&m->sx, &m->sy, &m->sz};
        for (int ax = 0; ax < 3; ++ax) {
            const long long n = n3[ax];
            const std::vector<double>& d = sp[ax];
            const std::vector<double>& dd = sp[ax + 3];
            std::vector<float> tb(6 * n, 0.f);
            for (int g = 0; g < c->ngrid; ++g) {
                const DevGrid& G = c->grids[g];
                const int off = ax == 0 ? G.ipx : (ax == 1 ? G.ipy : G.ipz);
                const int len = ax == 0 ? G.ii : (ax == 1 ? G.jj : G.kk);
                for (int q = 0; q < len; ++q) {
                    const long long x = off + q;
                    tb[x] = (float)d[x];
                    tb[n + x] = (float)dd[x];
                    tb[2 * n + x] = d[x] == 0.0 ? 0.f : (float)(1.0 / d[x]);
                    tb[3 * n + x] = dd[x] == 0.0 ? 0.f : (float)(1.0 / dd[x]);
                    tb[4 * n + x] = q + 1 < len ? (float)(d[x] / dd[x + 1]) : 0.f;
                    tb[5 * n + x] = q > 0 ? (float)(d[x - 1] / dd[x]) : 0.f;
                }
            }
            MG_CUDA(cudaMalloc(dst[ax], tb.size() * sizeof(float)));
            MG_CUDA(cudaMemcpy(*dst[ax], tb.data(), tb.size() * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    m->nclass = (int)reps.size();
    long long stride = 0;
    for (const DevGrid& G : c->grids) stride = std::max(stride, (long long)G.kk * G.jj * G.ii);
    m->cls_stride = stride;
    const size_t ncoef = (size_t)m->nclass * stride;
    for (float** p : {&m->lw, &m->ls, &m->lb, &m->lpr, &m->ue, &m->un, &m->ut, &m->ap32}) {
        MG_CUDA(cudaMalloc(p, ncoef * sizeof(float)));
        MG_CUDA(cudaMemset(*p, 0, ncoef * sizeof(float)));
    }
    MG_CUDA(cudaMalloc(&m->ap64, ncoef * sizeof(double)));
    MG_CUDA(cudaMemset(m->ap64, 0, ncoef * sizeof(double)));
    for (float** p : {&m->h32, &m->r32, &m->rhs32, &m->du32, &m->dv32, &m->dw32}) {
        MG_CUDA(cudaMalloc(p, (size_t)c->idim3d * sizeof(float)));
        MG_CUDA(cudaMemset(*p, 0, (size_t)c->idim3d * sizeof(float)));
    }
    MG_CUDA(cudaMalloc(&m->d_gcls, c->ngrid * sizeof(int)));
    MG_CUDA(cudaMemcpy(m->d_gcls, m->gcls.data(), c->ngrid * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMalloc(&m->d_ctl, 4 * sizeof(int)));
    MG_CUDA(cudaMalloc(&m->d_maxrhs, sizeof(double)));
    MG_CUDA(cudaMallocHost(&m->h_ctl, 4 * sizeof(int)));
    MG_CUDA(cudaMallocHost(&m->h_maxrhs, sizeof(double)));
    // every connect variant the stage issues, built before any graph capture
    const ConnectPlan* pl;
    if (int rc = get_plan(c, 0, 1, 1 << 3, false, false, 0, &pl)) return rc;
    if (int rc = get_plan(c, 0, 1, 1 << 3, false, false, -1, &pl)) return rc;
    if (int rc = get_plan(c, 0, 1, 7, false, true, 1, &pl)) return rc;
    if (int rc = get_plan(c, 0, 2, 15, true, false, 0, &pl)) return rc;
    for (int l = c->minlevel; l <= c->maxlevel; ++l)
        if (int rc = get_plan(c, l, 1, 7, false, true, 1, &pl)) return rc;
    // extract class coefficients from the representative grids
    int* d_reps = nullptr;
    MG_CUDA(cudaMalloc(&d_reps, reps.size() * sizeof(int)));
    MG_CUDA(cudaMemcpy(d_reps, reps.data(), reps.size() * sizeof(int), cudaMemcpyHostToDevice));
    std::vector<const int*> hi;
    for (const HpTable& t : c->hp) hi.push_back(t.d_idx);
    const int** d_idxs = nullptr;
    MG_CUDA(cudaMalloc(&d_idxs, hi.size() * sizeof(int*)));
    MG_CUDA(cudaMemcpy(d_idxs, hi.data(), hi.size() * sizeof(int*), cudaMemcpyHostToDevice));
    dim3 grid((interior_max(c) + 255) / 256, m->nclass);
    k_extract<<<grid, 256, 0, c->stream>>>(
        c->d_grids, d_reps, d_idxs, c->prm.psolver == MGLET_PSOLVER_CLASSIC ? 0 : 1, stride,
        c->F("SIPLW"), c->F("SIPLS"), c->F("SIPLB"), c->F("SIPLPR"), c->F("SIPUE"), c->F("SIPUN"),
        c->F("SIPUT"), c->F("GSAP"), m->lw, m->ls, m->lb, m->lpr, m->ue, m->un, m->ut, m->ap32,
        m->ap64);
    c->launches++;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(d_reps);
    cudaFree((void*)d_idxs);
    if (e != cudaSuccess) return cuda_fail(e, "mixed_init");
    return 0;
}

void mixed_release(Ctx* c) {
    MixedState* m = c->mx;
    if (!m) return;
    for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
    for (void* p : {(void*)m->lw, (void*)m->ls, (void*)m->lb, (void*)m->lpr, (void*)m->ue,
                    (void*)m->un, (void*)m->ut, (void*)m->ap32, (void*)m->ap64, (void*)m->h32,
                    (void*)m->r32, (void*)m->rhs32, (void*)m->d_gcls, (void*)m->d_ctl,
                    (void*)m->d_maxrhs, (void*)m->du32, (void*)m->dv32, (void*)m->dw32,
                    (void*)m->sx, (void*)m->sy, (void*)m->sz})
        cudaFree(p);
    if (m->h_ctl) cudaFreeHost(m->h_ctl);
    if (m->h_maxrhs) cudaFreeHost(m->h_maxrhs);
    delete m;
    c->mx = nullptr;
}

__global__ void k_cvt_64_32(float* d, const double* s, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) d[t] = (float)s[t];
}
__global__ void k_cvt_32_64(double* d, const float* s, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) d[t] = (double)s[t];
}

static float* du_buffer(Ctx* c, const char* name) {
    MixedState* m = c->mx;
    if (!m) return nullptr;
    if (!std::strcmp(name, "DU")) return m->du32;
    if (!std::strcmp(name, "DV")) return m->dv32;
    if (!std::strcmp(name, "DW")) return m->dw32;
    return nullptr;
}

// A field was uploaded: the FP32 RK registers follow DU/DV/DW, and a
// viscosity field that is not the uniform gmol takes the stage off the
// mixed path (LES models are outside this form).
void mixed_field_changed(Ctx* c, const char* name) {
    MixedState* m = c->mx;
    if (!m) return;
    if (!std::strcmp(name, "G")) m->g_uniform = false;
    if (float* f = du_buffer(c, name)) {
        k_cvt_64_32<<<(unsigned)((c->idim3d + 255) / 256), 256, 0, c->stream>>>(f, c->F(name), c->idim3d);
        cudaStreamSynchronize(c->stream);
    }
}

// Before a download: DU/DV/DW live in FP32 in this form.
void mixed_field_sync_out(Ctx* c, const char* name) {
    if (float* f = du_buffer(c, name)) {
        k_cvt_32_64<<<(unsigned)((c->idim3d + 255) / 256), 256, 0, c->stream>>>(c->F(name), f, c->idim3d);
    }
}

int mixed_mgpoisl(Ctx* c, double dt, mglet_stage_stats* st) {
    if (int rc = enqueue_mgpoisl(c, dt)) return rc;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    fill_stats(c, dt, st);
    return 0;
}

// One stage: captured once per (irk, dt) into a CUDA graph and replayed; with
// per-kernel profiling enabled the stage is issued eagerly so that every
// launch is bracketed by its events.
int mixed_stage(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk, mglet_stage_stats* st) {
    MixedState* m = c->mx;
    double frhs, fu, dtrk, dtrki;
    if (int rc = rk_coeffs(rk, irk, &frhs, &fu, &dtrk, &dtrki)) return rc;
    if (c->prof) {
        if (int rc = enqueue_stage(c, dt, irk, rk)) return rc;
    } else {
        MixedState::GraphKey k;
        const double vals[4] = {dt, frhs, fu, dtrk};
        k[0] = (unsigned long long)irk;
        for (int q = 0; q < 4; ++q) std::memcpy(&k[q + 1], &vals[q], sizeof(double));
        auto it = m->graphs.find(k);
        if (it == m->graphs.end()) {
            cudaGraph_t g;
            const long long l0 = c->launches;
            MG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_stage(c, dt, irk, rk);
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (rc) return rc;
            if (e != cudaSuccess) return cuda_fail(e, "graph capture");
            cudaGraphExec_t ex;
            e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
            it = m->graphs.emplace(k, ex).first;
            m->graph_launches[k] = c->launches - l0;
            c->launches = l0;
        }
        MG_CUDA(cudaGraphLaunch(it->second, c->stream));
        c->launches += m->graph_launches[k];
    }
    if (st) {
        MG_CUDA(cudaStreamSynchronize(c->stream));
        fill_stats(c, dtrk * dt, st);
    }
    return 0;
}

}  // namespace mg
