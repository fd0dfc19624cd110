// mixed.cu -- the batched mixed-precision form of the RK stage.
//
// Same algorithm and data flow as the reference's timeintegrate_flow +
// mgpoisl (src/flow/timeintegration_mod.F90:22-142,
// src/flow/pressuresolver_mod.F90:160-357): an FP64 defect-correction outer
// loop (laplacephi + rescal + maxabscal + accumulate_pcorr) around ninner SIP
// iterations with the lagged halo exchanges of the reference.  What changes:
//
//  * momentum RHS and RK update: one fused FP32 kernel over FP64 velocity
//    storage (mixed_flux.cu);
//  * inner SIP iterations in FP32, hyperplane layout, halos pulled from
//    the neighbours' plane-ordered arrays (mixed_sip.cu); the FP64 outer loop measures the
//    true residual of the accumulated correction, so the converged pressure
//    is an FP64 solution;
//  * grids with identical spacing and boundary types share one coefficient
//    set ("coefficient class"); on a uniform periodic tiling all grids read
//    the same ~0.4 MB of FP32 SIP factors, which stay in L2;
//  * convergence is decided on the device: the outer-loop kernels check a
//    device flag and return at once after convergence, so a whole stage is
//    one CUDA graph with no host round trip (the reference's
//    MPI_Allreduce + host test per outer iteration).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <cstring>
#include <map>
#include <vector>

#include "mixed.h"
#include "mixed_level.h"
#include "mixed_sip.h"

namespace mg {

int launch_mx_flux(Ctx* c, float* du, float* dv, float* dw, const float* sx, const float* sy,
                   const float* sz, const double* sprm, int* err, bool skip);
bool mx_flux_has_tma(Ctx* c);
int mx_flux_set_pw(Ctx* c, const unsigned char* d_pw);
void mx_flux_set_gfield(Ctx* c);
int mx_flux_prepare(Ctx* c);
void mx_flux_release(Ctx* c);
int mx_flux_tune(Ctx* c, float* du, float* dv, float* dw, const float* sx, const float* sy,
                 const float* sz, const double* sprm, int* err);
int mx_flux_force(Ctx* c, int v);
std::string mx_flux_tuning(Ctx* c);

struct MixedState {
    int nclass = 0;
    std::vector<int> gcls;          // coefficient class of each grid
    int* d_gcls = nullptr;
    // class coefficients in padded plane order: FP32 blocks [lw|ls|lb|lpr|ap]
    // and [ue|un|ut], FP64 ap
    float *cf = nullptr, *cb = nullptr;
    float* apx = nullptr;      // class ap as two floats (outer step)
    SipState sip;
    const int* d_idx = nullptr;     // plane position -> natural local index (hp table)
    // FP32 2N-storage registers DU, DV, DW of the RK scheme (natural layout)
    float *du32 = nullptr, *dv32 = nullptr, *dw32 = nullptr;
    // FP32 spacing tables per axis: d, dd, rd, rdd, d(i)/dd(i+1), d(i-1)/dd(i)
    float *sx = nullptr, *sy = nullptr, *sz = nullptr;
    bool walls = false;             // some grid has a FIX, OP1, NOS or SLI face
    LevelState lv;                  // hierarchies: per-level lists (set up at the first stage)
    // device control block: [0] converged flag, [1] outer iterations done
    int* d_ctl = nullptr;
    // stage scalars read by the kernels from device memory, so that one
    // captured graph serves every stage and every time step size:
    // [0] frhs, [1] dt*fu, [2] prefak = rho/dt of the solve, [3] dt/rho
    double* d_sprm = nullptr;
    double* d_maxrhs = nullptr;
    int* h_ctl = nullptr;           // pinned mirrors
    double* h_maxrhs = nullptr;
    // the whole stage captured once as a graph (its scalars come from
    // d_sprm), and the number of kernels inside it
    cudaGraphExec_t graph = nullptr;
    long long graph_launches = 0;
    // test switch (mglet_gpu_test_wait_timeout): the next stage's flux kernel
    // leaves one plane's copy out, so its bounded wait runs out
    bool skip_once = false;
};

namespace {

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

// mgpcorr (pressuresolver_mod.F90:808-844; BPF non-null: the bp form of the
// ghost-cell IB) over the reference's ranges -- the pressure on the box
// 2..n-1, each velocity on its faces 2..n-2 along its own axis -- in FP64,
// with dt/rho from the stage scalars.
__global__ void k_mx_mgpcorr(const DevGrid* __restrict__ grids, double* U, double* V, double* W,
                             double* P, const double* __restrict__ DP, const double* __restrict__ RDX,
                             const double* __restrict__ RDY, const double* __restrict__ RDZ,
                             const double* __restrict__ sprm, const double* __restrict__ BPF) {
    const DevGrid G = grids[blockIdx.y];
    const double rfak = sprm[3];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    const long long o = G.ip3;
    const double* dp = DP + o;
    const long long c = IX(k, j, i);
    const bool pi = i >= 2 && i <= ii - 1, pj = j >= 2 && j <= jj - 1, pk = k >= 2 && k <= kk - 1;
    const bool ci = i >= 3 && i <= ii - 2, cj = j >= 3 && j <= jj - 2, ck = k >= 3 && k <= kk - 2;
    if (!(pi && pj && pk)) return;
    const double d = dp[c];
    if (BPF) {
        const double* bp = BPF + o;
        P[o + c] = P[o + c] + d * bp[c];
        if (i <= ii - 2 && cj && ck)
            U[o + c] = U[o + c] + (d - dp[c + (long long)kk * jj]) * bp[c] * bp[c + (long long)kk * jj] *
                                      RDX[G.ipx + i - 1] * rfak;
        if (ci && j <= jj - 2 && ck)
            V[o + c] = V[o + c] + (d - dp[c + kk]) * bp[c] * bp[c + kk] * RDY[G.ipy + j - 1] * rfak;
        if (ci && cj && k <= kk - 2)
            W[o + c] = W[o + c] + (d - dp[c + 1]) * bp[c] * bp[c + 1] * RDZ[G.ipz + k - 1] * rfak;
        return;
    }
    P[o + c] = P[o + c] + d;
    if (i <= ii - 2 && cj && ck)
        U[o + c] = U[o + c] + (d - dp[c + (long long)kk * jj]) * RDX[G.ipx + i - 1] * rfak;
    if (ci && j <= jj - 2 && ck)
        V[o + c] = V[o + c] + (d - dp[c + kk]) * RDY[G.ipy + j - 1] * rfak;
    if (ci && cj && k <= kk - 2)
        W[o + c] = W[o + c] + (d - dp[c + 1]) * RDZ[G.ipz + k - 1] * rfak;
}

__global__ void k_mx_setprm(double* sprm, int* err, double frhs, double dtfu, double prefak,
                            double rfak) {
    *err = 0;
    sprm[0] = frhs;
    sprm[1] = dtfu;
    sprm[2] = prefak;
    sprm[3] = rfak;
}

__global__ void k_cvt_64_32(float* d, const double* s, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) d[t] = (float)s[t];
}

__global__ void k_cvt_32_64(double* d, const float* s, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) d[t] = (double)s[t];
}

// The reference's inner-iteration halo semantics mapped onto the rotating
// res slots: iteration G (1-based within one mgpoisl) writes slot G%3;
// its forward sweep reads low ghosts written by the last iteration whose
// conn(res) exchanged all faces (inner index < ninner), or zeros.  The
// solve's prefak and dt/rho come from the stage scalars (d_sprm).
int enqueue_mgpoisl(Ctx* c) {
    MixedState* m = c->mx;
    SipState& s = m->sip;
    const LevelState& lv = m->lv;
    const bool multi = c->minlevel != c->maxlevel;
    double *U = c->F("U"), *V = c->F("V"), *W = c->F("W"), *P = c->F("P"), *dp = c->F("DP");
    MG_CUDA(cudaMemsetAsync(s.dph, 0, (size_t)c->ngrid * s.npp * sizeof(float), c->stream));
    MG_CUDA(cudaMemsetAsync(s.dpl, 0, (size_t)c->ngrid * s.npp * sizeof(float), c->stream));
    // converged flag and outer count; the error flag ctl[2] is cleared when
    // the stage (or the solve) starts
    MG_CUDA(cudaMemsetAsync(m->d_ctl, 0, 2 * sizeof(int), c->stream));
    if (int rc = sip_divcal(c, s, m->d_sprm + 2)) return rc;
    int* ctl = m->d_ctl;
    // pressuresolver_mod.F90:196-199: the divergence restricted into the
    // coarse grids, finest level first
    for (int l = c->maxlevel; l > c->minlevel; --l)
        if (int rc = mx_ftoc(c, s, lv, l, true, ctl)) return rc;
    const int ninner = c->prm.ninner;
    // per level: inner iterations run and the last one whose res exchange
    // covered every face (the rotating res slots of each level's grids)
    const int nl = c->maxlevel - c->minlevel + 1;
    std::vector<int> gi(nl, 0), lastfull(nl, 0);
    // one level: the whole outer loop as one persistent launch when the
    // tuner (or the caller) chose it
    const bool persistent = !multi && s.solve_variant >= 0;
    // one level with the packed pre-pass: the outer step writes the pre-pass
    // of the next outer iteration's first inner iteration (hilf = 0)
    const bool fuse = !multi && s.prepk && s.fuse_pre;
    if (persistent)
        if (int rc = sip_solve(c, s, m->cf, m->apx, m->d_gcls, ctl, m->d_maxrhs, m->d_sprm)) return rc;
    for (int ipcount = 1; ipcount <= (persistent ? 0 : c->prm.nouter); ++ipcount) {
        // pressuresolver_mod.F90:218-302: level by level, coarse to fine
        for (int l = c->minlevel; l <= c->maxlevel; ++l) {
            const int li = l - c->minlevel;
            const int* glist = multi ? lv.d_grids[li] : nullptr;
            const int nlist = multi ? (int)lv.grids[li].size() : c->ngrid;
            if (!nlist) continue;
            if (multi && l > c->minlevel)
                if (int rc = mx_ctof(c, s, lv, l, ctl)) return rc;
            for (int iloop = 1; iloop <= ninner; ++iloop) {
                if (multi)
                    if (int rc = mx_bound_pressure(c, s, lv, l, ctl)) return rc;
                ++gi[li];
                // hilf starts at zero on the coarsest level (accumulate_pcorr
                // cleared it); the finer levels start from the ctof values
                const bool hz = iloop == 1 && l == c->minlevel;
                const int rlow = lastfull[li] > 0 ? lastfull[li] % 3 : -1;
                // the outer step before wrote this iteration's pre-pass
                const bool prewritten = fuse && hz && ipcount > 1;
                if (int rc = sip_forward(c, s, m->cf, m->d_gcls, ctl, rlow, gi[li] % 3, hz, glist,
                                         nlist, prewritten))
                    return rc;
                if (int rc = sip_backward(c, s, m->cb, m->d_gcls, ctl, gi[li] % 3, hz, glist, nlist))
                    return rc;
                if (iloop < ninner) lastfull[li] = gi[li];
            }
            if (multi)
                if (int rc = mx_bound_pressure(c, s, lv, l, ctl)) return rc;
        }
        for (int l = c->maxlevel; l > c->minlevel; --l)
            if (int rc = mx_ftoc(c, s, lv, l, false, ctl)) return rc;
        if (int rc = sip_outer(c, s, m->apx, m->d_gcls, ctl,
                               fuse && ipcount < c->prm.nouter ? s.rs[(gi[0] + 1) % 3] : nullptr))
            return rc;
        if (multi) {
            // the residual restricted into the coarse grids, then its maxima again
            for (int l = c->maxlevel; l > c->minlevel; --l)
                if (int rc = mx_ftoc(c, s, lv, l, true, ctl)) return rc;
            if (int rc = mx_gridmax(c, s, ctl)) return rc;
        }
        if (int rc = sip_conv(c, m->d_ctl, m->d_maxrhs, m->d_sprm)) return rc;
    }
    if (int rc = sip_scatter_dp(c, s)) return rc;
    // dp ghosts (the reference accumulates the connected hilf ghosts into dp)
    if (int rc = connect(c, 0, 1, nullptr, nullptr, nullptr, dp, nullptr, nullptr, false, false, 0))
        return rc;
    if (multi) {
        // pressuresolver_mod.F90:319-323: parent and bound_pressure of dp
        static const char* const none[3] = {nullptr, nullptr, nullptr};
        static const char* const sdp[3] = {"DP", nullptr, nullptr};
        double* dbuf = field_buffer(c, "DP");
        for (int l = c->minlevel; l <= c->maxlevel; ++l) {
            if (int rc = launch_parent(c, l, none, sdp, false)) return rc;
            if (int rc = launch_bound_pressure(c, l, dp, dbuf, c->ibtype == 1)) return rc;
        }
    }
    {
        ProfScope ps_(c, "mx_mgpcorr");
        dim3 grid((s.kk * s.jj * s.ii + 255) / 256, c->ngrid);
        k_mx_mgpcorr<<<grid, 256, 0, c->stream>>>(c->d_grids, U, V, W, P, dp, c->L("RDX"),
                                                  c->L("RDY"), c->L("RDZ"), m->d_sprm,
                                                  c->ibtype == 1 ? c->F("BP") : nullptr);
        MG_LAUNCHED(c);
    }
    if (multi) {
        // pressuresolver_mod.F90:334-348: ftoc fine to coarse, then per level
        // parent, bound_flow and the corner connect
        for (int l = c->maxlevel; l >= c->minlevel; --l) {
            if (int rc = launch_ftoc(c, l, U, U, 'U')) return rc;
            if (int rc = launch_ftoc(c, l, V, V, 'V')) return rc;
            if (int rc = launch_ftoc(c, l, W, W, 'W')) return rc;
            if (int rc = launch_ftoc(c, l, P, P, 'P')) return rc;
        }
        static const char* const vuvw[3] = {"U", "V", "W"};
        static const char* const sp[3] = {"P", nullptr, nullptr};
        for (int l = c->minlevel; l <= c->maxlevel; ++l) {
            if (int rc = launch_parent(c, l, vuvw, sp, false)) return rc;
            if (int rc = launch_bound_flow(c, U, V, W, P, l)) return rc;
            if (int rc = connect(c, l, 2, U, V, W, P, nullptr, nullptr, true, false, 0)) return rc;
        }
    } else {
        // pressuresolver_mod.F90:341-348: bound_flow, then the corner connect
        if (m->walls)
            if (int rc = launch_bound_flow(c, U, V, W, P, 0)) return rc;
        if (int rc = connect(c, 0, 2, U, V, W, P, nullptr, nullptr, true, false, 0)) return rc;
    }
    MG_CUDA(cudaMemcpyAsync(m->h_ctl, m->d_ctl, 3 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaMemcpyAsync(m->h_maxrhs, m->d_maxrhs, sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    return 0;
}

// The stage's scalars into d_sprm (a one-thread kernel on the stream, so the
// values are fixed at launch and need no host buffer that outlives the call).
int set_stage_scalars(Ctx* c, double frhs, double dtfu, double dtsolve) {
    k_mx_setprm<<<1, 1, 0, c->stream>>>(c->mx->d_sprm, c->mx->d_ctl + 2, frhs, dtfu,
                                        c->prm.rho / dtsolve, dtsolve / c->prm.rho);
    MG_LAUNCHED(c);
    return 0;
}

// The stage after the fluxes and the RK update: the connects, parent and
// bound_flow of each level, the pressure solve, and the LES model's G for
// the next stage (timeintegration_mod.F90:117-125).
static int enqueue_after_rk(Ctx* c);

int enqueue_stage(Ctx* c) {
    MixedState* m = c->mx;
    const bool skip = m->skip_once;
    m->skip_once = false;
    // ghost-cell IB: which grids' point values differ from U, V, W now (the
    // flux kernel transports their point values PWU, PWV, PWW by U, V, W,
    // timeintegration_mod.F90:100-101)
    if (c->ibtype == 1)
        if (int rc = mx_pw_flags(c, m->lv)) return rc;
    if (int rc = launch_mx_flux(c, m->du32, m->dv32, m->dw32, m->sx, m->sy, m->sz, m->d_sprm,
                                m->d_ctl + 2, skip))
        return rc;
    double *U = c->F("U"), *V = c->F("V"), *W = c->F("W"), *P = c->F("P");
    const bool gc = c->ibtype == 1;
    if (c->minlevel != c->maxlevel)
        // grids with a PAR face: tstle4_par (tstle4_mod.F90:114) on the fluxes
        // left in UO, VO, WO
        if (int rc = launch_tstle4_par(c, c->F("UO"), c->F("VO"), c->F("WO"), gc ? c->F("PWU") : U,
                                       gc ? c->F("PWV") : V, gc ? c->F("PWW") : W, U, V, W))
            return rc;
    // the RK update of the grids with a PAR face (their fluxes in UO, VO, WO)
    if (int rc = mx_rk_par(c, m->lv, m->du32, m->dv32, m->dw32, m->d_sprm)) return rc;
    if (gc) {   // timeintegration_mod.F90:110-116: maskbp, getibvalues
        if (int rc = launch_maskbp(c, U, V, W, P)) return rc;
        if (int rc = launch_gc_mode(c, 'R', U, V, W)) return rc;
    }
    return enqueue_after_rk(c);
}

static int enqueue_after_rk(Ctx* c) {
    MixedState* m = c->mx;
    double *U = c->F("U"), *V = c->F("V"), *W = c->F("W"), *P = c->F("P");
    if (c->minlevel == c->maxlevel) {
        if (int rc = connect(c, 0, 1, U, V, W, nullptr, nullptr, nullptr, false, true, 1)) return rc;
        // timeintegration_mod.F90:117-122: bound_flow after the connect
        if (m->walls)
            if (int rc = launch_bound_flow(c, U, V, W, P, 0)) return rc;
    } else {
        // timeintegration_mod.F90:117-122: per level connect, parent, bound_flow
        static const char* const vn[3] = {"U", "V", "W"};
        static const char* const sn[3] = {"P", nullptr, nullptr};
        for (int l = c->minlevel; l <= c->maxlevel; ++l) {
            if (int rc = connect(c, l, 1, U, V, W, nullptr, nullptr, nullptr, false, true, 1)) return rc;
            if (int rc = launch_parent(c, l, vn, sn, false)) return rc;
            if (int rc = launch_bound_flow(c, U, V, W, P, l)) return rc;
        }
    }
    if (int rc = enqueue_mgpoisl(c)) return rc;
    // timeintegration_mod.F90:125: the LES model's G from the new velocity
    // (FP64, the plain kernels), read by the next stage's fluxes
    return lesmodel(c);
}

// 0, or MGLET_ERR_CUDA when a kernel gave up waiting for its bulk copies or
// at a grid-wide barrier of the persistent solve (the device error flag of
// the control block).
int check_device_flag(Ctx* c) {
    MixedState* m = c->mx;
    if (m->h_ctl[2] != 0) {
        set_error("mixed form: a kernel timed out waiting for its bulk copies or at a grid-wide "
                  "barrier");
        return MGLET_ERR_CUDA;
    }
    return 0;
}

void fill_stats(Ctx* c, double dt, mglet_stage_stats* st) {
    MixedState* m = c->mx;
    st->nouter_done = m->h_ctl[1];
    st->ipc = m->h_ctl[1] * c->prm.ninner;
    st->maxrhs = m->h_maxrhs[0];
    st->prefak = c->prm.rho / dt;
}

float* du_buffer(Ctx* c, const char* name) {
    MixedState* m = c->mx;
    if (!m) return nullptr;
    if (!std::strcmp(name, "DU")) return m->du32;
    if (!std::strcmp(name, "DV")) return m->dv32;
    if (!std::strcmp(name, "DW")) return m->dw32;
    return nullptr;
}

}  // namespace

// Coefficient classes: grids with the same dimensions, boundary types and
// spacing arrays share one set of SIP factors; a grid flagged in own (BP not
// 1 everywhere: ghost-cell IB) keeps a class of its own.  sp: the spacing
// arrays DX, DY, DZ, DDX, DDY, DDZ.
static void class_keys(Ctx* c, const std::vector<std::vector<double>>& sp,
                       const std::vector<unsigned char>& own, std::vector<int>& gcls,
                       std::vector<int>& reps) {
    gcls.assign(c->ngrid, -1);
    reps.clear();
    std::map<std::vector<double>, int> seen;
    for (int g = 0; g < c->ngrid; ++g) {
        const DevGrid& G = c->grids[g];
        std::vector<double> key = {(double)G.kk, (double)G.jj, (double)G.ii};
        for (int f = 0; f < 6; ++f) key.push_back(G.bc[f]);
        const int off[3] = {G.ipx, G.ipy, G.ipz};
        const int len[3] = {G.ii, G.jj, G.kk};
        for (int q = 0; q < 6; ++q)
            key.insert(key.end(), sp[q].begin() + off[q % 3], sp[q].begin() + off[q % 3] + len[q % 3]);
        if (!own.empty() && own[g]) key.push_back(-1.0 - g);
        auto it = seen.find(key);
        if (it == seen.end()) {
            it = seen.emplace(key, (int)reps.size()).first;
            reps.push_back(g);
        }
        gcls[g] = it->second;
    }
}

// The class map to the device and the class coefficients (SIP factors,
// Laplacian records) from the representative grids; replaces earlier ones.
static int extract_classes(Ctx* c, const std::vector<int>& reps) {
    MixedState* m = c->mx;
    m->nclass = (int)reps.size();
    MG_CUDA(copy_on(c->stream, m->d_gcls, m->gcls.data(), c->ngrid * sizeof(int), cudaMemcpyHostToDevice));
    for (float** p : {&m->cf, &m->cb, &m->apx}) {
        cudaFree(*p);
        *p = nullptr;
    }
    int* d_reps = nullptr;
    MG_CUDA(cudaMalloc(&d_reps, reps.size() * sizeof(int)));
    MG_CUDA(copy_on(c->stream, d_reps, reps.data(), reps.size() * sizeof(int), cudaMemcpyHostToDevice));
    int rc = sip_extract(c, m->sip, m->nclass, d_reps, m->d_idx,
                         c->prm.psolver != MGLET_PSOLVER_CLASSIC, &m->cf, &m->cb, &m->apx);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(d_reps);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "mixed classes");
    return 0;
}

int mixed_init(Ctx* c) {
    if (!c->uniform) {
        set_error("mixed form: all grids must have the same dimensions");
        return MGLET_ERR_UNSUPPORTED;
    }
    if (c->prm.ninner < 1) {
        set_error("mixed form: ninner must be at least 1");
        return MGLET_ERR_UNSUPPORTED;
    }
    bool walls = false;
    for (const DevGrid& G : c->grids)
        for (int f = 0; f < 6; ++f) {
            const int t = G.bc[f];
            // tstle4 extends the flux ranges of an outflow face on the low
            // side over the ghost plane (nfu, nrv, nbw), which this form's
            // interior sweep does not visit
            if (t == MGLET_BC_OP1 && f % 2 == 0) {
                set_error("mixed form: OP1 only on the high faces (2, 4, 6)");
                return MGLET_ERR_UNSUPPORTED;
            }
            walls |= t == MGLET_BC_FIX || t == MGLET_BC_OP1 || t == MGLET_BC_NOS ||
                     t == MGLET_BC_SLI;
        }
    MixedState* m = new MixedState();
    c->mx = m;
    m->walls = walls;
    // the ghosts of DP that no exchange writes (faces without a neighbour)
    // must read zero in mgpcorr, as in the reference
    MG_CUDA(cudaMemsetAsync(c->F("DP"), 0, (size_t)c->idim3d * sizeof(double), c->stream));
    if (int rc = sip_init(c, m->sip)) return rc;
    if (int rc = mx_flux_prepare(c)) return rc;
    m->d_idx = c->hp[0].d_idx;
    // coefficient classes: same dims, BC types and spacing arrays
    std::vector<std::vector<double>> sp(6);
    const char* names[6] = {"DX", "DY", "DZ", "DDX", "DDY", "DDZ"};
    const long long lens[3] = {c->idimx, c->idimy, c->idimz};
    for (int q = 0; q < 6; ++q) {
        sp[q].resize(lens[q % 3]);
        MG_CUDA(copy_on(c->stream, sp[q].data(), c->L(names[q]), lens[q % 3] * sizeof(double),
                           cudaMemcpyDeviceToHost));
    }
    std::vector<int> reps;
    class_keys(c, sp, {}, m->gcls, reps);
    m->nclass = (int)reps.size();
    // FP32 spacing tables for the flux kernel
    {
        float** dst[3] = {&m->sx, &m->sy, &m->sz};
        for (int ax = 0; ax < 3; ++ax) {
            const long long n = lens[ax];
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
            MG_CUDA(copy_on(c->stream, *dst[ax], tb.data(), tb.size() * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    for (float** p : {&m->du32, &m->dv32, &m->dw32}) {
        MG_CUDA(cudaMalloc(p, (size_t)c->idim3d * sizeof(float)));
        MG_CUDA(zero_on(c->stream, *p, (size_t)c->idim3d * sizeof(float)));
    }
    MG_CUDA(cudaMalloc(&m->d_gcls, c->ngrid * sizeof(int)));
    MG_CUDA(cudaMalloc(&m->d_ctl, 4 * sizeof(int)));
    MG_CUDA(zero_on(c->stream, m->d_ctl, 4 * sizeof(int)));
    MG_CUDA(cudaMalloc(&m->d_maxrhs, sizeof(double)));
    MG_CUDA(cudaMalloc(&m->d_sprm, 4 * sizeof(double)));
    MG_CUDA(zero_on(c->stream, m->d_sprm, 4 * sizeof(double)));
    MG_CUDA(cudaMallocHost(&m->h_ctl, 4 * sizeof(int)));
    MG_CUDA(cudaMallocHost(&m->h_maxrhs, sizeof(double)));
    // every connect variant the stage issues, built before any graph capture
    const ConnectPlan* pl;
    if (int rc = get_plan(c, 0, 1, 1 << 3, false, false, 0, &pl)) return rc;
    if (int rc = get_plan(c, 0, 1, 7, false, true, 1, &pl)) return rc;
    if (int rc = get_plan(c, 0, 2, 15, true, false, 0, &pl)) return rc;
    // class coefficients from the representative grids
    if (int rc = extract_classes(c, reps)) return rc;
    // launch shapes picked by measurement on this case (MGLET_TUNE=0 keeps
    // the defaults)
    const char* tune = std::getenv("MGLET_TUNE");
    if (!(tune && tune[0] == '0')) {
        if (int rc2 = sip_tune(c, m->sip, m->cf, m->d_gcls, m->d_ctl)) return rc2;
        if (int rc2 = sip_tune_outer(c, m->sip, m->apx, m->d_gcls, m->d_ctl)) return rc2;
        if (int rc2 = sip_tune_solve(c, m->sip, m->cf, m->apx, m->d_gcls, m->d_ctl, m->d_maxrhs,
                                     m->d_sprm))
            return rc2;
        if (int rc2 = mx_flux_tune(c, m->du32, m->dv32, m->dw32, m->sx, m->sy, m->sz, m->d_sprm,
                                   m->d_ctl + 2))
            return rc2;
        MG_CUDA(cudaStreamSynchronize(c->stream));
    }
    return 0;
}

// Text of the launch variants in use ("kernel: variant (ms per launch)").
std::string mixed_tuning(Ctx* c) {
    MixedState* m = c->mx;
    if (!m) return "";
    const SipState& s = m->sip;
    char buf[512];
    std::snprintf(buf, sizeof buf,
                  "mx_sip_pre: %s%s (%.4f ms); uniform classes: %s; sweeps: %s%s (%.4f ms per "
                  "pair); ",
                  sip_pre_variant_name(s.pre_variant >= 0 ? s.pre_variant : 0),
                  s.pre_variant >= 0 ? "" : " [default]", s.pre_ms, s.unicls ? "yes" : "no",
                  sip_sweep_variant_name(s.sweep_variant >= 0 ? s.sweep_variant : 0),
                  s.sweep_variant >= 0 ? "" : " [default]", s.sweep_ms);
    char sbuf[512];
    int n = std::snprintf(sbuf, sizeof sbuf,
                          "mx_sip_solve: %s (fastest persistent: %s, %.4f ms; per-phase kernels "
                          "%.4f ms per outer iteration; variants",
                          sip_solve_variant_name(s.solve_variant),
                          s.solve_best >= 0 ? sip_solve_variant_name(s.solve_best) : "none",
                          s.solve_ms, s.phases_ms);
    for (int v = 0; v < sip_solve_variants() && n > 0 && n < (int)sizeof sbuf; ++v)
        n += std::snprintf(sbuf + n, sizeof sbuf - n, " %d: %.4f", v, s.solve_var_ms[v]);
    if (n > 0 && n < (int)sizeof sbuf) std::snprintf(sbuf + n, sizeof sbuf - n, "); ");
    char obuf[256];
    std::snprintf(obuf, sizeof obuf,
                  "mx_outer: %s%s (staged %.4f ms, direct 3 CTAs/SM %.4f ms, 4 CTAs/SM %.4f ms)%s; ",
                  sip_outer_variant_name(s.outer_variant >= 0 ? s.outer_variant : 0),
                  s.outer_variant >= 0 ? "" : " [default]", s.outer_ms[0], s.outer_ms[1],
                  s.outer_ms[2],
                  s.fuse_pre && s.prepk && c->minlevel == c->maxlevel
                      ? ", writes the next pre-pass from hilf = 0"
                      : "");
    return std::string(buf) + sbuf + obuf + mx_flux_tuning(c);
}

int mixed_test_wait_timeout(Ctx* c) {
    MixedState* m = c->mx;
    if (!m || !mx_flux_has_tma(c)) {
        set_error("test_wait_timeout: needs the mixed form with the TMA flux kernel");
        return MGLET_ERR_UNSUPPORTED;
    }
    m->skip_once = true;
    return 0;
}

int mixed_test_barrier_timeout(Ctx* c) {
    MixedState* m = c->mx;
    if (!m || m->sip.solve_variant < 0) {
        set_error("test_barrier_timeout: needs the mixed form with the persistent solve");
        return MGLET_ERR_UNSUPPORTED;
    }
    m->sip.solve_skip = true;
    return 0;
}

int mixed_force_variant(Ctx* c, const char* kernel, int v) {
    MixedState* m = c->mx;
    if (m && std::strcmp(kernel, "mx_outer") == 0) {
        if (v < -1 || v >= sip_outer_variants()) {
            set_error("force_variant: mx_outer variants are 0 (staged), 1, 2 (direct) or -1");
            return MGLET_ERR_ARG;
        }
        m->sip.outer_variant = v;
        if (m->graph) {
            cudaGraphExecDestroy(m->graph);
            m->graph = nullptr;
        }
        return 0;
    }
    if (m && std::strcmp(kernel, "mx_order") == 0) {
        if (v < -1 || v > 1) {
            set_error("force_variant: mx_order is 1 (divcal and scatter in natural order), 0 (plane "
                      "order) or -1 (default 1)");
            return MGLET_ERR_ARG;
        }
        m->sip.natural = v != 0;
        if (m->graph) {
            cudaGraphExecDestroy(m->graph);
            m->graph = nullptr;
        }
        return 0;
    }
    if (m && std::strcmp(kernel, "mx_outer_pre") == 0) {
        if (v < -1 || v > 1) {
            set_error("force_variant: mx_outer_pre is 1 (the outer step writes the next pre-pass), "
                      "0 (the pre-pass kernel does) or -1 (default 0)");
            return MGLET_ERR_ARG;
        }
        m->sip.fuse_pre = v == 1;
        if (m->graph) {
            cudaGraphExecDestroy(m->graph);
            m->graph = nullptr;
        }
        return 0;
    }
    if (m && std::strcmp(kernel, "mx_sip_solve") == 0) {
        if (v < -1 || v >= sip_solve_variants()) {
            set_error("force_variant: mx_sip_solve variants are 0..5 (-1: the per-phase kernels)");
            return MGLET_ERR_ARG;
        }
        if (v >= 0 && !sip_solve_fits(c, m->sip, v)) {
            set_error("force_variant: this persistent solve variant does not apply to this case");
            return MGLET_ERR_UNSUPPORTED;
        }
        if (v >= 0)
            if (int rc = sip_solve_alloc(m->sip)) return rc;
        m->sip.solve_variant = v;
        if (m->graph) {
            cudaGraphExecDestroy(m->graph);
            m->graph = nullptr;
        }
        return 0;
    }
    if (m && std::strcmp(kernel, "mx_sip_sweep") == 0) {
        if (v < -1 || v >= sip_sweep_variants()) {
            set_error("force_variant: mx_sip_sweep variants are 0..4 (-1 default)");
            return MGLET_ERR_ARG;
        }
        m->sip.sweep_variant = v;
        if (m->graph) {
            cudaGraphExecDestroy(m->graph);
            m->graph = nullptr;
        }
        return 0;
    }
    if (m && std::strcmp(kernel, "mx_flux") == 0) {
        if (int rc = mx_flux_force(c, v)) return rc;
        if (m->graph) {
            cudaGraphExecDestroy(m->graph);
            m->graph = nullptr;
        }
        return 0;
    }
    if (!m || std::strcmp(kernel, "mx_sip_pre") != 0 || v < -1 || v >= sip_pre_variants()) {
        set_error("force_variant: needs the mixed form, kernel mx_sip_pre and a valid variant");
        return MGLET_ERR_ARG;
    }
    if (sip_pre_variant_uniform(v) && !m->sip.unicls) {
        set_error("force_variant: the uniform pre-pass needs classes with constant coefficients");
        return MGLET_ERR_UNSUPPORTED;
    }
    m->sip.pre_variant = v;
    if (m->graph) {          // the captured stage holds the old launch
        cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
    }
    return 0;
}

void mixed_release(Ctx* c) {
    MixedState* m = c->mx;
    if (!m) return;
    if (m->graph) cudaGraphExecDestroy(m->graph);
    mx_flux_release(c);
    mx_level_release(m->lv);
    sip_release(m->sip);
    for (void* p : {(void*)m->cf, (void*)m->cb, (void*)m->apx, (void*)m->d_gcls,
                    (void*)m->d_ctl, (void*)m->d_maxrhs, (void*)m->d_sprm, (void*)m->du32, (void*)m->dv32,
                    (void*)m->dw32, (void*)m->sx, (void*)m->sy, (void*)m->sz})
        cudaFree(p);
    if (m->h_ctl) cudaFreeHost(m->h_ctl);
    if (m->h_maxrhs) cudaFreeHost(m->h_maxrhs);
    delete m;
    c->mx = nullptr;
}

// A field was uploaded: the FP32 RK registers follow DU/DV/DW, and a
// viscosity field that is not the uniform gmol takes the stage off the
// mixed path (LES models are outside this form).
// G becomes a field the fluxes read (an LES model, or a G the caller set):
// the stage graph holds the uniform-viscosity flux launch, so it is dropped.
void mixed_g_field(Ctx* c) {
    MixedState* m = c->mx;
    if (!m) return;
    mx_flux_set_gfield(c);
    if (m->graph) {
        cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
    }
}

void mixed_field_changed(Ctx* c, const char* name) {
    MixedState* m = c->mx;
    if (!m) return;
    if (!std::strcmp(name, "G")) mixed_g_field(c);
    if (float* f = du_buffer(c, name)) {
        k_cvt_64_32<<<(unsigned)((c->idim3d + 255) / 256), 256, 0, c->stream>>>(f, c->F(name), c->idim3d);
        cudaStreamSynchronize(c->stream);
    }
}

// Before a download: DU/DV/DW live in FP32 in this form.
void mixed_field_sync_out(Ctx* c, const char* name) {
    if (float* f = du_buffer(c, name))
        k_cvt_32_64<<<(unsigned)((c->idim3d + 255) / 256), 256, 0, c->stream>>>(c->F(name), f, c->idim3d);
}

// Hierarchies and the ghost-cell IB: the per-level lists and buffers, once
// the parents are known (before the first stage is captured).
static int levels_ready(Ctx* c) {
    MixedState* m = c->mx;
    if ((c->minlevel == c->maxlevel && c->ibtype != 1) || m->lv.ready) return 0;
    return mx_level_prepare(c, m->sip, m->lv);
}

// The ghost-cell IB in the mixed form, after mglet_gpu_set_ghostcell's plain
// set-up (SIP coefficients with BP, the lists on the device, SDIV):
//  * BP must be 0 or 1 (the couplings laplacephi's bp products close become
//    per-point masks); grids where it is not 1 everywhere get classes of their
//    own, whose Laplacian records carry the masks;
//  * at every stage the grids whose point values PWU, PWV, PWW differ from
//    U, V, W anywhere the flux kernel reads (those with lists, and the
//    neighbours and parents whose copies of them differ) are flagged, and
//    the flux kernel transports their point values by U, V, W.
int mixed_ghostcell(Ctx* c) {
    MixedState* m = c->mx;
    SipState& st = m->sip;
    if (!st.prepk) {
        set_error("mixed form: the ghost-cell IB needs the packed pre-pass (smaller grids)");
        return MGLET_ERR_UNSUPPORTED;
    }
    std::vector<double> bp((size_t)c->idim3d);
    MG_CUDA(copy_on(c->stream, bp.data(), c->F("BP"), bp.size() * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<unsigned char> own(c->ngrid, 0);
    for (int g = 0; g < c->ngrid; ++g) {
        const DevGrid& G = c->grids[g];
        const long long n = (long long)G.kk * G.jj * G.ii;
        for (long long t = 0; t < n; ++t) {
            const double v = bp[G.ip3 + t];
            if (v != 0.0 && v != 1.0) {
                set_error("mixed form: the ghost-cell IB needs BP of 0 or 1");
                return MGLET_ERR_UNSUPPORTED;
            }
            if (v != 1.0) own[g] = 1;
        }
    }
    // classes with the BP masks
    if (int rc = sip_bpmask(c, st)) return rc;
    std::vector<std::vector<double>> sp(6);
    const char* names[6] = {"DX", "DY", "DZ", "DDX", "DDY", "DDZ"};
    const long long lens[3] = {c->idimx, c->idimy, c->idimz};
    for (int q = 0; q < 6; ++q) {
        sp[q].resize(lens[q % 3]);
        MG_CUDA(copy_on(c->stream, sp[q].data(), c->L(names[q]), lens[q % 3] * sizeof(double),
                        cudaMemcpyDeviceToHost));
    }
    std::vector<int> reps;
    class_keys(c, sp, own, m->gcls, reps);
    if (int rc = extract_classes(c, reps)) return rc;
    // a uniform-coefficient pre-pass no longer applies: the same launch shape
    // with per-point records
    if (!st.unicls && sip_pre_variant_uniform(st.pre_variant)) st.pre_variant -= 5;
    // the same for the persistent solve (variants 3..5 are the uniform ones)
    if (st.solve_variant >= 0 && !sip_solve_fits(c, st, st.solve_variant))
        st.solve_variant = st.solve_variant >= 3 && sip_solve_fits(c, st, st.solve_variant - 3)
                               ? st.solve_variant - 3
                               : -1;
    // per-stage flags of the grids whose point values differ from U, V, W
    mx_level_release(m->lv);
    m->lv.ibflag.assign(c->ngrid, 1);
    if (int rc = mx_level_prepare(c, st, m->lv)) return rc;
    if (int rc = mx_flux_set_pw(c, m->lv.d_skip)) return rc;
    if (m->graph) {
        cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
    }
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int mixed_mgpoisl(Ctx* c, double dt, mglet_stage_stats* st) {
    if (int rc = levels_ready(c)) return rc;
    // frhs and dt*fu are not read by the solve
    if (int rc = set_stage_scalars(c, 0.0, 0.0, dt)) return rc;
    if (int rc = enqueue_mgpoisl(c)) return rc;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    fill_stats(c, dt, st);
    return check_device_flag(c);
}

// One stage: its scalars go to d_sprm, then the stage graph (captured on the
// first call, the same for every stage and time step size) is replayed; with
// per-kernel profiling enabled the stage is issued eagerly so that every
// launch is bracketed by its events.
int mixed_stage(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk, mglet_stage_stats* st) {
    MixedState* m = c->mx;
    double frhs, fu, dtrk, dtrki;
    if (int rc = rk_coeffs(rk, irk, &frhs, &fu, &dtrk, &dtrki)) return rc;
    if (int rc = levels_ready(c)) return rc;
    const bool gc = c->ibtype == 1;
    // timeintegration_mod.F90:96-99: the ghost-cell values of the step, issued
    // before the stage graph (the flux correction reads a device flag back)
    if (gc && irk == 1)
        if (int rc = gc_setibvalues(c, c->F("U"), c->F("V"), c->F("W"))) return rc;
    if (int rc = set_stage_scalars(c, frhs, dt * fu, dtrk * dt)) return rc;
    if (c->prof || m->skip_once || m->sip.solve_skip) {
        if (int rc = enqueue_stage(c)) return rc;
    } else {
        if (!m->graph) {
            cudaGraph_t g;
            const long long l0 = c->launches;
            MG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_stage(c);
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (rc) return rc;
            if (e != cudaSuccess) return cuda_fail(e, "graph capture");
            cudaGraphExec_t ex;
            e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
            m->graph = ex;
            m->graph_launches = c->launches - l0;
            c->launches = l0;
        }
        MG_CUDA(cudaGraphLaunch(m->graph, c->stream));
        c->launches += m->graph_launches;
    }
    // timeintegration_mod.F90:131-134: setpointvalues after the solve
    if (gc)
        if (int rc = gc_setpointvalues(c, irk == rk->nrk)) return rc;
    if (st) {
        MG_CUDA(cudaStreamSynchronize(c->stream));
        fill_stats(c, dtrk * dt, st);
        return check_device_flag(c);
    }
    return 0;
}

}  // namespace mg
