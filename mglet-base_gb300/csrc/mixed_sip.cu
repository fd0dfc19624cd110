// mixed_sip.cu -- inner SIP iterations of the mixed form in hyperplane layout.
//
// The reference stores its SIP factors in hyperplane ("iacc") order so that
// each wavefront step reads a contiguous run (sip_hyperplane_mod.F90:106-257,
// 450-569).  The mixed form carries that idea through the whole inner
// solve: hilf, res and the FP32 copy of the outer residual live in plane
// order too, so at every wavefront step the active threads of a warp touch
// consecutive addresses.  Halos are pulled instead of copied: each sweep
// writes the six boundary planes of its result into a per-grid face buffer,
// and the next sweep of a neighbour reads its ghost values straight from
// there (no conn kernels).  The lagged-coupling semantics of conn(res) and
// conn(dp) in sip/mgpoisit (pressuresolver_mod.F90:400-465) are kept
// exactly:
//   * the forward sweep of inner iteration G reads its low res ghosts from
//     the forward results of the last iteration whose conn(res) was a full
//     exchange (the last inner iteration only exchanges the high faces,
//     forward=-1), or zero if there was none since mgpoisl started;
//   * the backward sweep reads its high res ghosts from this iteration's
//     forward results;
//   * hilf ghosts are the neighbours' hilf after their last backward sweep;
//     the first inner iteration of an outer iteration starts from hilf = 0.
// res face buffers rotate over three slots, which is enough for those reads.
//
// Column wavefront: one CTA per grid, one thread per (j, i) column; at step
// t the thread is at k = t - (i-3) - (j-3) + 3, on hyperplane i+j+k = t+9.
// res(k-1) and hilf(k-1..k+1) of the own column stay in registers;
// res(j-1), res(i-1) and hilf of the four lateral columns come through
// double-buffered shared memory.
#include <algorithm>
#include <vector>

#include "internal.h"
#include "mixed_sip.h"

namespace mg {
namespace {

struct SipShape {
    int kk, jj, ii, ni, nj, nk, npts, fs;
    const int* tpos;   // [(ni+nj+nk-2)+2][ni]: pos(m0, io, jo) = tpos[m0*ni + io] + jo
};

// face-buffer index of a boundary point on slot f (0: x-low, 1: x-high,
// 2: y-low, 3: y-high, 4: z-low, 5: z-high), 0-based (ko, jo, io)
__device__ __forceinline__ int fidx_x(const SipShape& s, int ko, int jo) { return ko + jo * s.nk; }
__device__ __forceinline__ int fidx_y(const SipShape& s, int ko, int io) { return ko + io * s.nk; }
__device__ __forceinline__ int fidx_z(const SipShape& s, int jo, int io) { return jo + io * s.nj; }

struct FwdArgs {
    SipShape s;
    const int* fnbr;            // [ngrid][6] neighbour grid (0-based) across faces 1..6
    const int* gcls;
    const float *H, *RHS;       // plane order [ngrid][npts]
    float* R;                   // plane order, forward results
    const float* HOUT;          // [ngrid][6][fs]
    const float* RLOW;          // res face buffers to read low ghosts from (or null = 0)
    float* RW;                  // res face buffers to write
    const float *LW, *LS, *LB, *LPR, *AP;   // class coefficients, plane order
    const float *AW, *AE, *AS, *AN, *AB, *AT;   // FP32 1-D coefficients (concatenated)
    const DevGrid* grids;
    const int* conv;
    int hzero;                  // first inner iteration: hilf == 0
};

__global__ void __launch_bounds__(576) k_sip_fwd(FwdArgs a) {
    if (*a.conv) return;
    const SipShape s = a.s;
    const int nj = s.nj, ni = s.ni, nk = s.nk, npts = s.npts, fs = s.fs;
    __shared__ float xr[2][576];
    __shared__ float xkm[2][576], xkp[2][576];
    const int g = blockIdx.x;
    const DevGrid G = a.grids[g];
    const int col = threadIdx.x;
    const bool on = col < ni * nj;
    const int jo = on ? col % nj : 0, io = on ? col / nj : 0;
    const long long base = (long long)g * npts;
    const long long cb = (long long)a.gcls[g] * npts;
    const float *H = a.H + base, *RHS = a.RHS + base;
    float* R = a.R + base;
    const float *lw = a.LW + cb, *ls = a.LS + cb, *lb = a.LB + cb, *lpr = a.LPR + cb, *ap = a.AP + cb;
    const int* fn = a.fnbr + 6 * g;
    // ghost sources: hilf and res of the neighbours' facing boundary planes
    const float* hxm = a.HOUT + ((long long)fn[0] * 6 + 1) * fs;   // -x nbr, its x-high plane
    const float* hxp = a.HOUT + ((long long)fn[1] * 6 + 0) * fs;
    const float* hym = a.HOUT + ((long long)fn[2] * 6 + 3) * fs;
    const float* hyp = a.HOUT + ((long long)fn[3] * 6 + 2) * fs;
    const float* hzm = a.HOUT + ((long long)fn[4] * 6 + 5) * fs;
    const float* hzp = a.HOUT + ((long long)fn[5] * 6 + 4) * fs;
    const float* rxm = a.RLOW ? a.RLOW + ((long long)fn[0] * 6 + 1) * fs : nullptr;
    const float* rym = a.RLOW ? a.RLOW + ((long long)fn[2] * 6 + 3) * fs : nullptr;
    const float* rzm = a.RLOW ? a.RLOW + ((long long)fn[4] * 6 + 5) * fs : nullptr;
    float* rw = a.RW + (long long)g * 6 * fs;
    const int i = io + 3, j = jo + 3;
    const float aw = a.AW[G.ipx + i - 1], ae = a.AE[G.ipx + i - 1];
    const float as = a.AS[G.ipy + j - 1], an = a.AN[G.ipy + j - 1];
    const float* ab = a.AB + G.ipz - 1;   // 1-based k
    const float* at = a.AT + G.ipz - 1;
    const bool hz = a.hzero != 0;
    // own-column hilf window at virtual k: hm = h(k-1), hc = h(k), hp = h(k+1)
    auto hval = [&](int kv) -> float {     // h(kv, j, i) for kv in 2..kk-1 (ghosts from z nbrs)
        if (hz || !on) return 0.f;
        if (kv <= 2) return hzm[fidx_z(s, jo, io)];
        if (kv >= nk + 3) return hzp[fidx_z(s, jo, io)];
        const int ko = kv - 3;
        return H[s.tpos[(io + jo + ko) * ni + io] + jo];
    };
    const int nsteps = ni + nj + nk - 2;
    // own-column window at the virtual k of step 0 (k0 = 3 - io - jo); values
    // for virtual k outside 2..kk-1 are never read by an active neighbour
    const int k0 = 3 - io - jo;
    int kv = k0;
    auto hwin = [&](int kq) { return (on && kq >= 2 && kq <= nk + 3) ? hval(kq) : 0.f; };
    float hm = hwin(kv - 1), hc = hwin(kv), hp = hwin(kv + 1);
    float rprev = 0.f;
    for (int t = 0; t < nsteps; ++t) {
        kv = k0 + t;
        const int buf = t & 1;
        if (on) {
            xkm[buf][col] = hm;
            xkp[buf][col] = hp;
        }
        __syncthreads();
        const bool act = on && kv >= 3 && kv <= nk + 2;
        float r = 0.f;
        if (act) {
            const int ko = kv - 3;
            const int m0 = io + jo + ko;
            const int pc = s.tpos[m0 * ni + io] + jo;
            // lateral hilf: own neighbours in the row / column, ghosts from face buffers
            float hjm, hjp, him, hip;
            if (hz) {
                hjm = hjp = him = hip = 0.f;
            } else {
                hjm = jo > 0 ? xkm[buf][col - 1] : hym[fidx_y(s, ko, io)];
                hjp = jo < nj - 1 ? xkp[buf][col + 1] : hyp[fidx_y(s, ko, io)];
                him = io > 0 ? xkm[buf][col - nj] : hxm[fidx_x(s, ko, jo)];
                hip = io < ni - 1 ? xkp[buf][col + nj] : hxp[fidx_x(s, ko, jo)];
            }
            const float lap = -aw * him - ae * hip - as * hjm - an * hjp - ab[kv] * hm -
                              at[kv] * hp - ap[pc] * hc;
            const float rkm = ko > 0 ? rprev : (rzm ? rzm[fidx_z(s, jo, io)] : 0.f);
            const float rjm = jo > 0 ? xr[buf ^ 1][col - 1] : (rym ? rym[fidx_y(s, ko, io)] : 0.f);
            const float rim = io > 0 ? xr[buf ^ 1][col - nj] : (rxm ? rxm[fidx_x(s, ko, jo)] : 0.f);
            r = (RHS[pc] + lap) * lpr[pc];
            r = r - lb[pc] * rkm - ls[pc] * rjm - lw[pc] * rim;
            R[pc] = r;
            // boundary planes for the neighbours
            if (io == 0) rw[0 * fs + fidx_x(s, ko, jo)] = r;
            if (io == ni - 1) rw[1 * fs + fidx_x(s, ko, jo)] = r;
            if (jo == 0) rw[2 * fs + fidx_y(s, ko, io)] = r;
            if (jo == nj - 1) rw[3 * fs + fidx_y(s, ko, io)] = r;
            if (ko == 0) rw[4 * fs + fidx_z(s, jo, io)] = r;
            if (ko == nk - 1) rw[5 * fs + fidx_z(s, jo, io)] = r;
            rprev = r;
            xr[buf][col] = r;
        }
        // slide the own-column hilf window to virtual k + 1
        hm = hc;
        hc = hp;
        const int kn = kv + 2;
        hp = hwin(kn);
    }
}

struct BwdArgs {
    SipShape s;
    const int* fnbr;
    const int* gcls;
    float* H;                   // plane order, updated: h += res
    float* HOUT;                // [ngrid][6][fs], written
    const float* R;             // forward results, plane order
    const float* RHI;           // res face buffers of this iteration (high ghosts)
    const float *UE, *UN, *UT;
    const int* conv;
    int hzero;                  // first inner iteration: old hilf == 0
};

__global__ void __launch_bounds__(576) k_sip_bwd(BwdArgs a) {
    if (*a.conv) return;
    const SipShape s = a.s;
    const int nj = s.nj, ni = s.ni, nk = s.nk, npts = s.npts, fs = s.fs;
    __shared__ float xr[2][576];
    const int g = blockIdx.x;
    const int col = threadIdx.x;
    const bool on = col < ni * nj;
    const int jo = on ? col % nj : 0, io = on ? col / nj : 0;
    const int jr = nj - 1 - jo, ir = ni - 1 - io;
    const long long base = (long long)g * npts;
    const long long cb = (long long)a.gcls[g] * npts;
    float* H = a.H + base;
    const float* R = a.R + base;
    const float *ue = a.UE + cb, *un = a.UN + cb, *ut = a.UT + cb;
    const int* fn = a.fnbr + 6 * g;
    const float* rxp = a.RHI + ((long long)fn[1] * 6 + 0) * fs;   // +x nbr, its x-low plane
    const float* ryp = a.RHI + ((long long)fn[3] * 6 + 2) * fs;
    const float* rzp = a.RHI + ((long long)fn[5] * 6 + 4) * fs;
    float* hw = a.HOUT + (long long)g * 6 * fs;
    const int nsteps = ni + nj + nk - 2;
    float rprev = 0.f;
    for (int t = 0; t < nsteps; ++t) {
        const int kr = t - ir - jr;
        const int buf = t & 1;
        if (on && kr >= 0 && kr < nk) {
            const int ko = nk - 1 - kr;
            const int pc = s.tpos[(io + jo + ko) * ni + io] + jo;
            const float rkp = kr > 0 ? rprev : rzp[fidx_z(s, jo, io)];
            const float rjp = jo < nj - 1 ? xr[buf ^ 1][col + 1] : ryp[fidx_y(s, ko, io)];
            const float rip = io < ni - 1 ? xr[buf ^ 1][col + nj] : rxp[fidx_x(s, ko, jo)];
            const float r = R[pc] - ut[pc] * rkp - un[pc] * rjp - ue[pc] * rip;
            const float h = (a.hzero ? 0.f : H[pc]) + r;
            H[pc] = h;
            if (io == 0) hw[0 * fs + fidx_x(s, ko, jo)] = h;
            if (io == ni - 1) hw[1 * fs + fidx_x(s, ko, jo)] = h;
            if (jo == 0) hw[2 * fs + fidx_y(s, ko, io)] = h;
            if (jo == nj - 1) hw[3 * fs + fidx_y(s, ko, io)] = h;
            if (ko == 0) hw[4 * fs + fidx_z(s, jo, io)] = h;
            if (ko == nk - 1) hw[5 * fs + fidx_z(s, jo, io)] = h;
            rprev = r;
            xr[buf][col] = r;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ double block_max2(double v, double* sh) {
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

struct OuterArgs {
    SipShape s;
    const int* fnbr;
    const int* gcls;
    const int* idx;             // plane position -> natural local index
    const float* H;
    const float* HOUT;
    double* RHS64;              // plane order
    float* RHS32;
    double* DP64;               // plane order
    const double* AP64;         // class, plane order
    const double *AW, *AE, *AS, *AN, *AB, *AT;
    const DevGrid* grids;
    double* gridmax;
    const int* conv;
};

// Outer step in FP64 (laplacephi + rescal + maxabscal_grid + accumulate_pcorr).
__global__ void __launch_bounds__(512) k_sip_outer(OuterArgs a) {
    if (*a.conv) return;
    __shared__ double sh[32];
    const SipShape s = a.s;
    const int kk = s.kk, jj = s.jj, nj = s.nj, ni = s.ni, nk = s.nk, fs = s.fs;
    const int g = blockIdx.x;
    const DevGrid G = a.grids[g];
    const long long base = (long long)g * s.npts;
    const long long cb = (long long)a.gcls[g] * s.npts;
    const float* H = a.H + base;
    const int* fn = a.fnbr + 6 * g;
    const float* hxm = a.HOUT + ((long long)fn[0] * 6 + 1) * fs;
    const float* hxp = a.HOUT + ((long long)fn[1] * 6 + 0) * fs;
    const float* hym = a.HOUT + ((long long)fn[2] * 6 + 3) * fs;
    const float* hyp = a.HOUT + ((long long)fn[3] * 6 + 2) * fs;
    const float* hzm = a.HOUT + ((long long)fn[4] * 6 + 5) * fs;
    const float* hzp = a.HOUT + ((long long)fn[5] * 6 + 4) * fs;
    auto pos = [&](int ko, int jo, int io) { return s.tpos[(io + jo + ko) * ni + io] + jo; };
    double mx = 0.0;
    for (int q = threadIdx.x; q < s.npts; q += blockDim.x) {
        const int id = a.idx[q];
        const int k = id % kk + 1, j = (id / kk) % jj + 1, i = id / (kk * jj) + 1;
        const int ko = k - 3, jo = j - 3, io = i - 3;
        const double hc = H[q];
        const double him = io > 0 ? H[pos(ko, jo, io - 1)] : hxm[fidx_x(s, ko, jo)];
        const double hip = io < ni - 1 ? H[pos(ko, jo, io + 1)] : hxp[fidx_x(s, ko, jo)];
        const double hjm = jo > 0 ? H[pos(ko, jo - 1, io)] : hym[fidx_y(s, ko, io)];
        const double hjp = jo < nj - 1 ? H[pos(ko, jo + 1, io)] : hyp[fidx_y(s, ko, io)];
        const double hkm = ko > 0 ? H[pos(ko - 1, jo, io)] : hzm[fidx_z(s, jo, io)];
        const double hkp = ko < nk - 1 ? H[pos(ko + 1, jo, io)] : hzp[fidx_z(s, jo, io)];
        const double lap = -a.AW[G.ipx + i - 1] * him - a.AE[G.ipx + i - 1] * hip -
                           a.AS[G.ipy + j - 1] * hjm - a.AN[G.ipy + j - 1] * hjp -
                           a.AB[G.ipz + k - 1] * hkm - a.AT[G.ipz + k - 1] * hkp -
                           a.AP64[cb + q] * hc;
        const double r = a.RHS64[base + q] + lap;
        a.RHS64[base + q] = r;
        a.RHS32[base + q] = (float)r;
        a.DP64[base + q] = a.DP64[base + q] + hc;
        mx = fmax(fabs(r), mx);
    }
    mx = block_max2(mx, sh);
    if (threadIdx.x == 0) a.gridmax[g] = mx;
}

// divcal into the plane-ordered FP64/FP32 residual (noib_mod.F90:304-354)
__global__ void k_sip_divcal(const DevGrid* __restrict__ grids, int npts, const int* __restrict__ idx,
                             double* __restrict__ RHS64, float* __restrict__ RHS32,
                             const double* __restrict__ U, const double* __restrict__ V,
                             const double* __restrict__ W, const double* __restrict__ RDDX,
                             const double* __restrict__ RDDY, const double* __restrict__ RDDZ,
                             double fak) {
    const int g = blockIdx.y;
    const DevGrid G = grids[g];
    const int kk = G.kk, jj = G.jj;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    const int id = idx[q];
    const int k = id % kk + 1, j = (id / kk) % jj + 1, i = id / (kk * jj) + 1;
    const double *u = U + G.ip3, *v = V + G.ip3, *w = W + G.ip3;
    const double d = fak * ((u[id] - u[id - kk * jj]) * RDDX[G.ipx + i - 1] +
                            (v[id] - v[id - kk]) * RDDY[G.ipy + j - 1] +
                            (w[id] - w[id - 1]) * RDDZ[G.ipz + k - 1]);
    RHS64[(long long)g * npts + q] = d;
    RHS32[(long long)g * npts + q] = (float)d;
}

// dp (plane order) -> DP field (natural layout, interior)
__global__ void k_sip_scatter(const DevGrid* __restrict__ grids, int npts, const int* __restrict__ idx,
                              const double* __restrict__ DP64, double* __restrict__ DP) {
    const int g = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    DP[grids[g].ip3 + idx[q]] = DP64[(long long)g * npts + q];
}

}  // namespace

int sip_init(Ctx* c, SipState& st) {
    const DevGrid& G0 = c->grids[0];
    st.kk = G0.kk; st.jj = G0.jj; st.ii = G0.ii;
    st.nk = G0.kk - 4; st.nj = G0.jj - 4; st.ni = G0.ii - 4;
    st.npts = st.ni * st.nj * st.nk;
    st.fs = std::max(st.nj * st.nk, std::max(st.ni * st.nk, st.ni * st.nj));
    if (st.ni * st.nj > 576) {
        set_error("mixed form: at most 576 (j, i) columns per grid");
        return MGLET_ERR_UNSUPPORTED;
    }
    // plane positions: pos(m0, io, jo) = tpos[m0*ni + io] + jo
    const int nm = st.ni + st.nj + st.nk - 2;
    std::vector<int> tpos((size_t)(nm + 1) * st.ni, 0);
    int p = 0;
    for (int m0 = 0; m0 < nm; ++m0)
        for (int io = 0; io < st.ni; ++io) {
            const int jlo = std::max(0, m0 - io - (st.nk - 1));
            const int jhi = std::min(st.nj - 1, m0 - io);
            tpos[(size_t)m0 * st.ni + io] = p - jlo;
            if (jhi >= jlo) p += jhi - jlo + 1;
        }
    if (p != st.npts) {
        set_error("mixed form: hyperplane position table does not cover the grid");
        return MGLET_ERR_ARG;
    }
    MG_CUDA(cudaMalloc(&st.d_tpos, tpos.size() * sizeof(int)));
    MG_CUDA(cudaMemcpy(st.d_tpos, tpos.data(), tpos.size() * sizeof(int), cudaMemcpyHostToDevice));
    // face neighbours from the connection table (regular periodic tiling)
    std::vector<int> fn((size_t)6 * c->ngrid, -1);
    for (size_t r = 0; r < c->conns.size(); r += 4) {
        const int rg = c->conns[r], sg = c->conns[r + 1], rf = c->conns[r + 2], sf = c->conns[r + 3];
        if (rf > 6) continue;
        const int opp = rf % 2 ? rf + 1 : rf - 1;
        if (sf != opp) {
            set_error("mixed form: face connections must join opposite faces");
            return MGLET_ERR_UNSUPPORTED;
        }
        fn[(size_t)6 * (rg - 1) + rf - 1] = sg - 1;
    }
    for (int v : fn)
        if (v < 0) {
            set_error("mixed form: every face needs a CON neighbour");
            return MGLET_ERR_UNSUPPORTED;
        }
    MG_CUDA(cudaMalloc(&st.d_fnbr, fn.size() * sizeof(int)));
    MG_CUDA(cudaMemcpy(st.d_fnbr, fn.data(), fn.size() * sizeof(int), cudaMemcpyHostToDevice));
    const size_t n = (size_t)c->ngrid * st.npts;
    for (float** q : {&st.h32, &st.r32, &st.rhs32}) {
        MG_CUDA(cudaMalloc(q, n * sizeof(float)));
        MG_CUDA(cudaMemset(*q, 0, n * sizeof(float)));
    }
    for (double** q : {&st.rhs64, &st.dp64}) {
        MG_CUDA(cudaMalloc(q, n * sizeof(double)));
        MG_CUDA(cudaMemset(*q, 0, n * sizeof(double)));
    }
    const size_t nf = (size_t)c->ngrid * 6 * st.fs;
    MG_CUDA(cudaMalloc(&st.hout, nf * sizeof(float)));
    MG_CUDA(cudaMemset(st.hout, 0, nf * sizeof(float)));
    for (int b = 0; b < 3; ++b) {
        MG_CUDA(cudaMalloc(&st.rout[b], nf * sizeof(float)));
        MG_CUDA(cudaMemset(st.rout[b], 0, nf * sizeof(float)));
    }
    // FP32 copies of the 1-D Poisson coefficients
    const char* n1[6] = {"GSAW", "GSAE", "GSAS", "GSAN", "GSAB", "GSAT"};
    const long long len[6] = {c->idimx, c->idimx, c->idimy, c->idimy, c->idimz, c->idimz};
    for (int q = 0; q < 6; ++q) {
        std::vector<double> h(len[q]);
        MG_CUDA(cudaMemcpy(h.data(), c->L(n1[q]), len[q] * sizeof(double), cudaMemcpyDeviceToHost));
        std::vector<float> f(h.begin(), h.end());
        MG_CUDA(cudaMalloc(&st.a1[q], len[q] * sizeof(float)));
        MG_CUDA(cudaMemcpy(st.a1[q], f.data(), len[q] * sizeof(float), cudaMemcpyHostToDevice));
    }
    return 0;
}

void sip_release(SipState& st) {
    for (void* p : {(void*)st.d_tpos, (void*)st.d_fnbr, (void*)st.h32, (void*)st.r32,
                    (void*)st.rhs32, (void*)st.rhs64, (void*)st.dp64, (void*)st.hout,
                    (void*)st.rout[0], (void*)st.rout[1], (void*)st.rout[2], (void*)st.a1[0],
                    (void*)st.a1[1], (void*)st.a1[2], (void*)st.a1[3], (void*)st.a1[4],
                    (void*)st.a1[5]})
        cudaFree(p);
}

static SipShape shape(const SipState& st) {
    SipShape s;
    s.kk = st.kk; s.jj = st.jj; s.ii = st.ii; s.ni = st.ni; s.nj = st.nj; s.nk = st.nk;
    s.npts = st.npts; s.fs = st.fs; s.tpos = st.d_tpos;
    return s;
}

int sip_divcal(Ctx* c, SipState& st, const int* idx, double fak) {
    ProfScope ps_(c, "mx_divcal");
    dim3 grid((st.npts + 255) / 256, c->ngrid);
    k_sip_divcal<<<grid, 256, 0, c->stream>>>(c->d_grids, st.npts, idx, st.rhs64, st.rhs32,
                                              c->F("U"), c->F("V"), c->F("W"), c->L("RDDX"),
                                              c->L("RDDY"), c->L("RDDZ"), fak);
    MG_LAUNCHED(c);
    return 0;
}

int sip_forward(Ctx* c, SipState& st, const SipCoef& cf, const int* gcls, const int* conv,
                int rlow, int rwrite, bool hzero) {
    ProfScope ps_(c, "mx_sip_fwd");
    FwdArgs a;
    a.s = shape(st);
    a.fnbr = st.d_fnbr; a.gcls = gcls;
    a.H = st.h32; a.RHS = st.rhs32; a.R = st.r32;
    a.HOUT = st.hout;
    a.RLOW = rlow >= 0 ? st.rout[rlow] : nullptr;
    a.RW = st.rout[rwrite];
    a.LW = cf.lw; a.LS = cf.ls; a.LB = cf.lb; a.LPR = cf.lpr; a.AP = cf.ap;
    a.AW = st.a1[0]; a.AE = st.a1[1]; a.AS = st.a1[2]; a.AN = st.a1[3]; a.AB = st.a1[4];
    a.AT = st.a1[5];
    a.grids = c->d_grids;
    a.conv = conv;
    a.hzero = hzero ? 1 : 0;
    const int threads = (st.ni * st.nj + 31) / 32 * 32;
    k_sip_fwd<<<c->ngrid, threads, 0, c->stream>>>(a);
    MG_LAUNCHED(c);
    return 0;
}

int sip_backward(Ctx* c, SipState& st, const SipCoef& cf, const int* gcls, const int* conv,
                 int rhi, bool hzero) {
    ProfScope ps_(c, "mx_sip_bwd");
    BwdArgs a;
    a.s = shape(st);
    a.fnbr = st.d_fnbr; a.gcls = gcls;
    a.H = st.h32; a.HOUT = st.hout; a.R = st.r32; a.RHI = st.rout[rhi];
    a.UE = cf.ue; a.UN = cf.un; a.UT = cf.ut;
    a.conv = conv;
    a.hzero = hzero ? 1 : 0;
    const int threads = (st.ni * st.nj + 31) / 32 * 32;
    k_sip_bwd<<<c->ngrid, threads, 0, c->stream>>>(a);
    MG_LAUNCHED(c);
    return 0;
}

int sip_outer(Ctx* c, SipState& st, const int* idx, const double* ap64, const int* gcls,
              const int* conv) {
    ProfScope ps_(c, "mx_outer");
    OuterArgs a;
    a.s = shape(st);
    a.fnbr = st.d_fnbr; a.gcls = gcls; a.idx = idx;
    a.H = st.h32; a.HOUT = st.hout;
    a.RHS64 = st.rhs64; a.RHS32 = st.rhs32; a.DP64 = st.dp64; a.AP64 = ap64;
    a.AW = c->L("GSAW"); a.AE = c->L("GSAE"); a.AS = c->L("GSAS"); a.AN = c->L("GSAN");
    a.AB = c->L("GSAB"); a.AT = c->L("GSAT");
    a.grids = c->d_grids;
    a.gridmax = c->d_gridred;
    a.conv = conv;
    k_sip_outer<<<c->ngrid, 512, 0, c->stream>>>(a);
    MG_LAUNCHED(c);
    return 0;
}

int sip_scatter_dp(Ctx* c, SipState& st, const int* idx) {
    ProfScope ps_(c, "mx_scatter");
    dim3 grid((st.npts + 255) / 256, c->ngrid);
    k_sip_scatter<<<grid, 256, 0, c->stream>>>(c->d_grids, st.npts, idx, st.dp64, c->F("DP"));
    MG_LAUNCHED(c);
    return 0;
}

}  // namespace mg
