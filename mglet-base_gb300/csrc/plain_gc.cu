// plain_gc.cu -- ghost-cell immersed boundary runtime, FP64.
//
// The stencil lists come from the caller in the formats the reference reads
// (gc_flowstencils_mod.F90:37-100).  The reference walks each list in order,
// updating in place: a ghost value may feed a later stencil of the same list
// (wmxpolsol, :963-1005) and the flux correction updates faces shared by
// neighbouring cut cells (wmxpolsolcorr, :1113-1183).  At upload every list
// is cut into dependency levels (a cell goes after every earlier cell that
// writes a value it reads or writes, or reads a value it writes); one CTA
// per list runs the levels in order, the cells of a level in parallel, so
// every cell sees exactly the values of the ordered walk.  maskbp
// (timeintegration_mod.F90:255-303) is elementwise.  Compiled without FMA
// contraction.
#include <algorithm>
#include <unordered_map>
#include <vector>

#include "internal.h"
#include "mixed.h"

namespace mg {
namespace {

// modes F / X: var(intcell) = sum var(stcell) coeff + const
// One CTA per (grid, component) list.
__global__ void k_gc_sol(const DevGrid* __restrict__ grids, GcDev d, double* U, double* V,
                         double* W, int ngrid, int vel, int ilevel) {
    const int g = blockIdx.x / 3, cmp = blockIdx.x % 3;
    if (ilevel && grids[g].level != ilevel) return;
    const GcSeg s = d.seg[4 * g + cmp];
    if (s.n == 0) return;
    double* var = (cmp == 0 ? U : (cmp == 1 ? V : W)) + grids[g].ip3;
    const long long* xi = d.xpoli + s.xi;
    const double* xr = (vel ? d.xpolrvel : d.xpolr) + s.xr;
    for (int L = 0; L < s.nlv; ++L) {
        const int a = d.lvstart[s.lv0 + L], b = d.lvstart[s.lv0 + L + 1];
        for (int e = a + threadIdx.x; e < b; e += blockDim.x) {
            const int4 cr = d.cell[s.cell0 + e];
            long long pi = cr.x, pr = cr.y;
            const long long intcell = xi[pi++];
            const long long n = xi[pi++];
            double flux = 0.0;
            for (long long q = 0; q < n; ++q) {
                const long long st = xi[pi++];
                flux = flux + var[st - 1] * xr[pr++];
            }
            flux = flux + xr[pr++];
            var[intcell - 1] = flux;
        }
        __syncthreads();
    }
}

// modes S / Z (save) and R / Y (restore)
// One CTA per (grid, component) list; a restore writes in the levels of the
// list (a position written twice keeps the later cell's value).
__global__ void k_gc_savrst(const DevGrid* __restrict__ grids, GcDev d, double* U, double* V,
                            double* W, int ngrid, int vel, int save, int ilevel) {
    const int g = blockIdx.x / 3, cmp = blockIdx.x % 3;
    if (ilevel && grids[g].level != ilevel) return;
    const GcSeg s = d.seg[4 * g + cmp];
    if (s.n == 0) return;
    double* var = (cmp == 0 ? U : (cmp == 1 ? V : W)) + grids[g].ip3;
    double* old = (vel ? d.oldsolvel : d.oldsol) + s.sv;
    long long* pold = (vel ? d.poldsolvel : d.poldsol) + s.sv;
    const long long* xi = d.xpoli + s.xi;
    for (int L = 0; L < s.nlv; ++L) {
        const int a = d.lvstart[s.lv0 + L], b = d.lvstart[s.lv0 + L + 1];
        for (int e = a + threadIdx.x; e < b; e += blockDim.x) {
            const int4 cr = d.cell[s.cell0 + e];
            const int q = cr.z;
            if (save) {
                const long long idx = xi[cr.x];
                pold[q] = idx;
                old[q] = var[idx - 1];
            } else {
                var[pold[q] - 1] = old[q];
            }
        }
        __syncthreads();
    }
}

// mode C: wmxpolsolcorr, one CTA per grid
__global__ void k_gc_corr(const DevGrid* __restrict__ grids, GcDev d, double* U, double* V,
                          double* W, const double* __restrict__ DDX, const double* __restrict__ DDY,
                          const double* __restrict__ DDZ, int ngrid, int* err, int ilevel) {
    const int g = blockIdx.x;
    const DevGrid G = grids[g];
    if (ilevel && G.level != ilevel) return;
    const GcSeg s = d.seg[4 * g + 3];
    if (s.n == 0) return;
    double *u = U + G.ip3, *v = V + G.ip3, *w = W + G.ip3;
    const double *ddx = DDX + G.ipx - 1, *ddy = DDY + G.ipy - 1, *ddz = DDZ + G.ipz - 1;
    const long long ishift = (long long)G.jj * G.kk, jshift = G.kk, kshift = 1;
    const long long* fi = d.xpoli + s.xi;
    const double* fr = d.xpolr + s.xr;
    // a cut cell without open area stops the reference's walk: the cells of
    // later levels are skipped too
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int L = 0; L < s.nlv && !bad; ++L) {
      const int a = d.lvstart[s.lv0 + L], b = d.lvstart[s.lv0 + L + 1];
      for (int e = a + threadIdx.x; e < b; e += blockDim.x) {
        const int4 cr = d.cell[s.cell0 + e];
        long long pi = cr.x, pr = cr.y;
        pi++;   // foundnr
        const long long c0 = fi[pi++] - 1;
        const double ax1 = fr[pr++], ax2 = fr[pr++], ay1 = fr[pr++];
        const double ay2 = fr[pr++], az1 = fr[pr++], az2 = fr[pr++];
        const double acoeffstc = fr[pr++];
        const int k = (int)(c0 % G.kk) + 1, j = (int)((c0 / G.kk) % G.jj) + 1;
        const int i = (int)(c0 / ((long long)G.kk * G.jj)) + 1;
        double div = ddy[j] * ddz[k] * (u[c0] - u[c0 - ishift]) +
                     ddx[i] * ddz[k] * (v[c0] - v[c0 - jshift]) +
                     ddx[i] * ddy[j] * (w[c0] - w[c0 - kshift]) + acoeffstc;
        const double sarea = ax1 + ax2 + ay1 + ay2 + az1 + az2;
        if (sarea < 2.2250738585072014e-308) {   // TINY(1.0_realk): errr in the reference
            atomicExch(err, 1);
            bad = 1;
            continue;
        }
        div = div / sarea;
        u[c0] = u[c0] - ax1 * div / (ddy[j] * ddz[k]);
        u[c0 - ishift] = u[c0 - ishift] + ax2 * div / (ddy[j] * ddz[k]);
        v[c0] = v[c0] - ay1 * div / (ddx[i] * ddz[k]);
        v[c0 - jshift] = v[c0 - jshift] + ay2 * div / (ddx[i] * ddz[k]);
        w[c0] = w[c0] - az1 * div / (ddx[i] * ddy[j]);
        w[c0 - kshift] = w[c0 - kshift] + az2 * div / (ddx[i] * ddy[j]);
      }
      __syncthreads();
    }
}

// setsdivfield_grid / getsdivfield_grid (:1538-1604), one thread per grid
__global__ void k_gc_sdiv(const DevGrid* __restrict__ grids, GcDev d, double* SDIV,
                          const double* __restrict__ DDX, const double* __restrict__ DDY,
                          const double* __restrict__ DDZ, int ngrid, int put) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngrid) return;
    const DevGrid G = grids[g];
    const GcSeg s = d.seg[4 * g + 3];
    const double *ddx = DDX + G.ipx - 1, *ddy = DDY + G.ipy - 1, *ddz = DDZ + G.ipz - 1;
    const long long* fi = d.xpoli + s.xi;
    double* fr = d.xpolr + s.xr;
    double* sdiv = SDIV + G.ip3;
    long long pi = 0, pr = 0;
    for (int cell = 0; cell < s.n; ++cell) {
        pi++;
        const long long c0 = fi[pi++] - 1;
        pr += 6;
        const int k = (int)(c0 % G.kk) + 1, j = (int)((c0 / G.kk) % G.jj) + 1;
        const int i = (int)(c0 / ((long long)G.kk * G.jj)) + 1;
        if (put) sdiv[c0] = fr[pr] / (ddx[i] * ddy[j] * ddz[k]);
        else fr[pr] = sdiv[c0] * ddx[i] * ddy[j] * ddz[k];
        pr++;
    }
}

// maskbp_grid: u *= bp bp(i+1), v *= bp bp(j+1), w *= bp bp(k+1), p *= bp
// over 1..n-1 in every direction
__global__ void k_maskbp(const DevGrid* __restrict__ grids, double* U, double* V, double* W,
                         double* P, const double* __restrict__ BP) {
    const DevGrid G = grids[blockIdx.y];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kk * jj * ii) return;
    const int k = t % kk + 1, j = (t / kk) % jj + 1, i = t / (kk * jj) + 1;
    if (k > kk - 1 || j > jj - 1 || i > ii - 1) return;
    const long long o = G.ip3 + t;
    const double* bp = BP + G.ip3;
    const double b = bp[t];
    U[o] = U[o] * b * bp[t + (long long)kk * jj];
    V[o] = V[o] * b * bp[t + kk];
    W[o] = W[o] * b * bp[t + 1];
    P[o] = P[o] * b;
}

}  // namespace

int gc_upload(Ctx* c) {
    std::vector<GcSeg> seg(4 * (size_t)c->ngrid);
    std::vector<long long> xi;
    std::vector<double> xr, xv;
    long long sv = 0;
    for (int g = 0; g < c->ngrid; ++g) {
        const GcHostList& L = c->gch[g];
        for (int q = 0; q < 4; ++q) {
            GcSeg& s = seg[4 * g + q];
            s.xi = (long long)xi.size();
            s.xr = (long long)xr.size();
            s.sv = sv;
            s.n = L.n[q];
            xi.insert(xi.end(), L.xi[q].begin(), L.xi[q].end());
            xr.insert(xr.end(), L.xr[q].begin(), L.xr[q].end());
            if (q < 3) {
                xv.insert(xv.end(), L.xv[q].begin(), L.xv[q].end());
                sv += L.n[q];
            } else {
                xv.resize(xr.size(), 0.0);   // keep xpolrvel aligned with xpolr
            }
        }
    }
    // dependency levels of every list (see the file comment): a cell goes one
    // level after the last earlier cell that wrote a value it reads or
    // writes, or read a value it writes; within a level the list's order
    std::vector<int4> cells;
    std::vector<int> lvstart;
    for (int g = 0; g < c->ngrid; ++g) {
        const GcHostList& L = c->gch[g];
        const DevGrid& G = c->grids[g];
        const long long box = (long long)G.kk * G.jj * G.ii;
        for (int q = 0; q < 4; ++q) {
            GcSeg& sg = seg[4 * g + q];
            const int n = L.n[q];
            std::vector<int> lev(n, 0);
            std::vector<int4> rec(n);
            std::unordered_map<long long, int> lastw, maxr;
            const std::vector<long long>& x = L.xi[q];
            long long pi = 0, pr = 0;
            int nlv = 0;
            for (int cell = 0; cell < n; ++cell) {
                rec[cell] = make_int4((int)pi, (int)pr, cell, 0);
                int lv = 0;
                auto after_write = [&](long long loc) {
                    auto it = lastw.find(loc);
                    if (it != lastw.end()) lv = std::max(lv, it->second + 1);
                };
                auto after_read = [&](long long loc) {
                    auto it = maxr.find(loc);
                    if (it != maxr.end()) lv = std::max(lv, it->second + 1);
                };
                if (q < 3) {
                    const long long w = x[pi], m = x[pi + 1];
                    for (long long t = 0; t < m; ++t) after_write(x[pi + 2 + t]);
                    after_read(w);
                    after_write(w);
                    lastw[w] = lv;
                    for (long long t = 0; t < m; ++t) {
                        int& r = maxr[x[pi + 2 + t]];
                        r = std::max(r, lv);
                    }
                    pi += 2 + m;
                    pr += m + 1;
                } else {
                    // the six faces of wmxpolsolcorr, read and written
                    const long long c0 = x[pi + 1] - 1;
                    const long long loc[6] = {c0, c0 - (long long)G.kk * G.jj, box + c0, box + c0 - G.kk,
                                              2 * box + c0, 2 * box + c0 - 1};
                    for (long long l : loc) after_write(l);
                    for (long long l : loc) lastw[l] = lv;
                    pi += 2;
                    pr += 7;
                }
                lev[cell] = lv;
                nlv = std::max(nlv, lv + 1);
            }
            sg.cell0 = (int)cells.size();
            sg.lv0 = (int)lvstart.size();
            sg.nlv = n ? nlv : 0;
            std::vector<int> count(nlv + 1, 0);
            for (int cell = 0; cell < n; ++cell) count[lev[cell] + 1]++;
            for (int l = 0; l < nlv; ++l) count[l + 1] += count[l];
            lvstart.insert(lvstart.end(), count.begin(), count.end());
            std::vector<int4> ord(n);
            std::vector<int> fillp(count.begin(), count.end() - 1);
            for (int cell = 0; cell < n; ++cell) ord[fillp[lev[cell]]++] = rec[cell];
            cells.insert(cells.end(), ord.begin(), ord.end());
        }
    }
    GcDev& d = c->gcd;
    for (void* p : {(void*)d.seg, (void*)d.xpoli, (void*)d.xpolr, (void*)d.xpolrvel, (void*)d.oldsol,
                    (void*)d.oldsolvel, (void*)d.poldsol, (void*)d.poldsolvel, (void*)d.cell,
                    (void*)d.lvstart})
        cudaFree(p);
    d = GcDev();
    auto up = [&](auto** dst, const auto& v) -> int {
        using T = typename std::decay<decltype(v)>::type::value_type;
        const size_t n = std::max<size_t>(v.size(), 1);
        MG_CUDA(cudaMalloc(dst, n * sizeof(T)));
        if (!v.empty())
            MG_CUDA(copy_on(c->stream, *dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return 0;
    };
    if (int rc = up(&d.seg, seg)) return rc;
    if (int rc = up(&d.cell, cells)) return rc;
    if (int rc = up(&d.lvstart, lvstart)) return rc;
    if (int rc = up(&d.xpoli, xi)) return rc;
    if (int rc = up(&d.xpolr, xr)) return rc;
    if (int rc = up(&d.xpolrvel, xv)) return rc;
    const size_t ns = std::max<long long>(sv, 1);
    MG_CUDA(cudaMalloc(&d.oldsol, ns * sizeof(double)));
    MG_CUDA(cudaMalloc(&d.oldsolvel, ns * sizeof(double)));
    MG_CUDA(cudaMalloc(&d.poldsol, ns * sizeof(long long)));
    MG_CUDA(cudaMalloc(&d.poldsolvel, ns * sizeof(long long)));
    for (void* p : {(void*)d.oldsol, (void*)d.oldsolvel, (void*)d.poldsol, (void*)d.poldsolvel})
        MG_CUDA(zero_on(c->stream, p, ns * 8));
    for (const char* n : {"PWU", "PWV", "PWW"})
        if (!c->f3.count(n))
            if (int rc = alloc_field3(c, n)) return rc;
    // setsdivfield (:1488-1535): sdiv from the lists, connected, written back
    double* S = c->F("SDIV");
    MG_CUDA(zero_on(c->stream, S, (size_t)c->idim3d * sizeof(double)));
    const int nb = (c->ngrid + 127) / 128;
    k_gc_sdiv<<<nb, 128, 0, c->stream>>>(c->d_grids, d, S, c->L("DDX"), c->L("DDY"), c->L("DDZ"),
                                         c->ngrid, 1);
    MG_LAUNCHED(c);
    for (int l = c->maxlevel; l > c->minlevel; --l)
        if (int rc = launch_ftoc(c, l, S, S, 'S')) return rc;
    if (int rc = connect(c, 0, 2, nullptr, nullptr, nullptr, S, nullptr, nullptr, true, false, 0))
        return rc;
    k_gc_sdiv<<<nb, 128, 0, c->stream>>>(c->d_grids, d, S, c->L("DDX"), c->L("DDY"), c->L("DDZ"),
                                         c->ngrid, 0);
    MG_LAUNCHED(c);
    return 0;
}

int launch_gc_mode(Ctx* c, char mode, double* u, double* v, double* w, int ilevel) {
    ProfScope ps_(c, "gc");
    const GcDev& d = c->gcd;
    const int nt = 3 * c->ngrid;
    switch (mode) {
    case 'F':
    case 'X':
        k_gc_sol<<<nt, 128, 0, c->stream>>>(c->d_grids, d, u, v, w, c->ngrid, mode == 'X', ilevel);
        break;
    case 'S':
    case 'Z':
    case 'R':
    case 'Y': {
        // a restore reads positions only a save has written
        const int vel = mode == 'Z' || mode == 'Y', save = mode == 'S' || mode == 'Z';
        if (!save && !c->gc_saved[vel]) {
            set_error(vel ? "gc: restore Y before any save Z (setpointvalues with comp_new first, "
                            "as flow_mod.F90:83 does)"
                          : "gc: restore R before any save S (setibvalues first, as flow_mod.F90:84 does)");
            return MGLET_ERR_ARG;
        }
        k_gc_savrst<<<nt, 128, 0, c->stream>>>(c->d_grids, d, u, v, w, c->ngrid, vel, save, ilevel);
        if (save) c->gc_saved[vel] = true;
        break;
    }
    case 'C': {
        int* err = reinterpret_cast<int*>(c->d_scalar + 7);
        MG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
        k_gc_corr<<<c->ngrid, 128, 0, c->stream>>>(
            c->d_grids, d, u, v, w, c->L("DDX"), c->L("DDY"), c->L("DDZ"), c->ngrid, err, ilevel);
        MG_LAUNCHED(c);
        int herr = 0;
        MG_CUDA(copy_on(c->stream, &herr, err, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr) {
            set_error("wmxpolsolcorr: cut cell without open area");
            return MGLET_ERR_ARG;
        }
        return 0;
    }
    default:
        set_error("gc: unknown mode");
        return MGLET_ERR_ARG;
    }
    MG_LAUNCHED(c);
    return 0;
}

int launch_maskbp(Ctx* c, double* u, double* v, double* w, double* p) {
    ProfScope ps_(c, "maskbp");
    int m = 0;
    for (const DevGrid& g : c->grids) m = std::max(m, g.kk * g.jj * g.ii);
    const dim3 grid((m + 255) / 256, c->ngrid);
    k_maskbp<<<grid, 256, 0, c->stream>>>(c->d_grids, u, v, w, p, c->F("BP"));
    MG_LAUNCHED(c);
    return 0;
}

// setibvalues (gc_flowstencils_mod.F90:1393-1438) of U, V, W: per level
// (parent,) the extrapolation F and the flux correction C, each followed by
// bound_flow and connect; fine to coarse (ftoc of U, V, W, par_ftoc_norm);
// per level again (parent,) C and the save S
int gc_setibvalues(Ctx* c, double* u, double* v, double* w) {
    static const char* const vn[3] = {"U", "V", "W"};
    static const char* const none[3] = {nullptr, nullptr, nullptr};
    const bool ml = c->minlevel != c->maxlevel;
    auto bound = [&](int l) { return launch_bound_flow(c, u, v, w, nullptr, ml ? l : 0); };
    auto conn = [&](int l, int layers, bool corners) {
        return connect(c, ml ? l : 0, layers, u, v, w, nullptr, nullptr, nullptr, corners, false, 0);
    };
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        if (ml)
            if (int rc = launch_parent(c, l, vn, none, false)) return rc;
        if (int rc = bound(l)) return rc;
        if (int rc = conn(l, 2, false)) return rc;
        if (int rc = launch_gc_mode(c, 'F', u, v, w, l)) return rc;
        if (int rc = bound(l)) return rc;
        if (int rc = conn(l, 1, true)) return rc;
        if (int rc = launch_gc_mode(c, 'C', u, v, w, l)) return rc;
        if (int rc = bound(l)) return rc;
        if (int rc = conn(l, 1, true)) return rc;
    }
    for (int l = c->maxlevel; l > c->minlevel; --l) {
        if (int rc = launch_ftoc(c, l, u, u, 'U')) return rc;
        if (int rc = launch_ftoc(c, l, v, v, 'V')) return rc;
        if (int rc = launch_ftoc(c, l, w, w, 'W')) return rc;
        if (int rc = launch_par_ftoc_norm(c, l, u, v, w, false)) return rc;
    }
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        if (ml)
            if (int rc = launch_parent(c, l, vn, none, false)) return rc;
        if (int rc = bound(l)) return rc;
        if (int rc = conn(l, 1, true)) return rc;
        if (int rc = launch_gc_mode(c, 'C', u, v, w, l)) return rc;
        if (int rc = bound(l)) return rc;
        if (int rc = conn(l, 1, true)) return rc;
        if (int rc = launch_gc_mode(c, 'S', u, v, w, l)) return rc;
    }
    return 0;
}

// setpointvalues (:1323-1367)
int gc_setpointvalues(Ctx* c, bool comp_new) {
    double *pu = c->F("PWU"), *pv = c->F("PWV"), *pw = c->F("PWW");
    const size_t n = (size_t)c->idim3d * sizeof(double);
    MG_CUDA(cudaMemcpyAsync(pu, c->F("U"), n, cudaMemcpyDeviceToDevice, c->stream));
    MG_CUDA(cudaMemcpyAsync(pv, c->F("V"), n, cudaMemcpyDeviceToDevice, c->stream));
    MG_CUDA(cudaMemcpyAsync(pw, c->F("W"), n, cudaMemcpyDeviceToDevice, c->stream));
    if (int rc = launch_gc_mode(c, comp_new ? 'X' : 'Y', pu, pv, pw)) return rc;
    // pwu%buffers = u%buffers: bound_flow takes the U, V, W boundary buffers
    const bool ml = c->minlevel != c->maxlevel;
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        if (int rc = connect(c, ml ? l : 0, 1, pu, pv, pw, nullptr, nullptr, nullptr, false, false, 0))
            return rc;
        if (int rc = launch_bound_flow(c, pu, pv, pw, nullptr, ml ? l : 0)) return rc;
    }
    if (comp_new) return launch_gc_mode(c, 'Z', pu, pv, pw);
    return 0;
}

}  // namespace mg
