// api.cu -- the C ABI of include/mglet_gpu.h and the host-side runtime
// behind it: context set-up (grid tables, connection task lists,
// hyperplane traversal tables, coefficient set-up on the device), field
// transfers and the orchestration of the RK stage.
//
// Host logic mirrored from the reference (single rank):
//   init_connect_core / get_nbrs     src/core/connect/connect_core_mod.F90:167-433
//   start_and_stop(_face), corr_start_stop, decide
//                                    src/core/connect/connect_core_mod.F90:454-682
//   sip_hyperplane_init_grid/sort    src/flow/sip_hyperplane_mod.F90:269-393
//   timeintegrate_flow               src/flow/timeintegration_mod.F90:22-142
//   mgpoisl / mgpoisit / sip         src/flow/pressuresolver_mod.F90:160-465
//   rk_2n_t                          src/core/rungekutta_mod.F90:29-309
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <string>

#include "internal.h"
#include "mixed.h"

namespace mg {

static thread_local std::string t_err;

void set_error(const std::string& msg) { t_err = msg; }

int cuda_fail(cudaError_t e, const char* what) {
    t_err = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    return MGLET_ERR_CUDA;
}

static int fail(int code, const std::string& msg) {
    t_err = msg;
    return code;
}


namespace {

// Face geometry of the 26 connection slots (facelist, facenbr, rescue_dir,
// rescue_nbr of connect_core_mod.F90:38-159).  These tables are part of the
// reference's connection contract and are reproduced as data.
const int kFaces[27][4] = {
    {0, 0, 0, 0},
    {1, 1, 0, 0}, {1, 2, 0, 0}, {1, 3, 0, 0}, {1, 4, 0, 0}, {1, 5, 0, 0}, {1, 6, 0, 0},
    {2, 1, 3, 0}, {2, 1, 4, 0}, {2, 1, 5, 0}, {2, 1, 6, 0}, {2, 2, 3, 0}, {2, 2, 4, 0},
    {2, 2, 5, 0}, {2, 2, 6, 0}, {2, 3, 5, 0}, {2, 3, 6, 0}, {2, 4, 5, 0}, {2, 4, 6, 0},
    {3, 1, 3, 5}, {3, 1, 3, 6}, {3, 1, 4, 5}, {3, 1, 4, 6}, {3, 2, 3, 5}, {3, 2, 3, 6},
    {3, 2, 4, 5}, {3, 2, 4, 6}};
const int kOpposite[27] = {0, 2, 1, 4, 3, 6, 5, 12, 11, 14, 13, 8, 7, 10, 9,
                           18, 17, 16, 15, 26, 25, 24, 23, 22, 21, 20, 19};
const int kRescueDir[27][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {1, 0, 0, 0, 0, 0, 0}, {2, 0, 0, 0, 0, 0, 0}, {3, 0, 0, 0, 0, 0, 0},
    {4, 0, 0, 0, 0, 0, 0}, {5, 0, 0, 0, 0, 0, 0}, {6, 0, 0, 0, 0, 0, 0},
    {7, 1, 3, 0, 0, 0, 0}, {8, 4, 1, 0, 0, 0, 0}, {9, 1, 5, 0, 0, 0, 0},
    {10, 6, 1, 0, 0, 0, 0}, {11, 2, 3, 0, 0, 0, 0}, {12, 2, 4, 0, 0, 0, 0},
    {13, 2, 5, 0, 0, 0, 0}, {14, 2, 6, 0, 0, 0, 0}, {15, 3, 5, 0, 0, 0, 0},
    {16, 6, 3, 0, 0, 0, 0}, {17, 4, 5, 0, 0, 0, 0}, {18, 4, 6, 0, 0, 0, 0},
    {19, 7, 9, 15, 1, 3, 5}, {20, 7, 10, 16, 1, 3, 6}, {21, 8, 9, 17, 1, 4, 5},
    {22, 8, 10, 18, 1, 4, 6}, {23, 11, 13, 15, 2, 3, 5}, {24, 11, 14, 16, 2, 3, 6},
    {25, 12, 13, 17, 2, 4, 5}, {26, 12, 14, 18, 2, 4, 6}};
const int kRescueNbr[27][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {2, 0, 0, 0, 0, 0, 0}, {1, 0, 0, 0, 0, 0, 0}, {4, 0, 0, 0, 0, 0, 0},
    {3, 0, 0, 0, 0, 0, 0}, {6, 0, 0, 0, 0, 0, 0}, {5, 0, 0, 0, 0, 0, 0},
    {12, 11, 8, 0, 0, 0, 0}, {11, 7, 12, 0, 0, 0, 0}, {14, 13, 10, 0, 0, 0, 0},
    {13, 9, 14, 0, 0, 0, 0}, {8, 7, 12, 0, 0, 0, 0}, {7, 8, 11, 0, 0, 0, 0},
    {10, 9, 14, 0, 0, 0, 0}, {9, 10, 13, 0, 0, 0, 0}, {18, 17, 16, 0, 0, 0, 0},
    {17, 15, 18, 0, 0, 0, 0}, {16, 15, 18, 0, 0, 0, 0}, {15, 16, 17, 0, 0, 0, 0},
    {26, 25, 24, 22, 23, 21, 20}, {25, 26, 23, 21, 24, 22, 19},
    {24, 23, 26, 20, 25, 19, 22}, {23, 24, 25, 19, 26, 20, 21},
    {22, 21, 20, 26, 19, 25, 24}, {21, 22, 19, 25, 20, 26, 23},
    {20, 19, 22, 24, 21, 23, 26}, {19, 20, 21, 23, 22, 24, 25}};

bool coupled(int t) { return t == MGLET_BC_CON || t == MGLET_BC_CO1; }



struct Box {
    int lo[3], hi[3];   // k, j, i ranges (1-based, inclusive)
};

// Ghost (or, with inner=true, the matching interior) slab of one elementary
// face, applied to the box in place.
void face_range(const DevGrid& G, int face, Box& b, int nplane, bool inner) {
    const int ax = (face - 1) / 2 == 0 ? 2 : ((face - 1) / 2 == 1 ? 1 : 0);   // i, j, k axis
    const int n = ax == 2 ? G.ii : (ax == 1 ? G.jj : G.kk);
    const bool low = (face % 2) == 1;
    if (low) { b.lo[ax] = 3 - nplane; b.hi[ax] = 2; }
    else { b.lo[ax] = n - 1; b.hi[ax] = n - (2 - nplane); }
    if (inner) {
        const int s = low ? nplane : -nplane;
        b.lo[ax] += s;
        b.hi[ax] += s;
    }
}

Box slot_box(const DevGrid& G, int slot, int nplane, bool inner) {
    Box b{{3, 3, 3}, {G.kk - 2, G.jj - 2, G.ii - 2}};
    for (int q = 1; q <= kFaces[slot][0]; ++q) face_range(G, kFaces[slot][q], b, nplane, inner);
    return b;
}

void neighbour_of(const Ctx* c, int g, int slot, int& ng, int& nf) {
    ng = 0;
    nf = 0;
    const std::vector<int>& nb = c->nbr[g];
    for (int q = 0; q < 7; ++q) {
        const int dir = kRescueDir[slot][q];
        if (dir == 0) break;
        if (nb[dir] <= 0) continue;
        ng = nb[dir];
        nf = kRescueNbr[slot][q];
        if (nf > 18) {
            const DevGrid& N = c->grids[ng - 1];
            if (!coupled(N.bc[kFaces[nf][1] - 1]) && !coupled(N.bc[kFaces[nf][2] - 1]) &&
                !coupled(N.bc[kFaces[nf][3] - 1])) {
                ng = 0;
                nf = 0;
                continue;
            }
        }
        return;
    }
}

void build_connection_table(Ctx* c) {
    c->conns.clear();
    for (int g = 1; g <= c->ngrid; ++g) {
        const DevGrid& G = c->grids[g - 1];
        for (int slot = 1; slot <= 26; ++slot) {
            bool any = false;
            for (int q = 1; q <= kFaces[slot][0]; ++q) any |= coupled(G.bc[kFaces[slot][q] - 1]);
            if (!any) continue;
            int ng, nf;
            neighbour_of(c, g, slot, ng, nf);
            if (ng == 0) continue;
            c->conns.insert(c->conns.end(), {g, ng, slot, nf});
        }
    }
}

long long lidx(const DevGrid& G, int k, int j, int i) {
    return G.ip3 + (long long)(i - 1) * G.kk * G.jj + (long long)(j - 1) * G.kk + (k - 1);
}

// Task list of one connect variant; slots = bitmask of present fields
// (bit 0..5 = v1 v2 v3 s1 s2 s3).
int build_plan(Ctx* c, int ilevel, int layers, int slots, bool corners, bool normal, int fwd,
               ConnectPlan& plan) {
    std::vector<BoxCopy> tasks;
    long long npts = 0;
    for (size_t r = 0; r < c->conns.size(); r += 4) {
        const int rg = c->conns[r], sg = c->conns[r + 1], rf = c->conns[r + 2],
                  sf = c->conns[r + 3];
        const DevGrid& D = c->grids[rg - 1];
        const DevGrid& S = c->grids[sg - 1];
        if (ilevel > 0 && D.level != ilevel) continue;
        if (!corners && rf > 6) continue;
        if (fwd == 1 && (rf == 2 || rf == 4 || rf == 6)) continue;
        if (fwd == -1 && (rf == 1 || rf == 3 || rf == 5)) continue;
        Box src = slot_box(S, kOpposite[rf], layers, true);
        if (rf > 6)   // corr_start_stop: elementary faces shared by send and recv slot
            for (int a = 1; a <= kFaces[sf][0]; ++a)
                for (int b = 1; b <= kFaces[rf][0]; ++b)
                    if (kFaces[sf][a] == kFaces[rf][b]) face_range(S, kFaces[sf][a], src, layers, false);
        Box dst = slot_box(D, rf, layers, false);
        const int n[3] = {dst.hi[0] - dst.lo[0] + 1, dst.hi[1] - dst.lo[1] + 1,
                          dst.hi[2] - dst.lo[2] + 1};
        const long long ns = (long long)(src.hi[0] - src.lo[0] + 1) * (src.hi[1] - src.lo[1] + 1) *
                             (src.hi[2] - src.lo[2] + 1);
        if (ns != (long long)n[0] * n[1] * n[2])
            return fail(MGLET_ERR_ARG, "connect: source and destination sizes differ");
        const bool exu = !normal || rf < 3;
        const bool exv = !normal || (rf > 2 && rf < 5);
        const bool exw = !normal || rf > 4;
        const bool ex[6] = {exu, exv, exw, true, true, true};
        for (int s = 0; s < 6; ++s) {
            if (!(slots & (1 << s)) || !ex[s]) continue;
            BoxCopy t;
            t.dst = lidx(D, dst.lo[0], dst.lo[1], dst.lo[2]);
            t.src = lidx(S, src.lo[0], src.lo[1], src.lo[2]);
            t.nk = n[0]; t.nj = n[1]; t.ni = n[2];
            t.dkk = D.kk; t.djj = D.kk * D.jj;
            t.skk = S.kk; t.sjj = S.kk * S.jj;
            t.slot = s;
            t.npts = n[0] * n[1] * n[2];
            npts += t.npts;
            tasks.push_back(t);
        }
    }
    plan.ntasks = (int)tasks.size();
    plan.npts = npts;
    if (!tasks.empty()) {
        MG_CUDA(cudaMalloc(&plan.d_tasks, tasks.size() * sizeof(BoxCopy)));
        MG_CUDA(copy_on(c->stream, plan.d_tasks, tasks.data(), tasks.size() * sizeof(BoxCopy),
                           cudaMemcpyHostToDevice));
    }
    return 0;
}

// Hyperplane traversal table for one grid shape: the same index lists as
// sip_hyperplane_init_grid + sip_hyperplane_sort, 0-based.
int build_hp_table(cudaStream_t stream, int kk, int jj, int ii, HpTable& t) {
    t.kk = kk; t.jj = jj; t.ii = ii;
    t.n3dmin = 9;
    t.n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    std::vector<int> mip(kk + jj + ii + 2, 0), idx;
    idx.reserve((size_t)(kk - 4) * (jj - 4) * (ii - 4));
    for (int m = t.n3dmin; m <= t.n3dmax; ++m) {
        mip[m] = (int)idx.size();
        // ascending linear index k + (j-1)kk + (i-1)kk jj == ascending (i, j)
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j) {
                const int k = m - i - j;
                if (k < 3 || k > kk - 2) continue;
                idx.push_back((k - 1) + (j - 1) * kk + (i - 1) * kk * jj);
            }
        t.maxplane = std::max(t.maxplane, (int)idx.size() - mip[m]);
    }
    mip[t.n3dmax + 1] = (int)idx.size();
    t.npts = (int)idx.size();
    if (t.npts != (kk - 4) * (jj - 4) * (ii - 4))
        return fail(MGLET_ERR_ARG, "hyperplane table does not cover the interior");
    MG_CUDA(cudaMalloc(&t.d_mip, mip.size() * sizeof(int)));
    MG_CUDA(cudaMalloc(&t.d_idx, idx.size() * sizeof(int)));
    MG_CUDA(copy_on(stream, t.d_mip, mip.data(), mip.size() * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(copy_on(stream, t.d_idx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice));
    return 0;
}

__global__ void k_reciprocal(double* r, const double* a, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) r[t] = a[t] == 0.0 ? 0.0 : 1.0 / a[t];   // divide0
}

__global__ void k_fill(double* a, double v, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; t < n; t += stride) a[t] = v;
}

int alloc3(Ctx* c, const char* name) {
    double* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (size_t)c->idim3d * sizeof(double));
    if (e != cudaSuccess) return fail(MGLET_ERR_NOMEM, std::string("cudaMalloc ") + name);
    MG_CUDA(cudaMemsetAsync(p, 0, (size_t)c->idim3d * sizeof(double), c->stream));
    c->f3[name] = p;
    return 0;
}

int alloc1(Ctx* c, const char* name, long long n, const double* host) {
    double* p = nullptr;
    MG_CUDA(cudaMalloc(&p, (size_t)n * sizeof(double)));
    if (host) MG_CUDA(copy_on(c->stream, p, host, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    else MG_CUDA(zero_on(c->stream, p, (size_t)n * sizeof(double)));
    c->f1[name] = p;
    return 0;
}

int fill(Ctx* c, double* a, double v) {
    long long n = c->idim3d;
    int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    k_fill<<<blocks, 256, 0, c->stream>>>(a, v, n);
    MG_LAUNCHED(c);
    return 0;
}

std::string plan_key(int ilevel, int layers, int slots, bool corners, bool normal, int fwd) {
    char b[96];
    std::snprintf(b, sizeof(b), "%d/%d/%d/%d/%d/%d", ilevel, layers, slots, (int)corners,
                  (int)normal, fwd);
    return b;
}

}  // namespace

int alloc_field3(Ctx* c, const char* name) { return alloc3(c, name); }
int fill_field(Ctx* c, double* a, double v) { return fill(c, a, v); }

int connect(Ctx* c, int ilevel, int layers, double* v1, double* v2, double* v3, double* s1,
            double* s2, double* s3, bool corners, bool normal, int forward) {
    if (layers < 1 || layers > 2) return fail(MGLET_ERR_ARG, "connect: layers must be 1 or 2");
    const int fwd = forward > 0 ? 1 : (forward < 0 ? -1 : 0);
    if ((fwd != 0 || normal) && corners)
        return fail(MGLET_ERR_ARG, "connect: corners excludes forward and normal");
    if (normal && !(v1 && v2 && v3)) return fail(MGLET_ERR_ARG, "connect: normal needs v1..v3");
    double* f[6] = {v1, v2, v3, s1, s2, s3};
    int slots = 0;
    for (int q = 0; q < 6; ++q)
        if (f[q]) slots |= 1 << q;
    if (!slots) return fail(MGLET_ERR_ARG, "connect: no fields");
    const std::string key = plan_key(ilevel, layers, slots, corners, normal, fwd);
    auto it = c->plans.find(key);
    if (it == c->plans.end()) {
        ConnectPlan p;
        if (int rc = build_plan(c, ilevel, layers, slots, corners, normal, fwd, p)) return rc;
        it = c->plans.emplace(key, p).first;
    }
    // several ranks: the copies of remote grids first get their owners'
    // current boxes (the receive half of connect2_mod.F90:406-548)
    if (c->part)
        if (int rc = part_exchange(c, f)) return rc;
    return launch_connect(c, it->second, f);
}

int get_plan(Ctx* c, int ilevel, int layers, int slots, bool corners, bool normal, int fwd,
             const ConnectPlan** out) {
    const std::string key = plan_key(ilevel, layers, slots, corners, normal, fwd);
    auto it = c->plans.find(key);
    if (it == c->plans.end()) {
        ConnectPlan p;
        if (int rc = build_plan(c, ilevel, layers, slots, corners, normal, fwd, p)) return rc;
        it = c->plans.emplace(key, p).first;
    }
    *out = &it->second;
    return 0;
}

long long connect_points(Ctx* c, int ilevel, int layers, int slots, bool corners, bool normal,
                         int fwd) {
    const std::string key = plan_key(ilevel, layers, slots, corners, normal, fwd);
    auto it = c->plans.find(key);
    return it == c->plans.end() ? -1 : it->second.npts;
}

// ---------------------------------------------------------------------------
// mgpoisl, plain FP64 form (pressuresolver_mod.F90:160-357) over every level
// of the hierarchy; on one level ftoc, ctof, parent and bound_pressure have
// no work.  mgpoisit works on HILF, whose PAR buffers parent fills.
static int mgpoisit_plain(Ctx* c, int ilevel, double* dp, double* rhs, double* res) {
    const int ninner = c->prm.ninner;
    const bool withbp = c->ibtype == 1;
    double* hbuf = field_buffer(c, "HILF");
    if (!hbuf) return fail(MGLET_ERR_CUDA, "mgpoisl: buffer allocation");
    for (int iloop = 1; iloop <= ninner; ++iloop) {
        if (int rc = launch_bound_pressure(c, ilevel, dp, hbuf, withbp)) return rc;
        if (c->prm.psolver == MGLET_PSOLVER_SOR && ilevel > c->minlevel) {
            if (int rc = MG_PLAIN_FN(c, launch_sor)(c, ilevel, dp, rhs)) return rc;
        } else {
            if (int rc = MG_PLAIN_FN(c, launch_laplacephi)(c, ilevel, res, dp)) return rc;
            if (int rc = MG_PLAIN_FN(c, launch_sipiter1)(c, ilevel, rhs, res)) return rc;
            if (int rc = connect(c, ilevel, 1, nullptr, nullptr, nullptr, res, nullptr, nullptr,
                                 false, false, iloop < ninner ? 0 : -1))
                return rc;
            if (int rc = MG_PLAIN_FN(c, launch_sipiter2)(c, ilevel, dp, res)) return rc;
        }
        if (int rc = connect(c, ilevel, 1, nullptr, nullptr, nullptr, dp, nullptr, nullptr, false,
                             false, 0))
            return rc;
    }
    return launch_bound_pressure(c, ilevel, dp, hbuf, withbp);
}

// The outer defect-correction loop of mgpoisl (pressuresolver_mod.F90:
// 203-305) on RHS, accumulating DP; HILF, RES and DP start at zero (cleared
// here when zero_work is set).  prefak scales the convergence test; 0 takes
// max|RHS| (a relative test), and an all-zero RHS returns DP = 0.
int solve_pressure_system(Ctx* c, double prefak, mglet_stage_stats* st, bool zero_work) {
    double* dp = c->F("DP"); double* hilf = c->F("HILF");
    double* rhs = c->F("RHS"); double* res = c->F("RES");
    const size_t bytes = (size_t)c->idim3d * sizeof(double);
    if (zero_work)
        for (double* a : {dp, hilf, res}) MG_CUDA(cudaMemsetAsync(a, 0, bytes, c->stream));
    if (int rc = launch_bp_ones(c)) return rc;
    if (prefak <= 0.0) {
        if (int rc = MG_PLAIN_FN(c, launch_rescal_maxabs)(c, rhs, nullptr)) return rc;
        MG_CUDA(cudaMemcpyAsync(c->h_scalar, c->d_scalar, sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        if (int rc = part_allreduce(c, c->h_scalar, 1, 1)) return rc;
        prefak = c->h_scalar[0];
        if (!(prefak > 0.0)) {
            if (st) *st = mglet_stage_stats{0, 0, 0.0, 0.0};
            return 0;
        }
    }
    const bool multi = c->minlevel != c->maxlevel;
    const char* const none[3] = {nullptr, nullptr, nullptr};
    const char* const shilf[3] = {"HILF", nullptr, nullptr};
    int ipc = 0, done = 0;
    double maxrhs = 0.0;
    for (int ipcount = 1; ipcount <= c->prm.nouter; ++ipcount) {
        for (int l = c->minlevel; l <= c->maxlevel; ++l) {
            if (int rc = launch_ctof(c, l, hilf, hilf)) return rc;
            if (int rc = launch_parent(c, l, none, shilf, false)) return rc;
            if (int rc = mgpoisit_plain(c, l, hilf, rhs, res)) return rc;
        }
        for (int l = c->maxlevel; l >= c->minlevel; --l)
            if (int rc = launch_ftoc(c, l, hilf, hilf, 'P')) return rc;
        if (int rc = connect(c, 0, 1, nullptr, nullptr, nullptr, hilf, nullptr, nullptr, false,
                             false, 0))
            return rc;
        if (int rc = MG_PLAIN_FN(c, launch_laplacephi)(c, 0, res, hilf)) return rc;
        if (int rc = MG_PLAIN_FN(c, launch_rescal_maxabs)(c, rhs, res)) return rc;
        if (multi) {
            // rhs restricted into the coarse grids, then its maximum again
            for (int l = c->maxlevel; l >= c->minlevel + 1; --l)
                if (int rc = launch_ftoc(c, l, rhs, rhs, 'R')) return rc;
            if (int rc = MG_PLAIN_FN(c, launch_rescal_maxabs)(c, rhs, nullptr)) return rc;
        }
        if (int rc = MG_PLAIN_FN(c, launch_accumulate)(c, dp, hilf)) return rc;
        ipc += c->prm.ninner;
        done = ipcount;
        if (ipcount >= c->prm.nouter_min) {
            MG_CUDA(cudaMemcpyAsync(c->h_scalar, c->d_scalar, sizeof(double),
                                    cudaMemcpyDeviceToHost, c->stream));
            MG_CUDA(cudaStreamSynchronize(c->stream));
            // MPI_Allreduce(MAX) of pressuresolver_mod.F90:295
            if (int rc = part_allreduce(c, c->h_scalar, 1, 1)) return rc;
            maxrhs = c->h_scalar[0];
            if (maxrhs / prefak < c->prm.epcorr) break;
        }
    }
    if (done < c->prm.nouter_min || c->prm.nouter_min > c->prm.nouter || done == 0) {
        // maxrhs of the last outer iteration if it was not read above
        MG_CUDA(cudaMemcpyAsync(c->h_scalar, c->d_scalar, sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        if (int rc = part_allreduce(c, c->h_scalar, 1, 1)) return rc;
        maxrhs = c->h_scalar[0];
    }
    if (st) {
        st->ipc = ipc;
        st->nouter_done = done;
        st->maxrhs = maxrhs;
        st->prefak = prefak;
    }
    return 0;
}

static int mgpoisl_plain(Ctx* c, double dt, mglet_stage_stats* st) {
    double* U = c->F("U"); double* V = c->F("V"); double* W = c->F("W"); double* P = c->F("P");
    double* dp = c->F("DP"); double* hilf = c->F("HILF");
    double* rhs = c->F("RHS"); double* res = c->F("RES");
    const size_t bytes = (size_t)c->idim3d * sizeof(double);
    for (double* a : {dp, hilf, rhs, res}) MG_CUDA(cudaMemsetAsync(a, 0, bytes, c->stream));
    const double prefak = c->prm.rho / dt;
    const char* const none[3] = {nullptr, nullptr, nullptr};
    if (int rc = MG_PLAIN_FN(c, launch_divcal)(c, rhs, U, V, W, prefak)) return rc;
    for (int l = c->maxlevel; l >= c->minlevel; --l)
        if (int rc = launch_ftoc(c, l, rhs, rhs, 'R')) return rc;
    if (int rc = solve_pressure_system(c, prefak, st, false)) return rc;
    const char* const sdp[3] = {"DP", nullptr, nullptr};
    double* dbuf = field_buffer(c, "DP");
    if (!dbuf) return fail(MGLET_ERR_CUDA, "mgpoisl: buffer allocation");
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        if (int rc = launch_parent(c, l, none, sdp, false)) return rc;
        if (int rc = launch_bound_pressure(c, l, dp, dbuf, c->ibtype == 1)) return rc;
    }
    if (int rc = MG_PLAIN_FN(c, launch_mgpcorr)(c, U, V, W, P, dp, dt / c->prm.rho)) return rc;
    // pressuresolver_mod.F90:334-348: ftoc fine to coarse, then per level
    // parent, bound and the corner connect
    for (int l = c->maxlevel; l >= c->minlevel; --l) {
        if (int rc = launch_ftoc(c, l, U, U, 'U')) return rc;
        if (int rc = launch_ftoc(c, l, V, V, 'V')) return rc;
        if (int rc = launch_ftoc(c, l, W, W, 'W')) return rc;
        if (int rc = launch_ftoc(c, l, P, P, 'P')) return rc;
    }
    const char* const vuvw[3] = {"U", "V", "W"};
    const char* const sp[3] = {"P", nullptr, nullptr};
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        if (int rc = launch_parent(c, l, vuvw, sp, false)) return rc;
        if (int rc = launch_bound_flow(c, U, V, W, P, l)) return rc;
        if (int rc = connect(c, l, 2, U, V, W, P, nullptr, nullptr, true, false, 0)) return rc;
    }
    return 0;
}

// The pressure solve and the stage run on hierarchies once the parents are
// known.
int hierarchy_ready(Ctx* c) {
    for (int g = 0; g < c->ngrid; ++g)
        if (c->grids[g].level != c->minlevel && c->hier[g].x < 0)
            return fail(MGLET_ERR_ARG, "a fine grid without parent (mglet_gpu_set_hierarchy first)");
    return 0;
}

int mgpoisl(Ctx* c, double dt, mglet_stage_stats* st) {
    if (int rc = hierarchy_ready(c)) return rc;
    if (c->prm.form == MGLET_FORM_MIXED) return mixed_mgpoisl(c, dt, st);
    return mgpoisl_plain(c, dt, st);
}

int rk_coeffs(const mglet_rk_scheme* rk, int irk, double* frhs, double* fu, double* dtrk,
              double* dtrki) {
    if (!rk || irk < 1 || irk > rk->nrk) return fail(MGLET_ERR_ARG, "rk: irk out of range");
    *frhs = rk->a[irk - 1];
    *fu = rk->b[irk - 1];
    *dtrk = irk < rk->nrk ? rk->c[irk] : 1.0;
    *dtrki = *dtrk - rk->c[irk - 1];
    return 0;
}

static int stage_plain(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk,
                       mglet_stage_stats* st) {
    double frhs, fu, dtrk, dtrki;
    if (int rc = rk_coeffs(rk, irk, &frhs, &fu, &dtrk, &dtrki)) return rc;
    double *U = c->F("U"), *V = c->F("V"), *W = c->F("W"), *P = c->F("P"), *G = c->F("G");
    double *UO = c->F("UO"), *VO = c->F("VO"), *WO = c->F("WO");
    const bool gc = c->ibtype == 1;
    // timeintegration_mod.F90:96-99: the ghost-cell fluxes of the step
    if (irk == 1 && gc)
        if (int rc = gc_setibvalues(c, U, V, W)) return rc;
    if (int rc = MG_PLAIN_FN(c, launch_tstle4)(c, UO, VO, WO, gc ? c->F("PWU") : U,
                                               gc ? c->F("PWV") : V, gc ? c->F("PWW") : W, U, V, W,
                                               P, G))
        return rc;
    if (int rc = launch_momentum_sources(c)) return rc;     // :102-103 boussinesq, coriolis
    if (int rc = MG_PLAIN_FN(c, launch_rkstep)(c, U, c->F("DU"), UO, frhs, dt * fu)) return rc;
    if (int rc = MG_PLAIN_FN(c, launch_rkstep)(c, V, c->F("DV"), VO, frhs, dt * fu)) return rc;
    if (int rc = MG_PLAIN_FN(c, launch_rkstep)(c, W, c->F("DW"), WO, frhs, dt * fu)) return rc;
    if (gc) {   // timeintegration_mod.F90:110-116: maskbp, getibvalues
        if (int rc = launch_maskbp(c, U, V, W, P)) return rc;
        if (int rc = launch_gc_mode(c, 'R', U, V, W)) return rc;
    }
    // timeintegration_mod.F90:117-122: per level connect (normal, forward),
    // parent (u, v, w, p into the PAR buffers) and bound_flow
    static const char* const vn[3] = {"U", "V", "W"};
    static const char* const sn[3] = {"P", nullptr, nullptr};
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        if (int rc = connect(c, l, 1, U, V, W, nullptr, nullptr, nullptr, false, true, 1)) return rc;
        if (c->minlevel != c->maxlevel)
            if (int rc = launch_parent(c, l, vn, sn, false)) return rc;
        if (int rc = launch_bound_flow(c, U, V, W, P, c->minlevel != c->maxlevel ? l : 0)) return rc;
    }
    if (int rc = mgpoisl(c, dtrk * dt, st)) return rc;
    if (int rc = lesmodel(c)) return rc;                  // :125
    if (gc) return gc_setpointvalues(c, irk == rk->nrk);   // :131-134
    return 0;
}

int timeintegrate(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk, mglet_stage_stats* st) {
    if (int rc = hierarchy_ready(c)) return rc;
    if (c->prm.form == MGLET_FORM_MIXED) return mixed_stage(c, dt, irk, rk, st);
    return stage_plain(c, dt, irk, rk, st);
}

}  // namespace mg

// ===========================================================================
// C ABI
using namespace mg;

struct mglet_ctx : mg::Ctx {};

static double* field_ptr(mglet_ctx* c, const char* name) {
    if (!name) return nullptr;
    auto it = c->f3.find(name);
    return it == c->f3.end() ? nullptr : it->second;
}

extern "C" {

int32_t mglet_gpu_abi_version(void) { return MGLET_GPU_ABI_VERSION; }

const char* mglet_gpu_last_error(void) { return t_err.c_str(); }

// Williamson (1980) 3-stage, Berland-Bogey-Bailly (2006) 6-stage,
// Carpenter-Kennedy (1994) 5-stage and Bernardini-Pirozzoli (2009) 5-stage
// 2N-storage schemes with the coefficient values the reference uses.
int mglet_rk_init(const char* name, mglet_rk_scheme* rk) {
    if (!name || !rk) return fail(MGLET_ERR_ARG, "rk_init: null argument");
    std::memset(rk, 0, sizeof(*rk));
    std::string n(name);
    for (char& ch : n) ch = (char)std::tolower((unsigned char)ch);
    auto fill_c = [rk]() {   // c_i = sum_{j<i} b_j prod (a_k ... + 1)
        for (int i = 0; i < rk->nrk; ++i) {
            double ci = 0.0;
            for (int j = 1; j <= i; ++j) {
                double f = 1.0;
                for (int k = 2; k <= j; ++k) f = rk->a[k - 1] * f + 1.0;
                ci = ci + rk->b[j - 1] * f;
            }
            rk->c[i] = ci;
        }
    };
    if (n == "williamson") {
        rk->nrk = 3;
        rk->cflmax = (1.0 - 2.220446049250313e-16) * std::sqrt(3.0);
        const double a[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
        const double b[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
        const double cc[3] = {0.0, 1.0 / 3.0, 3.0 / 4.0};
        for (int q = 0; q < 3; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; rk->c[q] = cc[q]; }
    } else if (n == "berland") {
        rk->nrk = 6;
        rk->cflmax = (double)(3.80f - 0.01f);
        const double a[6] = {0.0, -0.737101392796, -1.634740794341, -0.744739003780,
                             -1.469897351522, -2.813971388035};
        const double b[6] = {0.032918605146, 0.823256998200, 0.381530948900, 0.200092213184,
                             1.718581042715, 0.27};
        for (int q = 0; q < 6; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; }
        fill_c();
    } else if (n == "carpenter") {
        rk->nrk = 5;
        rk->cflmax = (double)(3.34f - 0.01f);
        const double a[5] = {0.0, -567301805773.0 / 1357537059087.0,
                             -2404267990393.0 / 2016746695238.0,
                             -3550918686646.0 / 2091501179385.0,
                             -1275806237668.0 / 842570457699.0};
        const double b[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                             1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                             2277821191437.0 / 14882151754819.0};
        for (int q = 0; q < 5; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; }
        fill_c();
    } else if (n == "bernardini") {
        rk->nrk = 5;
        rk->cflmax = (double)(3.47f - 0.01f);
        const double e = -3.88856487394645e-7;
        const double a[5] = {0.0, -1.0, -1.55798 + e, -1.0, -0.45031 + e};
        const double b[5] = {0.2, 0.83204 + e, 0.6, 0.35394 + e, 0.2};
        for (int q = 0; q < 5; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; }
        fill_c();
    } else {
        return fail(MGLET_ERR_ARG, "rk_init: unknown scheme '" + n + "'");
    }
    return 0;
}

int mglet_rk_get_coeffs(const mglet_rk_scheme* rk, int32_t irk, double* frhs, double* fu,
                        double* dtrk, double* dtrki) {
    return rk_coeffs(rk, irk, frhs, fu, dtrk, dtrki);
}

int mglet_gpu_create(const mglet_grid_desc* d, const mglet_flow_params* prm, int32_t device,
                     mglet_ctx** out) {
    if (!d || !prm || !out || d->ngrid <= 0 || !d->mgdims || !d->level || !d->bctype ||
        !d->nbrgrid)
        return fail(MGLET_ERR_ARG, "create: incomplete grid description");
    if (prm->ninner < 0 || prm->nouter < 0 || prm->nouter_min < 0 || prm->epcorr < 0.0 ||
        prm->rho <= 0.0 || prm->gmol < 0.0)
        return fail(MGLET_ERR_ARG, "create: invalid flow parameters");
    if (prm->psolver < 0 || prm->psolver > 2) return fail(MGLET_ERR_ARG, "create: bad psolver");
    if (prm->psolver == MGLET_PSOLVER_SOR && (prm->omega <= 0.0 || prm->omega >= 2.0))
        return fail(MGLET_ERR_ARG, "create: invalid omega");
    if (prm->form != MGLET_FORM_PLAIN && prm->form != MGLET_FORM_MIXED &&
        prm->form != MGLET_FORM_PLAIN_FMA)
        return fail(MGLET_ERR_ARG, "create: bad form");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(MGLET_ERR_CUDA, "create: no CUDA device");
    if (device < 0 || device >= ndev) return fail(MGLET_ERR_ARG, "create: bad device index");
    MG_CUDA(cudaSetDevice(device));
    mglet_ctx* c = new mglet_ctx();
    c->device = device;
    c->prm = *prm;
    // the contracted build runs the plain form's code path with its own kernels
    c->fma = prm->form == MGLET_FORM_PLAIN_FMA;
    if (c->fma) c->prm.form = MGLET_FORM_PLAIN;
    c->ngrid = d->ngrid;
    auto bail = [&](int rc) {
        mglet_gpu_destroy(c);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(MGLET_ERR_CUDA, "create: stream"));
    long long o3 = 0;
    int ox = 0, oy = 0, oz = 0;
    c->minlevel = 1 << 30;
    c->maxlevel = -1;
    c->grids.resize(c->ngrid);
    c->nbr.assign(c->ngrid + 1, std::vector<int>(27, 0));
    std::vector<long long> shapes;
    for (int g = 0; g < c->ngrid; ++g) {
        DevGrid& G = c->grids[g];
        G.kk = d->mgdims[3 * g]; G.jj = d->mgdims[3 * g + 1]; G.ii = d->mgdims[3 * g + 2];
        if (G.kk < 6 || G.jj < 6 || G.ii < 6)
            return bail(fail(MGLET_ERR_ARG, "create: grid smaller than 2 interior cells"));
        G.level = d->level[g];
        for (int f = 0; f < 6; ++f) {
            G.bc[f] = d->bctype[6 * g + f];
            const int t = G.bc[f];
            if (!(coupled(t) || t == MGLET_BC_FIX || t == MGLET_BC_OP1 || t == MGLET_BC_NOS ||
                  t == MGLET_BC_SLI || t == MGLET_BC_PAR))
                return bail(fail(MGLET_ERR_UNSUPPORTED,
                                 "create: faces must be CON, CO1, FIX, OP1, NOS, SLI or PAR"));
        }
        for (int s = 1; s <= 26; ++s) {
            const int nb = d->nbrgrid[26 * g + s - 1];
            if (nb < 0 || nb > c->ngrid) return bail(fail(MGLET_ERR_ARG, "create: bad NBRGRID"));
            c->nbr[g + 1][s] = nb;
        }
        G.gradpflag = d->gradpflag ? d->gradpflag[g] : 1;
        G.halo = 0;
        G.ip3 = o3; G.ipx = ox; G.ipy = oy; G.ipz = oz;
        o3 += (long long)G.kk * G.jj * G.ii;
        ox += G.ii; oy += G.jj; oz += G.kk;
        c->minlevel = std::min(c->minlevel, G.level);
        c->maxlevel = std::max(c->maxlevel, G.level);
        const long long key = ((long long)G.kk << 40) | ((long long)G.jj << 20) | G.ii;
        auto it = std::find(shapes.begin(), shapes.end(), key);
        G.cls = (int)(it - shapes.begin());
        if (it == shapes.end()) shapes.push_back(key);
    }
    // hierarchies: the level operators (parent, ftoc, ctof, bound_pressure,
    // bound_flow on PAR faces), tstle4 with tstle4_par, mgpoisl and the
    // stage run on them in both forms; the mixed form's inner solver is SIP
    // on every level
    if (c->minlevel != c->maxlevel && prm->form == MGLET_FORM_MIXED &&
        prm->psolver == MGLET_PSOLVER_SOR)
        return bail(fail(MGLET_ERR_UNSUPPORTED, "create: the mixed form runs SIP on every level"));
    c->uniform = shapes.size() == 1;
    c->idim3d = o3; c->idimx = ox; c->idimy = oy; c->idimz = oz;
    MG_CUDA(cudaMalloc(&c->d_grids, c->ngrid * sizeof(DevGrid)));
    MG_CUDA(copy_on(c->stream, c->d_grids, c->grids.data(), c->ngrid * sizeof(DevGrid),
                       cudaMemcpyHostToDevice));
    for (long long key : shapes) {
        HpTable t;
        if (int rc = build_hp_table(c->stream, (int)(key >> 40), (int)((key >> 20) & 0xFFFFF),
                                    (int)(key & 0xFFFFF), t))
            return bail(rc);
        c->hp.push_back(t);
    }
    for (const char* n : {"U", "V", "W", "P", "G", "DU", "DV", "DW", "BP", "SDIV", "UO", "VO",
                          "WO", "DP", "HILF", "RHS", "RES", "GSAP", "SIPLW", "SIPLS", "SIPLB",
                          "SIPLPR", "SIPUE", "SIPUN", "SIPUT"})
        if (int rc = alloc3(c, n)) return bail(rc);
    if (prm->psolver == MGLET_PSOLVER_SOR)
        if (int rc = alloc3(c, "SOR_RAP")) return bail(rc);
    const double* h1[9] = {d->x, d->y, d->z, d->dx, d->dy, d->dz, d->ddx, d->ddy, d->ddz};
    const char* n1[9] = {"X", "Y", "Z", "DX", "DY", "DZ", "DDX", "DDY", "DDZ"};
    const long long len1[3] = {ox, oy, oz};
    for (int q = 0; q < 9; ++q) {
        if (!h1[q]) return bail(fail(MGLET_ERR_ARG, "create: missing spacing array"));
        if (int rc = alloc1(c, n1[q], len1[q % 3], h1[q])) return bail(rc);
    }
    // tauwin's dds**(-cwb) for every cell width (wernerwengle_mod.F90:81),
    // taken once on the host
    for (int q = 0; q < 3; ++q) {
        std::vector<double> wv(h1[6 + q], h1[6 + q] + len1[q]);
        for (double& x : wv) x = std::pow(x, -(1.0 / 7.0));
        const char* wn[3] = {"WWX", "WWY", "WWZ"};
        if (int rc = alloc1(c, wn[q], len1[q], wv.data())) return bail(rc);
    }
    const char* rn[6] = {"RDX", "RDY", "RDZ", "RDDX", "RDDY", "RDDZ"};
    const char* sn[6] = {"DX", "DY", "DZ", "DDX", "DDY", "DDZ"};
    for (int q = 0; q < 6; ++q) {
        if (int rc = alloc1(c, rn[q], len1[q % 3], nullptr)) return bail(rc);
        k_reciprocal<<<(int)((len1[q % 3] + 255) / 256), 256, 0, c->stream>>>(c->L(rn[q]),
                                                                              c->L(sn[q]), len1[q % 3]);
        c->launches++;
    }
    for (const char* n : {"GSAW", "GSAE"}) if (int rc = alloc1(c, n, ox, nullptr)) return bail(rc);
    for (const char* n : {"GSAS", "GSAN"}) if (int rc = alloc1(c, n, oy, nullptr)) return bail(rc);
    for (const char* n : {"GSAB", "GSAT"}) if (int rc = alloc1(c, n, oz, nullptr)) return bail(rc);
    MG_CUDA(cudaMalloc(&c->d_gridred, (size_t)4 * c->ngrid * sizeof(double)));
    MG_CUDA(cudaMalloc(&c->d_bpone, (size_t)c->ngrid * sizeof(int)));
    MG_CUDA(cudaMalloc(&c->d_guni, (size_t)2 * c->ngrid * sizeof(double)));
    MG_CUDA(cudaMalloc(&c->d_scalar, 8 * sizeof(double)));
    MG_CUDA(cudaMallocHost(&c->h_scalar, 8 * sizeof(double)));
    // noib_mod.F90:45-52 (BP = 1, SDIV = 0)
    if (int rc = fill(c, c->F("BP"), 1.0)) return bail(rc);
    build_connection_table(c);
    if (int rc = bound_init(c)) return bail(rc);
    if (int rc = level_init(c)) return bail(rc);
    if (int rc = init_viscosity(c)) return bail(rc);
    if (int rc = launch_giteig(c)) return bail(rc);
    MG_CUDA(cudaStreamSynchronize(c->stream));
    int rc = prm->psolver == MGLET_PSOLVER_CLASSIC ? launch_sip_lu_classic(c) : launch_sip_lu_hp(c);
    if (rc) return bail(rc);
    if (prm->psolver == MGLET_PSOLVER_SOR) {
        k_reciprocal<<<(int)((c->idim3d + 255) / 256), 256, 0, c->stream>>>(
            c->F("SOR_RAP"), c->F("GSAP"), c->idim3d);
        c->launches++;
    }
    if (prm->form == MGLET_FORM_MIXED)
        if (int rc2 = mixed_init(c)) return bail(rc2);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "create"));
    *out = c;
    return 0;
}

int mglet_gpu_destroy(mglet_ctx* c) {
    if (!c) return 0;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    part_release(c);
    for (auto& kv : c->profd)
        for (auto& ev : kv.second.pending) {
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
    mixed_release(c);
    release_tables(c);
    contract::release_tables(c);
    for (auto& kv : c->f3) cudaFree(kv.second);
    for (auto& kv : c->f1) cudaFree(kv.second);
    for (auto& kv : c->plans) {
        cudaFree(kv.second.d_tasks);
        cudaFree(kv.second.d_bysrc);
        cudaFree(kv.second.d_srcstart);
    }
    for (HpTable& t : c->hp) { cudaFree(t.d_mip); cudaFree(t.d_idx); }
    cudaFree(c->d_grids);
    for (double* b : c->d_buf) cudaFree(b);
    cudaFree(c->d_bface);
    for (void* p : {(void*)c->gcd.seg, (void*)c->gcd.xpoli, (void*)c->gcd.xpolr,
                    (void*)c->gcd.xpolrvel, (void*)c->gcd.oldsol, (void*)c->gcd.oldsolvel,
                    (void*)c->gcd.poldsol, (void*)c->gcd.poldsolvel, (void*)c->gcd.cell,
                    (void*)c->gcd.lvstart})
        cudaFree(p);
    for (int* b : c->d_bgrids) cudaFree(b);
    for (int* b : c->d_pgrids) cudaFree(b);
    for (auto& m : c->d_plist)
        for (auto& kv : m) cudaFree(kv.second);
    for (auto& kv : c->d_children) cudaFree(kv.second);
    for (auto& kv : c->fbuf) cudaFree(kv.second);
    cudaFree(c->d_hier);
    cudaFree(c->d_ftoc_skip);
    cudaFree(c->d_pargrids);
    cudaFree(c->d_sptab);
    cudaFree(c->d_scabc_kind);
    for (void* p : {(void*)c->d_sxi, (void*)c->d_sxr, (void*)c->d_sxrv, (void*)c->d_scell0}) cudaFree(p);
    cudaFree(c->d_scabc_type);
    for (auto& kv : c->d_pftasks) cudaFree(kv.second);
    cudaFree(c->d_gridred);
    cudaFree(c->d_bpone);
    cudaFree(c->d_guni);
    cudaFree(c->d_scalar);
    if (c->h_scalar) cudaFreeHost(c->h_scalar);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return 0;
}

int64_t mglet_gpu_idim3d(const mglet_ctx* c) { return c ? c->idim3d : -1; }

int64_t mglet_gpu_kernel_launches(const mglet_ctx* c) { return c ? c->launches : -1; }

int mglet_gpu_set_field(mglet_ctx* c, const char* name, const double* host, int64_t n) {
    if (!c || !name || !host) return fail(MGLET_ERR_ARG, "set_field: null argument");
    double* p = field_ptr(c, name);
    if (!p) return fail(MGLET_ERR_NAME, std::string("set_field: unknown field ") + name);
    if (n != c->idim3d) return fail(MGLET_ERR_SIZE, "set_field: element count != idim3d");
    cudaSetDevice(c->device);
    MG_CUDA(cudaMemcpyAsync(p, host, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    if (std::strcmp(name, "G") == 0) c->g_user = true;
    if (c->prm.form == MGLET_FORM_MIXED) mixed_field_changed(c, name);
    return 0;
}

int mglet_gpu_get_field(mglet_ctx* c, const char* name, double* host, int64_t n) {
    if (!c || !name || !host) return fail(MGLET_ERR_ARG, "get_field: null argument");
    double* p = field_ptr(c, name);
    long long len = c->idim3d;
    if (!p) {
        auto it = c->f1.find(name);
        if (it == c->f1.end()) return fail(MGLET_ERR_NAME, std::string("get_field: unknown field ") + name);
        p = it->second;
        const char ax = name[std::strlen(name) - 1];
        len = ax == 'X' || ax == 'W' || ax == 'E' ? c->idimx
              : (ax == 'Y' || ax == 'S' || ax == 'N') ? c->idimy : c->idimz;
    }
    if (n != len) return fail(MGLET_ERR_SIZE, "get_field: element count mismatch");
    cudaSetDevice(c->device);
    if (c->prm.form == MGLET_FORM_MIXED) mixed_field_sync_out(c, name);
    MG_CUDA(cudaMemcpyAsync(host, p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int mglet_gpu_timeintegrate_flow(mglet_ctx* c, int32_t itstep, int32_t ittot, double timeph,
                                 double dt, int32_t irk, const mglet_rk_scheme* rk,
                                 mglet_stage_stats* stats) {
    (void)itstep; (void)ittot; (void)timeph;
    if (!c || !rk) return fail(MGLET_ERR_ARG, "timeintegrate_flow: null argument");
    cudaSetDevice(c->device);
    mglet_stage_stats tmp;
    return timeintegrate(c, dt, irk, rk, stats ? stats : &tmp);
}

int mglet_gpu_tstle4(mglet_ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "tstle4: null context");
    cudaSetDevice(c->device);
    const bool gc = c->ibtype == 1;
    return MG_PLAIN_FN(c, launch_tstle4)(c, c->F("UO"), c->F("VO"), c->F("WO"),
                                         c->F(gc ? "PWU" : "U"), c->F(gc ? "PWV" : "V"),
                                         c->F(gc ? "PWW" : "W"), c->F("U"), c->F("V"), c->F("W"),
                                         c->F("P"), c->F("G"));
}

int mglet_gpu_rkstep(mglet_ctx* c, const char* p, const char* dp, const char* rhsp, double frhs,
                     double dtfu) {
    if (!c) return fail(MGLET_ERR_ARG, "rkstep: null context");
    double *a = field_ptr(c, p), *b = field_ptr(c, dp), *r = field_ptr(c, rhsp);
    if (!a || !b || !r) return fail(MGLET_ERR_NAME, "rkstep: unknown field");
    cudaSetDevice(c->device);
    return MG_PLAIN_FN(c, launch_rkstep)(c, a, b, r, frhs, dtfu);
}

int mglet_gpu_connect(mglet_ctx* c, int32_t ilevel, int32_t layers, const char* v1,
                      const char* v2, const char* v3, const char* s1, const char* s2,
                      const char* s3, int32_t corners, int32_t normal, int32_t forward) {
    if (!c) return fail(MGLET_ERR_ARG, "connect: null context");
    const char* names[6] = {v1, v2, v3, s1, s2, s3};
    double* f[6];
    for (int q = 0; q < 6; ++q) {
        f[q] = field_ptr(c, names[q]);
        if (names[q] && !f[q]) return fail(MGLET_ERR_NAME, std::string("connect: unknown field ") + names[q]);
    }
    cudaSetDevice(c->device);
    return connect(c, ilevel, layers, f[0], f[1], f[2], f[3], f[4], f[5], corners != 0,
                   normal != 0, forward);
}

int mglet_gpu_divcal(mglet_ctx* c, const char* div, double fak) {
    if (!c) return fail(MGLET_ERR_ARG, "divcal: null context");
    double* d = field_ptr(c, div);
    if (!d) return fail(MGLET_ERR_NAME, "divcal: unknown field");
    cudaSetDevice(c->device);
    return MG_PLAIN_FN(c, launch_divcal)(c, d, c->F("U"), c->F("V"), c->F("W"), fak);
}

int mglet_gpu_laplacephi(mglet_ctx* c, const char* res, const char* phi) {
    if (!c) return fail(MGLET_ERR_ARG, "laplacephi: null context");
    double *r = field_ptr(c, res), *p = field_ptr(c, phi);
    if (!r || !p) return fail(MGLET_ERR_NAME, "laplacephi: unknown field");
    cudaSetDevice(c->device);
    if (int rc = launch_bp_ones(c)) return rc;
    return MG_PLAIN_FN(c, launch_laplacephi)(c, 0, r, p);
}

int mglet_gpu_mgpoisl(mglet_ctx* c, double dt, int32_t ittot, int32_t irk, mglet_stage_stats* st) {
    (void)ittot; (void)irk;
    if (!c) return fail(MGLET_ERR_ARG, "mgpoisl: null context");
    cudaSetDevice(c->device);
    mglet_stage_stats tmp;
    return mgpoisl(c, dt, st ? st : &tmp);
}

int mglet_gpu_bound_flow(mglet_ctx* c, int32_t ilevel) {
    if (!c) return fail(MGLET_ERR_ARG, "bound_flow: null context");
    cudaSetDevice(c->device);
    return launch_bound_flow(c, c->F("U"), c->F("V"), c->F("W"), c->F("P"), ilevel);
}

int mglet_gpu_set_hierarchy(mglet_ctx* c, const int32_t* iparent, const int32_t* position) {
    if (!c || !iparent || !position) return fail(MGLET_ERR_ARG, "set_hierarchy: null argument");
    cudaSetDevice(c->device);
    return set_hierarchy(c, iparent, position);
}

int mglet_gpu_parent(mglet_ctx* c, int32_t ilevel, const char* v1, const char* v2, const char* v3,
                     const char* s1, const char* s2, const char* s3, int32_t normal) {
    if (!c) return fail(MGLET_ERR_ARG, "parent: null context");
    if ((v1 != nullptr) != (v2 != nullptr) || (v1 != nullptr) != (v3 != nullptr))
        return fail(MGLET_ERR_ARG, "parent: give all three vector components or none");
    const char* const v[3] = {v1, v2, v3};
    const char* const s[3] = {s1, s2, s3};
    for (const char* n : {v1, v2, v3, s1, s2, s3})
        if (n && !field_ptr(c, n)) return fail(MGLET_ERR_NAME, std::string("parent: unknown field ") + n);
    cudaSetDevice(c->device);
    return launch_parent(c, ilevel, v, s, normal != 0);
}

int mglet_gpu_ftoc(mglet_ctx* c, int32_t ilevel, const char* ff, const char* fc, char flag) {
    if (!c) return fail(MGLET_ERR_ARG, "ftoc: null context");
    double *f = field_ptr(c, ff), *g = field_ptr(c, fc);
    if (!f || !g) return fail(MGLET_ERR_NAME, "ftoc: unknown field");
    if (!flag || !std::strchr("UVWPRST", flag))
        return fail(MGLET_ERR_ARG, "ftoc: flag is one of U V W P R S T");
    cudaSetDevice(c->device);
    return launch_ftoc(c, ilevel, f, g, flag);
}

int mglet_gpu_set_body_force(mglet_ctx* c, const double* fx, const double* fy, const double* fz,
                             int64_t n) {
    if (!c || !fx || !fy || !fz) return fail(MGLET_ERR_ARG, "set_body_force: null argument");
    if (c->prm.form != MGLET_FORM_PLAIN)
        return fail(MGLET_ERR_UNSUPPORTED, "set_body_force: the plain form only");
    if (n != c->idim3d) return fail(MGLET_ERR_SIZE, "set_body_force: n must equal idim3d");
    cudaSetDevice(c->device);
    const char* nm[3] = {"FBX", "FBY", "FBZ"};
    const double* h[3] = {fx, fy, fz};
    for (int q = 0; q < 3; ++q) {
        if (!c->f3.count(nm[q]))
            if (int rc = alloc3(c, nm[q])) return rc;
        MG_CUDA(copy_on(c->stream, c->F(nm[q]), h[q], (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    }
    c->bodyforce = true;
    return 0;
}

int mglet_gpu_set_scalars(mglet_ctx* c, int32_t nsca, const double* prmol, const int32_t* kayscrawford,
                          const double* source, double prturb) {
    if (!c) return fail(MGLET_ERR_ARG, "set_scalars: null context");
    cudaSetDevice(c->device);
    if (int rc = set_scalars(c, nsca, prmol, kayscrawford, source, prturb)) return rc;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int mglet_gpu_timeintegrate_scalar(mglet_ctx* c, double dt, int32_t irk, const mglet_rk_scheme* rk) {
    if (!c || !rk) return fail(MGLET_ERR_ARG, "timeintegrate_scalar: null argument");
    cudaSetDevice(c->device);
    if (int rc = hierarchy_ready(c)) return rc;
    if (int rc = timeintegrate_scalar(c, dt, irk, rk)) return rc;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int mglet_gpu_set_scalar_bc(mglet_ctx* c, int32_t igrid, int32_t iface, int32_t kind, const int32_t* types) {
    if (!c) return fail(MGLET_ERR_ARG, "set_scalar_bc: null context");
    cudaSetDevice(c->device);
    return set_scalar_bc(c, igrid, iface, kind, types);
}

int mglet_gpu_add_scalar_source(mglet_ctx* c, int32_t isca, const char* field, double value) {
    if (!c) return fail(MGLET_ERR_ARG, "add_scalar_source: null context");
    return add_scalar_source(c, isca, field, value);
}

int mglet_gpu_set_buoyancy(mglet_ctx* c, const double* gravity, double beta, int32_t iscalar) {
    if (!c || !gravity || iscalar < 1 || iscalar > (int)c->sca.size())
        return fail(MGLET_ERR_ARG, "set_buoyancy: gravity and a scalar 1..nsca");
    if (c->prm.form != MGLET_FORM_PLAIN) return fail(MGLET_ERR_UNSUPPORTED, "set_buoyancy: the plain form only");
    for (int q = 0; q < 3; ++q) c->gravity[q] = gravity[q];
    c->beta = beta;
    c->buoyancy_scalar = iscalar;
    c->buoyancy = true;
    return 0;
}

int mglet_gpu_set_coriolis(mglet_ctx* c, const double* omega) {
    if (!c || !omega) return fail(MGLET_ERR_ARG, "set_coriolis: null argument");
    if (c->prm.form != MGLET_FORM_PLAIN) return fail(MGLET_ERR_UNSUPPORTED, "set_coriolis: the plain form only");
    for (int q = 0; q < 3; ++q) c->omega[q] = omega[q];
    c->coriolis = true;
    return 0;
}

int mglet_gpu_set_lesmodel(mglet_ctx* c, int32_t model, double cm) {
    if (!c) return fail(MGLET_ERR_ARG, "set_lesmodel: null context");
    cudaSetDevice(c->device);
    if (int rc = set_lesmodel(c, model, cm)) return rc;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int mglet_gpu_adjoint_rk_stage(mglet_ctx* c, int32_t irk, double dt, const mglet_rk_scheme* rk) {
    if (!c || !rk) return fail(MGLET_ERR_ARG, "adjoint_rk_stage: null argument");
    cudaSetDevice(c->device);
    if (int rc = adjoint_ready(c)) return rc;
    if (int rc = adjoint_stage(c, dt, irk, rk)) return rc;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int mglet_gpu_energy_gradient(mglet_ctx* c, int32_t nsteps, int32_t ncheck, double dt,
                              const mglet_rk_scheme* rk, double* energy) {
    if (!c) return fail(MGLET_ERR_ARG, "energy_gradient: null context");
    cudaSetDevice(c->device);
    return energy_gradient(c, nsteps, ncheck, dt, rk, energy);
}

int mglet_gpu_par_ftoc_norm(mglet_ctx* c, int32_t ilevel, const char* v1, const char* v2,
                            const char* v3, int32_t sum) {
    if (!c) return fail(MGLET_ERR_ARG, "par_ftoc_norm: null context");
    double *u = field_ptr(c, v1), *v = field_ptr(c, v2), *w = field_ptr(c, v3);
    if (!u || !v || !w) return fail(MGLET_ERR_NAME, "par_ftoc_norm: unknown field");
    cudaSetDevice(c->device);
    return launch_par_ftoc_norm(c, ilevel, u, v, w, sum != 0);
}

int mglet_gpu_ftoc_multiple(mglet_ctx* c, int32_t ilevel, const char* v1, const char* v2,
                            const char* v3, const char* s1, const char* s2, const char* s3) {
    if (!c) return fail(MGLET_ERR_ARG, "ftoc: null context");
    const char* n[6] = {v1, v2, v3, s1, s2, s3};
    const char fl[6] = {'U', 'V', 'W', 'P', 'P', 'P'};
    for (int q = 0; q < 6; ++q)
        if (n[q] && !field_ptr(c, n[q])) return fail(MGLET_ERR_NAME, "ftoc: unknown field");
    cudaSetDevice(c->device);
    for (int q = 0; q < 6; ++q)
        if (n[q])
            if (int rc = launch_ftoc(c, ilevel, field_ptr(c, n[q]), field_ptr(c, n[q]), fl[q])) return rc;
    return 0;
}

int mglet_gpu_ctof(mglet_ctx* c, int32_t ilevel, const char* ff, const char* fc) {
    if (!c) return fail(MGLET_ERR_ARG, "ctof: null context");
    double *f = field_ptr(c, ff), *g = field_ptr(c, fc);
    if (!f || !g) return fail(MGLET_ERR_NAME, "ctof: unknown field");
    cudaSetDevice(c->device);
    return launch_ctof(c, ilevel, f, g);
}

int mglet_gpu_bound_pressure(mglet_ctx* c, int32_t ilevel, const char* dp, int32_t with_bp) {
    if (!c) return fail(MGLET_ERR_ARG, "bound_pressure: null context");
    double* p = field_ptr(c, dp);
    if (!p) return fail(MGLET_ERR_NAME, "bound_pressure: unknown field");
    cudaSetDevice(c->device);
    double* b = field_buffer(c, dp);
    if (!b) return fail(MGLET_ERR_CUDA, "bound_pressure: buffer allocation");
    return launch_bound_pressure(c, ilevel, p, b, with_bp != 0);
}

int mglet_gpu_get_buffer(mglet_ctx* c, const char* name, int32_t igrid, int32_t iface, double* host,
                         int64_t n) {
    if (!c || !name || !host || igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6)
        return fail(MGLET_ERR_ARG, "get_buffer: bad arguments");
    const DevGrid& G = c->grids[igrid - 1];
    const long long sz[3] = {(long long)G.kk * G.jj, (long long)G.kk * G.ii, (long long)G.jj * G.ii};
    if (n != sz[(iface - 1) / 2]) return fail(MGLET_ERR_SIZE, "get_buffer: wrong plane size");
    if (!field_ptr(c, name)) return fail(MGLET_ERR_NAME, "get_buffer: unknown field");
    cudaSetDevice(c->device);
    double* b = field_buffer(c, name);
    if (!b) return fail(MGLET_ERR_CUDA, "get_buffer: buffer allocation");
    MG_CUDA(copy_on(c->stream, host, b + c->bface[6 * (igrid - 1) + iface - 1].off,
                    (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int mglet_gpu_set_buffer(mglet_ctx* c, const char* name, int32_t igrid, int32_t iface,
                         const double* host, int64_t n) {
    if (!c || !name || !host || igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6)
        return fail(MGLET_ERR_ARG, "set_buffer: bad arguments");
    const DevGrid& G = c->grids[igrid - 1];
    const long long sz[3] = {(long long)G.kk * G.jj, (long long)G.kk * G.ii, (long long)G.jj * G.ii};
    if (n != sz[(iface - 1) / 2]) return fail(MGLET_ERR_SIZE, "set_buffer: wrong plane size");
    if (!field_ptr(c, name)) return fail(MGLET_ERR_NAME, "set_buffer: unknown field");
    cudaSetDevice(c->device);
    double* b = field_buffer(c, name);
    if (!b) return fail(MGLET_ERR_CUDA, "set_buffer: buffer allocation");
    MG_CUDA(copy_on(c->stream, b + c->bface[6 * (igrid - 1) + iface - 1].off, host,
                    (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    return 0;
}

int mglet_gpu_set_bc_real(mglet_ctx* c, int32_t igrid, int32_t iface, double value) {
    if (!c || igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6)
        return fail(MGLET_ERR_ARG, "set_bc_real: bad arguments");
    BFace& b = c->bface[6 * (igrid - 1) + iface - 1];
    b.pinf = value;
    cudaSetDevice(c->device);
    MG_CUDA(copy_on(c->stream, c->d_bface + 6 * (igrid - 1) + iface - 1, &b, sizeof(BFace),
                    cudaMemcpyHostToDevice));
    return 0;
}

int mglet_gpu_set_stencils(mglet_ctx* c, int32_t igrid, int32_t comp, int32_t ncells,
                           const int64_t* xpoli, int64_t nxi, const double* xpolr, int64_t nxr,
                           const double* xpolrvel, int64_t nxrv) {
    if (!c || igrid < 1 || igrid > c->ngrid || comp < 1 || comp > 4 || ncells < 0 || nxi < 0 ||
        nxr < 0 || (nxi > 0 && !xpoli) || (nxr > 0 && !xpolr))
        return fail(MGLET_ERR_ARG, "set_stencils: bad arguments");
    if (c->gch.empty()) c->gch.resize(c->ngrid);
    GcHostList& L = c->gch[igrid - 1];
    const int q = comp - 1;
    const DevGrid& G = c->grids[igrid - 1];
    const long long npts = (long long)G.kk * G.jj * G.ii;
    if (comp == 4) {
        if (nxi != 2LL * ncells || nxr != 7LL * ncells)
            return fail(MGLET_ERR_SIZE, "set_stencils: flux list sizes");
        for (long long e = 1; e < nxi; e += 2)
            if (xpoli[e] < 1 + (long long)G.kk * G.jj || xpoli[e] > npts)
                return fail(MGLET_ERR_ARG, "set_stencils: flux cell outside the grid");
    } else {
        if (nxrv != nxr || (nxrv > 0 && !xpolrvel))
            return fail(MGLET_ERR_SIZE, "set_stencils: xpolrvel must match xpolr");
        // walk the list once: every position inside the grid, sizes consistent
        long long pi = 0, pr = 0;
        for (int cell = 0; cell < ncells; ++cell) {
            if (pi + 2 > nxi) return fail(MGLET_ERR_SIZE, "set_stencils: xpoli too short");
            const long long ic = xpoli[pi++], n = xpoli[pi++];
            if (ic < 1 || ic > npts || n < 0 || pi + n > nxi || pr + n + 1 > nxr)
                return fail(MGLET_ERR_ARG, "set_stencils: inconsistent list");
            for (long long e = 0; e < n; ++e)
                if (xpoli[pi + e] < 1 || xpoli[pi + e] > npts)
                    return fail(MGLET_ERR_ARG, "set_stencils: stencil cell outside the grid");
            pi += n;
            pr += n + 1;
        }
        if (pi != nxi || pr != nxr) return fail(MGLET_ERR_SIZE, "set_stencils: list lengths");
        L.xv[q].assign(xpolrvel, xpolrvel + nxrv);
    }
    L.n[q] = ncells;
    L.xi[q].assign(xpoli, xpoli + nxi);
    L.xr[q].assign(xpolr, xpolr + nxr);
    return 0;
}

int mglet_gpu_set_ghostcell(mglet_ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "set_ghostcell: null context");
    cudaSetDevice(c->device);
    if (c->minlevel != c->maxlevel)   // setsdivfield restricts SDIV level by level
        if (int rc = hierarchy_ready(c)) return rc;
    if (c->gch.empty()) c->gch.resize(c->ngrid);
    c->ibtype = 1;
    if (int rc = launch_giteig(c)) return rc;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    int rc = c->prm.psolver == MGLET_PSOLVER_CLASSIC ? launch_sip_lu_classic(c) : launch_sip_lu_hp(c);
    if (rc) return rc;
    if (c->prm.psolver == MGLET_PSOLVER_SOR)
        return fail(MGLET_ERR_UNSUPPORTED, "set_ghostcell: SOR with blocked cells");
    if ((rc = gc_upload(c))) return rc;
    c->gc_saved[0] = c->gc_saved[1] = false;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    if (c->prm.form == MGLET_FORM_MIXED) return mixed_ghostcell(c);
    // scalars set before the blocking: their BT from BP now
    return scalar_blockbt(c);
}

int mglet_gpu_set_scastencils(mglet_ctx* c, int32_t igrid, int32_t ncells, const int64_t* xpoli,
                              const double* xpolr, const double* xpolrvel) {
    if (!c) return fail(MGLET_ERR_ARG, "set_scastencils: null context");
    cudaSetDevice(c->device);
    return set_scastencils(c, igrid, ncells, xpoli, xpolr, xpolrvel);
}

int mglet_gpu_set_scalar_geometry(mglet_ctx* c, int32_t isca, int32_t nbody, const int32_t* flag,
                                  const double* value) {
    if (!c) return fail(MGLET_ERR_ARG, "set_scalar_geometry: null context");
    return set_scalar_geometry(c, isca, nbody, flag, value);
}

static int gc_ready(Ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "ghost-cell call: null context");
    if (c->ibtype != 1) return fail(MGLET_ERR_ARG, "ghost-cell call before set_ghostcell");
    cudaSetDevice(c->device);
    return 0;
}

int mglet_gpu_setibvalues(mglet_ctx* c) {
    if (int rc = gc_ready(c)) return rc;
    return gc_setibvalues(c, c->F("U"), c->F("V"), c->F("W"));
}

int mglet_gpu_getibvalues(mglet_ctx* c) {
    if (int rc = gc_ready(c)) return rc;
    return launch_gc_mode(c, 'R', c->F("U"), c->F("V"), c->F("W"));
}

int mglet_gpu_setpointvalues(mglet_ctx* c, int32_t comp_new) {
    if (int rc = gc_ready(c)) return rc;
    return gc_setpointvalues(c, comp_new != 0);
}

int mglet_gpu_maskbp(mglet_ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "maskbp: null context");
    cudaSetDevice(c->device);
    return launch_maskbp(c, c->F("U"), c->F("V"), c->F("W"), c->F("P"));
}

int mglet_gpu_itinfo(mglet_ctx* c, double dt, mglet_itinfo* out) {
    if (!c || !out) return fail(MGLET_ERR_ARG, "itinfo: null argument");
    cudaSetDevice(c->device);
    if (int rc = launch_itinfo(c, dt)) return rc;
    std::vector<double> red((size_t)4 * c->ngrid);
    MG_CUDA(cudaMemcpyAsync(red.data(), c->d_gridred, red.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    double cm = 0.0, dm = 0.0, es = 0.0, vol = 0.0;
    bool bad = false;
    for (int g = 0; g < c->ngrid; ++g) {
        if (c->grids[g].halo) continue;   // another rank's grid
        const double gc = red[4 * g], gd = red[4 * g + 1];
        const double ge = red[4 * g + 2] / red[4 * g + 3], gv = red[4 * g + 3];
        cm = std::max(cm, gc);
        dm = std::max(dm, gd);
        es = (vol + gv > 0.0) ? (es * vol + ge * gv) / (vol + gv) : 0.0;
        vol = vol + gv;
        if (!std::isfinite(gc) || !std::isfinite(gd) || !std::isfinite(ge)) bad = true;
    }
    if (c->part) {
        // the maxima and the volume-weighted energy over all ranks
        double mx[3] = {cm, dm, bad ? 1.0 : 0.0}, sm[2] = {es * vol, vol};
        if (int rc = part_allreduce(c, mx, 3, 1)) return rc;
        if (int rc = part_allreduce(c, sm, 2, 2)) return rc;
        cm = mx[0];
        dm = mx[1];
        bad = mx[2] != 0.0;
        es = sm[1] > 0.0 ? sm[0] / sm[1] : 0.0;
    }
    out->cflmax = cm;
    out->divmax = dm;
    out->energy = es;
    out->exploded = bad ? 1 : 0;
    out->reserved = 0;
    return bad ? fail(MGLET_ERR_EXPLODED, "itinfo: NaN/Inf detected (exploded)") : 0;
}

void* mglet_gpu_stream(const mglet_ctx* c) { return c ? (void*)c->stream : nullptr; }

int mglet_gpu_profile(mglet_ctx* c, int32_t enable) {
    if (!c) return fail(MGLET_ERR_ARG, "profile: null context");
    c->prof = enable != 0;
    return 0;
}

static int prof_settle(mglet_ctx* c) {
    MG_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& kv : c->profd) {
        for (auto& ev : kv.second.pending) {
            float ms = 0.f;
            MG_CUDA(cudaEventElapsedTime(&ms, ev.first, ev.second));
            kv.second.total_ms += ms;
            kv.second.launches += 1;
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
        kv.second.pending.clear();
    }
    return 0;
}

int mglet_gpu_profile_get(mglet_ctx* c, const char* kernel, double* total_ms, int64_t* launches) {
    if (!c || !kernel || !total_ms || !launches) return fail(MGLET_ERR_ARG, "profile_get: null argument");
    if (int rc = prof_settle(c)) return rc;
    auto it = c->profd.find(kernel);
    if (it == c->profd.end()) {
        *total_ms = 0.0;
        *launches = 0;
        return 0;
    }
    *total_ms = it->second.total_ms;
    *launches = it->second.launches;
    it->second.total_ms = 0.0;
    it->second.launches = 0;
    return 0;
}

int mglet_gpu_profile_names(mglet_ctx* c, char* buf, int64_t buflen) {
    if (!c || !buf || buflen <= 0) return fail(MGLET_ERR_ARG, "profile_names: bad buffer");
    if (int rc = prof_settle(c)) return rc;
    std::string s;
    for (auto& kv : c->profd) {
        if (!s.empty()) s += ",";
        s += kv.first;
    }
    if ((int64_t)s.size() + 1 > buflen) return fail(MGLET_ERR_SIZE, "profile_names: buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return 0;
}

int mglet_gpu_set_partition(mglet_ctx* c, const int32_t* halo, int32_t nsend, const int32_t* send,
                            int32_t nrecv, const int32_t* recv, mglet_exchange_fn fn, void* user) {
    if (!c) return fail(MGLET_ERR_ARG, "set_partition: null context");
    cudaSetDevice(c->device);
    return set_partition(c, halo, nsend, send, nrecv, recv, fn, user);
}

int mglet_gpu_tuning(mglet_ctx* c, char* buf, int64_t buflen) {
    if (!c || !buf || buflen <= 0) return fail(MGLET_ERR_ARG, "tuning: bad buffer");
    const std::string s = mixed_tuning(c);
    if ((int64_t)s.size() + 1 > buflen) return fail(MGLET_ERR_SIZE, "tuning: buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return 0;
}

int mglet_gpu_test_wait_timeout(mglet_ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "test_wait_timeout: null context");
    return mixed_test_wait_timeout(c);
}

int mglet_gpu_test_barrier_timeout(mglet_ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "test_barrier_timeout: null context");
    return mixed_test_barrier_timeout(c);
}

int mglet_gpu_force_variant(mglet_ctx* c, const char* kernel, int32_t variant) {
    if (!c || !kernel) return fail(MGLET_ERR_ARG, "force_variant: null argument");
    return mixed_force_variant(c, kernel, variant);
}

int mglet_gpu_synchronize(mglet_ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "synchronize: null context");
    cudaSetDevice(c->device);
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

}  // extern "C"
