// mglet_oracle.cpp -- CPU restatement of MGLET-base's Runge-Kutta stage.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// it.  The product path never links, loads or calls it.
//
// What it restates (FP64 build of the reference, -DMGLET_REAL64=ON), loop by
// loop and in the reference's operation order, compiled with
// -ffp-contract=off so no FMA contraction changes the rounding:
//   src/flow/timeintegration_mod.F90:22-142   timeintegrate_flow (noib)
//   src/core/rungekutta_mod.F90:70-333        RK coefficients, rkstep
//   src/flow/tstle4_mod.F90:13-529            tstle4 kon / diff / gradp
//   src/ib/noib_mod.F90:81-354                giteig, divcal
//   src/flow/sip_hyperplane_mod.F90:22-569    hyperplane SIP init/LU/iter
//   src/flow/sip_classic_mod.F90:17-198       classic SIP
//   src/flow/sor_mod.F90:18-203               red-black SOR
//   src/flow/laplacephi_mod.F90:134-165       laplacephi
//   src/flow/pressuresolver_mod.F90:160-908   mgpoisl, mgpoisit, sip,
//                                             maxabscal, rescal, mgpcorr,
//                                             accumulate_pcorr
//   src/core/connect/connect_core_mod.F90     connection table, box extents
//   src/core/connect/connect2_mod.F90:839-998 connect_self
//   src/flow/timeintegration_mod.F90:306-452  compcflmax, compdivmax, enerfg
//
// Parity status: the reference is Fortran and cannot be compiled here (no
// Fortran compiler, MPI or HDF5), and its own tests hold no golden field
// vectors.  This restatement is therefore pinned only by known-answer
// checks (analytic Taylor-Green decay, discrete Fourier eigenvalues of the
// Poisson operator, kinetic-energy conservation of the skew-symmetric
// convection, SIP hyperplane self-checks, connect message sizes, RK order):
// "parity unpinned" against reference outputs.
//
// Single-rank, single- or multi-grid, one level, ib type "noib", CON/CO1
// faces; other boundary types are rejected with MGLET_ERR_UNSUPPORTED.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <array>
#include <cstring>
#include <limits>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mglet_gpu.h"

namespace {

// Fortran default-kind (REAL32) literals widened to REAL64, as a REAL64 build
// of the reference evaluates them (sip_hyperplane_mod.F90:123,202).
const double kAlfa = (double)0.92f;
const double kTiny = (double)1.0e-20f;

struct Grid {
    int kk, jj, ii;
    int level;
    int bc[7];        // 1..6
    int nbr[27];      // 1..26
    int gradpflag;
    int64_t ip3;      // 0-based element offset of the 3-D slab
    int64_t ipx, ipy, ipz;   // 0-based; view pointers use base + ipx - 1 for 1-based i
    int halo = 0;     // 1: read-only copy of a grid another rank owns
};

struct Conn {         // one row of sendconns (single rank: send == recv)
    int recvgrid, sendgrid, recvface, sendface;
};

// facelist(4, 26), facenbr(26), rescue_dir(7, 26), rescue_nbr(7, 26) of
// src/core/connect/connect_core_mod.F90:38-159.
const int facelist[27][4] = {
    {0, 0, 0, 0},
    {1, 1, 0, 0}, {1, 2, 0, 0}, {1, 3, 0, 0}, {1, 4, 0, 0}, {1, 5, 0, 0}, {1, 6, 0, 0},
    {2, 1, 3, 0}, {2, 1, 4, 0}, {2, 1, 5, 0}, {2, 1, 6, 0}, {2, 2, 3, 0}, {2, 2, 4, 0},
    {2, 2, 5, 0}, {2, 2, 6, 0}, {2, 3, 5, 0}, {2, 3, 6, 0}, {2, 4, 5, 0}, {2, 4, 6, 0},
    {3, 1, 3, 5}, {3, 1, 3, 6}, {3, 1, 4, 5}, {3, 1, 4, 6}, {3, 2, 3, 5}, {3, 2, 3, 6},
    {3, 2, 4, 5}, {3, 2, 4, 6}};
const int facenbr[27] = {0, 2, 1, 4, 3, 6, 5, 12, 11, 14, 13, 8, 7, 10, 9,
                         18, 17, 16, 15, 26, 25, 24, 23, 22, 21, 20, 19};
const int rescue_dir[27][7] = {
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
const int rescue_nbr[27][7] = {
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

inline bool is_con(int t) { return t == MGLET_BC_CON || t == MGLET_BC_CO1; }

// Ghost-cell stencil lists of one velocity component of one grid
// (gc_flowstencils_mod.F90:37-100): per ghost cell xpoli holds
// [intcell, n, stcell x n] (1-based positions in the grid's flat array) and
// xpolr / xpolrvel [coeff x n, const]; oldsol / poldsol are the save buffers
// of the 'S'/'R' and 'Z'/'Y' modes.
struct GcList {
    std::vector<int64_t> xpoli;
    std::vector<double> xpolr, xpolrvel;
    int ncells = 0;
    std::vector<double> oldsol, oldsolvel;
    std::vector<int64_t> poldsol, poldsolvel;
};
// Flux-correction list of one grid: per cell [foundnr, intcell] and
// [ax1, ax2, ay1, ay2, az1, az2, acoeff].
struct GcFlux {
    std::vector<int64_t> fxpoli;
    std::vector<double> fxpolr;
    int ncells = 0;
};

struct Ctx {
    std::vector<Grid> g;   // 1-based (g[0] unused)
    int ngrid = 0;
    int minlevel = 0, maxlevel = 0;
    int64_t idim3d = 0, idimx = 0, idimy = 0, idimz = 0;
    mglet_flow_params prm{};
    int ilesmodel = 0;
    std::map<std::string, std::vector<double>> f3;   // 3-D fields
    std::map<std::string, std::vector<double>> f1;   // 1-D fields
    std::vector<int64_t> mip, idxsip;                // SIP_MIP_HP, SIP_IDX_HP
    std::vector<Conn> conns;
    // boundary buffers of U, V, W (field_t%get_buffer): per grid and face a
    // (kk,jj), (kk,ii) or (jj,ii) plane, column-major; bufoff[6*(g-1)+f-1]
    std::vector<double> bufU, bufV, bufW;
    std::vector<int64_t> bufoff;
    std::vector<double> pinf;    // OP1 real parameter per grid and face (nreal = 1)
    std::vector<int> npinf;      // 0: no parameter (pinf = 0), 1: pinf given
    int ibtype = 0;              // 0: NONE (noib), 1: GHOSTCELL
    bool bodyforce = false;      // FBX, FBY, FBZ added in tstle4
    bool g_user = false;         // G set by the caller: set_hierarchy keeps it
    // scalars (scacore_mod.F90): T<n> and DT<n>, their molecular Prandtl
    // number, the Kays/Crawford switch and a constant source
    struct ScalarDef {
        std::string name;
        double prmol = 1.0;
        int kayscrawford = 0;
        // the scalar's sources in order (sca%sources): an empty field name
        // is sourceterm_const, else sourceterm_field of that field
        std::vector<std::pair<std::string, double>> sources;
        // per body of the ghost-cell IB (sca%geometries): flag 0 fixed
        // value, 1 fixed flux, and the value
        std::vector<int> geo_flag;
        std::vector<double> geo_value;
    };
    std::vector<ScalarDef> sca;
    double prturb = 1.0;
    // boussinesqterm_mod.F90 / coriolisterm_mod.F90 parameters
    // scalar boundary conditions beside a face's flow condition: kind 1 SWA
    // (wall), 2 SIO (in/outflow), per scalar 0 fixed value, 1 fixed flux
    std::vector<int> scabc_kind, scabc_type;
    bool buoyancy = false, coriolis = false;
    double gravity[3] = {0.0, 0.0, 0.0}, beta = 0.0, omega[3] = {0.0, 0.0, 0.0};
    int buoyancy_scalar = 1;
    double cm = 0.0;             // LES model constant
    std::vector<std::array<GcList, 3>> gcl;   // [grid][component], 1-based grids
    // scalar ghost-cell lists (gc_scastencils_mod.F90:10-16), 1-based grids:
    // per cell 9 integers {intcell, body, nstencils, six stencil cells} and
    // 8 reals {areabyvol, six coefficients, acoeffvel}
    struct ScaList {
        int ncells = 0;
        std::vector<int64_t> xpoli;
        std::vector<double> xpolr, xpolrvel;
    };
    std::vector<ScaList> scal;
    std::vector<GcFlux> gcf;
    // grid hierarchy (gridinfo%iparent and i/j/kposition, grids_mod.F90):
    // iparent[g] 1-based (0 = none), pos[g] = (iposition, jposition,
    // kposition) of the fine grid in its parent; boundary buffers of fields
    // other than U, V, W (parent fills them for P, DP, HILF, ...)
    std::vector<int> iparent;
    std::vector<std::array<int, 3>> pos;
    std::map<std::string, std::vector<double>> bufx;

    // grid partition over ranks (the receive half of connect and the
    // MPI_Allreduce of the reference, caller-provided): per peer the boxes
    // sent from owned grids and received into halo copies, [g, k0, k1, j0,
    // j1, i0, i1] rows
    mglet_exchange_fn xfn = nullptr;
    void* xuser = nullptr;
    std::vector<int> peers;
    std::vector<std::vector<std::array<int, 7>>> xsend, xrecv;

    double* F(const char* n) { return f3.at(n).data(); }
    double* L(const char* n) { return f1.at(n).data(); }
};

std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

// ---------------------------------------------------------------------------
// Index helpers: Fortran 1-based (k, j, i) into a grid slab of (kk, jj, ii).
#define IX(k, j, i) ((int64_t)((i) - 1) * kk * jj + (int64_t)((j) - 1) * kk + ((k) - 1))

// ---------------------------------------------------------------------------
// connect_core_mod.F90:373-433 get_nbrs
void get_nbrs(const Ctx& c, int iface, const int* neighbours, int& nbrgrid, int& nbrface) {
    nbrgrid = 0;
    nbrface = 0;
    for (int i = 0; i < 7; ++i) {
        int dir = rescue_dir[iface][i];
        if (dir == 0) break;
        if (neighbours[dir] > 0) {
            nbrgrid = neighbours[dir];
            nbrface = rescue_nbr[iface][i];
            if (nbrface > 18) {
                int t1 = c.g[nbrgrid].bc[facelist[nbrface][1]];
                int t2 = c.g[nbrgrid].bc[facelist[nbrface][2]];
                int t3 = c.g[nbrgrid].bc[facelist[nbrface][3]];
                if (!is_con(t1) && !is_con(t2) && !is_con(t3)) {
                    nbrgrid = 0;
                    nbrface = 0;
                    continue;
                }
            }
            break;
        }
    }
}

// connect_core_mod.F90:167-370 init_connect_core (single rank: the
// Alltoallv leaves sendconns identical to recvconns)
void init_connect_core(Ctx& c) {
    c.conns.clear();
    for (int igrid = 1; igrid <= c.ngrid; ++igrid) {
        const Grid& G = c.g[igrid];
        for (int iface = 1; iface <= 6; ++iface) {
            if (is_con(G.bc[iface])) {
                int ng, nf;
                get_nbrs(c, iface, G.nbr, ng, nf);
                if (ng == 0) continue;
                c.conns.push_back({igrid, ng, iface, nf});
            }
        }
        for (int iface = 7; iface <= 18; ++iface) {
            int t1 = G.bc[facelist[iface][1]], t2 = G.bc[facelist[iface][2]];
            if (is_con(t1) || is_con(t2)) {
                int ng, nf;
                get_nbrs(c, iface, G.nbr, ng, nf);
                if (ng == 0) continue;
                c.conns.push_back({igrid, ng, iface, nf});
            }
        }
        for (int iface = 19; iface <= 26; ++iface) {
            int t1 = G.bc[facelist[iface][1]], t2 = G.bc[facelist[iface][2]],
                t3 = G.bc[facelist[iface][3]];
            if (is_con(t1) || is_con(t2) || is_con(t3)) {
                int ng, nf;
                get_nbrs(c, iface, G.nbr, ng, nf);
                if (ng == 0) continue;
                c.conns.push_back({igrid, ng, iface, nf});
            }
        }
    }
}

// connect_core_mod.F90:488-572 start_and_stop_face
void start_and_stop_face(const Grid& G, int iface, int& is, int& ie, int& js, int& je,
                         int& ks, int& ke, int nplane, bool nghost) {
    switch (iface) {
        case 1: is = 3 - nplane; ie = 2; break;
        case 2: is = G.ii - 1; ie = G.ii - (2 - nplane); break;
        case 3: js = 3 - nplane; je = 2; break;
        case 4: js = G.jj - 1; je = G.jj - (2 - nplane); break;
        case 5: ks = 3 - nplane; ke = 2; break;
        case 6: ks = G.kk - 1; ke = G.kk - (2 - nplane); break;
    }
    if (nghost) {   // flag /= 'Y' and nghost present
        switch (iface) {
            case 1: is += nplane; ie += nplane; break;
            case 2: is -= nplane; ie -= nplane; break;
            case 3: js += nplane; je += nplane; break;
            case 4: js -= nplane; je -= nplane; break;
            case 5: ks += nplane; ke += nplane; break;
            case 6: ks -= nplane; ke -= nplane; break;
        }
    }
}

// connect_core_mod.F90:454-485 start_and_stop
void start_and_stop(const Grid& G, int iface, int& is, int& ie, int& js, int& je, int& ks,
                    int& ke, int nplane, bool nghost) {
    is = 3; ie = G.ii - 2;
    js = 3; je = G.jj - 2;
    ks = 3; ke = G.kk - 2;
    for (int i = 1; i <= facelist[iface][0]; ++i)
        start_and_stop_face(G, facelist[iface][i], is, ie, js, je, ks, ke, nplane, nghost);
}

// connect_core_mod.F90:575-602 corr_start_stop
void corr_start_stop(const Grid& G, int fsend, int frecv, int& is, int& ie, int& js, int& je,
                     int& ks, int& ke, int nplane) {
    if (frecv <= 6) return;
    for (int i = 1; i <= facelist[fsend][0]; ++i)
        for (int j = 1; j <= facelist[frecv][0]; ++j)
            if (facelist[fsend][i] == facelist[frecv][j])
                start_and_stop_face(G, facelist[fsend][i], is, ie, js, je, ks, ke, nplane, false);
}

// connect_core_mod.F90:640-682 decide (geometry flag never set on this path)
bool decide(const Ctx& c, const Conn& cn, bool vertices, int fwd, int minl, int maxl) {
    bool ex = true;
    int lvl = c.g[cn.recvgrid].level;
    if (lvl > maxl || lvl < minl) ex = false;
    if (!vertices && cn.recvface > 6) ex = false;
    if (fwd == 1 && (cn.recvface == 2 || cn.recvface == 4 || cn.recvface == 6)) ex = false;
    else if (fwd == -1 && (cn.recvface == 1 || cn.recvface == 3 || cn.recvface == 5)) ex = false;
    return ex;
}

// connect2_mod.F90:947-995 connect_self_single
int64_t connect_self_single(Ctx& c, double* arr, int sg, int dg, int is, int js, int ks,
                            int isd, int ied, int jsd, int jed, int ksd, int ked) {
    const Grid& S = c.g[sg];
    const Grid& D = c.g[dg];
    int koff = ks - ksd, joff = js - jsd, ioff = is - isd;
    double* src = arr + S.ip3;
    double* dst = arr + D.ip3;
    int64_t n = 0;
    for (int i = isd; i <= ied; ++i)
        for (int j = jsd; j <= jed; ++j)
            for (int k = ksd; k <= ked; ++k) {
                int64_t di = (int64_t)(i - 1) * D.kk * D.jj + (int64_t)(j - 1) * D.kk + (k - 1);
                int64_t si = (int64_t)(i + ioff - 1) * S.kk * S.jj +
                             (int64_t)(j + joff - 1) * S.kk + (k + koff - 1);
                dst[di] = src[si];
                ++n;
            }
    return n;
}

// connect2_mod.F90:75-139,208-402,481-520,839-944: connect / conn1 for one
// rank (all connections are self connections).  Returns copied points.
// Boxes of one peer, field after field, each box k fastest, then j, then i.
void part_pack(Ctx& c, const std::vector<std::array<int, 7>>& boxes, double* const* flds, int nf,
               std::vector<double>& buf, bool unpack) {
    size_t o = 0;
    for (int q = 0; q < nf; ++q)
        for (const auto& b : boxes) {
            const Grid& G = c.g[b[0]];
            const int kk = G.kk, jj = G.jj;
            double* a = flds[q] + G.ip3;
            for (int i = b[5]; i <= b[6]; ++i)
                for (int j = b[3]; j <= b[4]; ++j)
                    for (int k = b[1]; k <= b[2]; ++k) {
                        if (unpack) a[IX(k, j, i)] = buf[o++];
                        else buf[o++] = a[IX(k, j, i)];
                    }
        }
}

// halo copies of the present fields refreshed from their owners
int part_exchange(Ctx& c, double* v1, double* v2, double* v3, double* s1, double* s2, double* s3) {
    if (!c.xfn) return 0;
    double* all[6] = {v1, v2, v3, s1, s2, s3};
    double* flds[6];
    int nf = 0;
    for (double* a : all)
        if (a) flds[nf++] = a;
    const int np = (int)c.peers.size();
    std::vector<std::vector<double>> sb(np), rb(np);
    std::vector<double*> sp(np), rp(np);
    std::vector<int64_t> sn(np), rn(np);
    for (int q = 0; q < np; ++q) {
        size_t ns = 0, nr = 0;
        for (const auto& b : c.xsend[q]) ns += (size_t)(b[2] - b[1] + 1) * (b[4] - b[3] + 1) * (b[6] - b[5] + 1);
        for (const auto& b : c.xrecv[q]) nr += (size_t)(b[2] - b[1] + 1) * (b[4] - b[3] + 1) * (b[6] - b[5] + 1);
        sb[q].resize(ns * nf);
        rb[q].resize(nr * nf);
        part_pack(c, c.xsend[q], flds, nf, sb[q], false);
        sp[q] = sb[q].data();
        rp[q] = rb[q].data();
        sn[q] = (int64_t)sb[q].size();
        rn[q] = (int64_t)rb[q].size();
    }
    if (np && c.xfn(c.xuser, 0, np, c.peers.data(), sp.data(), sn.data(), rp.data(), rn.data()))
        return fail(MGLET_ERR_ARG, "partition: the exchange function failed");
    for (int q = 0; q < np; ++q) part_pack(c, c.xrecv[q], flds, nf, rb[q], true);
    return 0;
}

// v[0..n) <- its maximum (op 1) or sum (op 2) over all ranks
int part_allreduce(Ctx& c, double* v, int n, int op) {
    if (!c.xfn) return 0;
    double* b[1] = {v};
    int64_t cnt[1] = {n};
    if (c.xfn(c.xuser, op, 0, nullptr, b, cnt, nullptr, nullptr))
        return fail(MGLET_ERR_ARG, "partition: the reduction failed");
    return 0;
}

int64_t connect(Ctx& c, int ilevel, int layers, double* v1, double* v2, double* v3, double* s1,
                double* s2, double* s3, bool corners, bool normal, int forward) {
    if (part_exchange(c, v1, v2, v3, s1, s2, s3)) return -1;
    int nplane = layers;
    int minl = c.minlevel, maxl = c.maxlevel;
    if (ilevel > 0) { minl = ilevel; maxl = ilevel; }
    int fwd = forward > 0 ? 1 : (forward < 0 ? -1 : 0);
    bool sn = normal;
    int64_t ncopied = 0;
    for (const Conn& cn : c.conns) {
        if (!decide(c, cn, corners, fwd, minl, maxl)) continue;
        const Grid& S = c.g[cn.sendgrid];
        const Grid& D = c.g[cn.recvgrid];
        int is, ie, js, je, ks, ke;
        start_and_stop(S, facenbr[cn.recvface], is, ie, js, je, ks, ke, nplane, true);
        corr_start_stop(S, cn.sendface, cn.recvface, is, ie, js, je, ks, ke, nplane);
        int isd, ied, jsd, jed, ksd, ked;
        start_and_stop(D, cn.recvface, isd, ied, jsd, jed, ksd, ked, nplane, false);
        int64_t ssz = (int64_t)(ie - is + 1) * (je - js + 1) * (ke - ks + 1);
        int64_t dsz = (int64_t)(ied - isd + 1) * (jed - jsd + 1) * (ked - ksd + 1);
        if (ssz != dsz) { g_err = "connect: source/destination size mismatch"; return -1; }
        int rf = cn.recvface;
        bool exU = (sn && rf < 3) || !sn;
        bool exV = (sn && (rf > 2 && rf < 5)) || !sn;
        bool exW = (sn && rf > 4) || !sn;
        double* flds[6] = {exU ? v1 : nullptr, exV ? v2 : nullptr, exW ? v3 : nullptr, s1, s2, s3};
        for (double* a : flds)
            if (a)
                ncopied += connect_self_single(c, a, cn.sendgrid, cn.recvgrid, is, js, ks, isd,
                                               ied, jsd, jed, ksd, ked);
    }
    return ncopied;
}

// ---------------------------------------------------------------------------
// noib_mod.F90:81-250 giteig
void giteig(Ctx& c) {
    double* aw = c.L("GSAW"); double* ae = c.L("GSAE");
    double* as = c.L("GSAS"); double* an = c.L("GSAN");
    double* ab = c.L("GSAB"); double* at = c.L("GSAT");
    double* AP = c.F("GSAP"); double* BP = c.F("BP");
    const double* DX = c.L("DX"); const double* DY = c.L("DY"); const double* DZ = c.L("DZ");
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const double* dx = DX + G.ipx - 1;   // dx[i], i 1-based
        const double* dy = DY + G.ipy - 1;
        const double* dz = DZ + G.ipz - 1;
        double* AW = aw + G.ipx - 1; double* AE = ae + G.ipx - 1;
        double* AS = as + G.ipy - 1; double* AN = an + G.ipy - 1;
        double* AB = ab + G.ipz - 1; double* AT = at + G.ipz - 1;
        double* ap = AP + G.ip3;
        const double* bp = BP + G.ip3;
        for (int i = 3; i <= ii - 2; ++i) {
            AE[i] = 2.0 / ((dx[i - 1] + dx[i]) * dx[i]);
            AW[i] = 2.0 / ((dx[i - 1] + dx[i]) * dx[i - 1]);
        }
        for (int j = 3; j <= jj - 2; ++j) {
            AN[j] = 2.0 / ((dy[j - 1] + dy[j]) * dy[j]);
            AS[j] = 2.0 / ((dy[j - 1] + dy[j]) * dy[j - 1]);
        }
        for (int k = 3; k <= kk - 2; ++k) {
            AT[k] = 2.0 / ((dz[k - 1] + dz[k]) * dz[k]);
            AB[k] = 2.0 / ((dz[k - 1] + dz[k]) * dz[k - 1]);
        }
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k)
                    ap[IX(k, j, i)] = -2.0 / (dx[i - 1] * dx[i]) - 2.0 / (dy[j - 1] * dy[j]) -
                                      2.0 / (dz[k - 1] * dz[k]);
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k)
                    ap[IX(k, j, i)] = ap[IX(k, j, i)] +
                                      AW[i] * (1.0 - bp[IX(k, j, i - 1)] * bp[IX(k, j, i)]) +
                                      AE[i] * (1.0 - bp[IX(k, j, i)] * bp[IX(k, j, i + 1)]) +
                                      AS[j] * (1.0 - bp[IX(k, j - 1, i)] * bp[IX(k, j, i)]) +
                                      AN[j] * (1.0 - bp[IX(k, j, i)] * bp[IX(k, j + 1, i)]) +
                                      AB[k] * (1.0 - bp[IX(k - 1, j, i)] * bp[IX(k, j, i)]) +
                                      AT[k] * (1.0 - bp[IX(k, j, i)] * bp[IX(k + 1, j, i)]);
        auto wall_lo = [](int t) { return t == 2 || t == 5 || t == 6 || t == 19; };
        auto wall_hi = [](int t) { return t == 2 || t == 5 || t == 6; };
        if (wall_lo(G.bc[1])) {
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k)
                    ap[IX(k, j, 3)] = ap[IX(k, j, 3)] + AW[3] * (bp[IX(k, j, 2)] * bp[IX(k, j, 3)]);
            AW[3] = 0.0;
        }
        if (wall_hi(G.bc[2])) {
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k)
                    ap[IX(k, j, ii - 2)] = ap[IX(k, j, ii - 2)] +
                                           AE[ii - 2] * (bp[IX(k, j, ii - 2)] * bp[IX(k, j, ii - 1)]);
            AE[ii - 2] = 0.0;
        }
        if (wall_lo(G.bc[3])) {
            for (int i = 3; i <= ii - 2; ++i)
                for (int k = 3; k <= kk - 2; ++k)
                    ap[IX(k, 3, i)] = ap[IX(k, 3, i)] + AS[3] * (bp[IX(k, 2, i)] * bp[IX(k, 3, i)]);
            AS[3] = 0.0;
        }
        if (wall_hi(G.bc[4])) {
            for (int i = 3; i <= ii - 2; ++i)
                for (int k = 3; k <= kk - 2; ++k)
                    ap[IX(k, jj - 2, i)] = ap[IX(k, jj - 2, i)] +
                                           AN[jj - 2] * (bp[IX(k, jj - 2, i)] * bp[IX(k, jj - 1, i)]);
            AN[jj - 2] = 0.0;
        }
        if (wall_lo(G.bc[5])) {
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    ap[IX(3, j, i)] = ap[IX(3, j, i)] + AB[3] * (bp[IX(2, j, i)] * bp[IX(3, j, i)]);
            AB[3] = 0.0;
        }
        if (wall_hi(G.bc[6])) {
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    ap[IX(kk - 2, j, i)] = ap[IX(kk - 2, j, i)] +
                                           AT[kk - 2] * (bp[IX(kk - 2, j, i)] * bp[IX(kk - 1, j, i)]);
            AT[kk - 2] = 0.0;
        }
    }
}

// ---------------------------------------------------------------------------
// sip_hyperplane_mod.F90:269-334,339-393,398-447: index lists, sort, check.
// mip and idx use the reference's 1-based values, stored in the grid's slab.
int sip_hyperplane_init_grid(int kk, int jj, int ii, int64_t* mip, int64_t* idx) {
    // mip(1..ii+jj+kk) -> mip[m-1]; idxsip(1..) -> idx[n-1]
    const int n3dmin = 9, n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    for (int m = 1; m <= ii + jj + kk; ++m) mip[m - 1] = 0;
    for (int64_t n = 0; n < (int64_t)ii * jj * kk; ++n) idx[n] = -1;
    for (int m = n3dmin; m <= n3dmax; ++m) {
        int64_t ic1 = 0;
        int64_t lm = mip[m - 1];
        int nkmin = std::max(m - (ii - 2) - (jj - 2), 3);
        int nkmax = std::min(m - 2 * 3, kk - 2);
        for (int k = nkmin; k <= nkmax; ++k) {
            int nimin = std::max(m - (jj - 2) - k, 3);
            int nimax = std::min(m - k - 1 * 3, ii - 2);
            for (int i = nimin; i <= nimax; ++i) {
                int j = m - k - i;
                if (i < 3 || i > ii - 2 || j < 3 || j > jj - 2 || k < 3 || k > kk - 2)
                    return fail(MGLET_ERR_ARG, "hyperplane_init_grid: index out of bounds");
                ++ic1;
                idx[lm + ic1 - 1] = (int64_t)k + (int64_t)(j - 1) * kk + (int64_t)(i - 1) * kk * jj;
            }
        }
        mip[m] = mip[m - 1] + ic1;   // mip(m+1)
    }
    // selection sort within each plane (any ascending sort gives the same list)
    for (int m = n3dmin; m <= n3dmax; ++m) {
        int64_t s = mip[m - 1], e = mip[m];
        std::vector<int64_t> v(idx + s, idx + e);
        std::sort(v.begin(), v.end());
        for (size_t q = 1; q < v.size(); ++q)
            if (v[q] <= v[q - 1]) return fail(MGLET_ERR_ARG, "sort: sorting failed");
        std::copy(v.begin(), v.end(), idx + s);
    }
    // check
    std::vector<int> test((size_t)kk * jj * ii, 0);
    for (int m = n3dmin; m <= n3dmax; ++m) {
        for (int64_t ip = mip[m - 1]; ip < mip[m]; ++ip) {
            int64_t id = idx[ip];
            int64_t r = id - 1;
            int k = (int)(r % kk) + 1;
            int j = (int)((r / kk) % jj) + 1;
            int i = (int)(r / ((int64_t)kk * jj)) + 1;
            test[IX(k, j, i)] += 1;
            if (k + j + i != m) return fail(MGLET_ERR_ARG, "hyperplane_check_grid: index error");
        }
    }
    int64_t sum = 0;
    for (int i = 1; i <= ii; ++i)
        for (int j = 1; j <= jj; ++j)
            for (int k = 1; k <= kk; ++k) {
                int t = test[IX(k, j, i)];
                if (t > 1) return fail(MGLET_ERR_ARG, "hyperplane_check_grid: duplicated");
                if (i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2 && t < 1)
                    return fail(MGLET_ERR_ARG, "hyperplane_check_grid: missing");
                sum += t;
            }
    if (sum != (int64_t)(kk - 4) * (jj - 4) * (ii - 4))
        return fail(MGLET_ERR_ARG, "hyperplane_check_grid: summation failed");
    return 0;
}

// sip_hyperplane_mod.F90:106-257 sip_hyperplane_lu
void sip_hyperplane_lu(int kk, int jj, int ii, double* lw, double* ls, double* lb, double* lpr,
                       double* ue, double* un, double* ut, const double* aw, const double* ae,
                       const double* as, const double* an, const double* ab, const double* at,
                       const double* ap, const double* bp, const int64_t* mip,
                       const int64_t* idxsip) {
    // aw..at are 1-based views (aw[i]); ap, bp are grid slabs.
    const int64_t n = (int64_t)kk * jj * ii;
    std::vector<double> lw_t(n + 1, 0.0), ls_t(n + 1, 0.0), lb_t(n + 1, 0.0), lpr_t(n + 1, 0.0),
        ue_t(n + 1, 0.0), un_t(n + 1, 0.0), ut_t(n + 1, 0.0);
    auto BP = [&](int k, int j, int i) { return bp[IX(k, j, i)]; };
    auto bu = [&](int k, int j, int i) { return BP(k, j, i) * BP(k, j, i + 1); };
    auto bv = [&](int k, int j, int i) { return BP(k, j, i) * BP(k, j + 1, i); };
    auto bw = [&](int k, int j, int i) { return BP(k, j, i) * BP(k + 1, j, i); };
    const int n3dmin = 9, n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    for (int m = n3dmin; m <= n3dmax; ++m) {
        int64_t lm = mip[m - 1];
        int64_t lp = mip[m] - lm;
        for (int64_t ip = 1; ip <= lp; ++ip) {
            int64_t iacc = lm + ip;
            int64_t id = idxsip[iacc - 1];
            int64_t km = id - 1, jm = id - kk, im = id - (int64_t)kk * jj;
            int64_t r = id - 1;
            int k = (int)(r % kk) + 1;
            int j = (int)((r / kk) % jj) + 1;
            int i = (int)(r / ((int64_t)kk * jj)) + 1;
            lw_t[id] = aw[i] * bu(k, j, i - 1) / (1.0 + kAlfa * (un_t[im] + ut_t[im]));
            ls_t[id] = as[j] * bv(k, j - 1, i) / (1.0 + kAlfa * (ue_t[jm] + ut_t[jm]));
            lb_t[id] = ab[k] * bw(k - 1, j, i) / (1.0 + kAlfa * (un_t[km] + ue_t[km]));
            double p1 = kAlfa * (lb_t[id] * ue_t[km] + ls_t[id] * ue_t[jm]);
            double p2 = kAlfa * (lb_t[id] * un_t[km] + lw_t[id] * un_t[im]);
            double p3 = kAlfa * (lw_t[id] * ut_t[im] + ls_t[id] * ut_t[jm]);
            lpr_t[id] = 1.0 / (ap[IX(k, j, i)] + p1 + p2 + p3 - lb_t[id] * ut_t[km] -
                               lw_t[id] * ue_t[im] - ls_t[id] * un_t[jm] + kTiny);
            ue_t[id] = (ae[i] * bu(k, j, i) - p1) * lpr_t[id];
            un_t[id] = (an[j] * bv(k, j, i) - p2) * lpr_t[id];
            ut_t[id] = (at[k] * bw(k, j, i) - p3) * lpr_t[id];
            lw_t[id] = lw_t[id] * lpr_t[id];
            ls_t[id] = ls_t[id] * lpr_t[id];
            lb_t[id] = lb_t[id] * lpr_t[id];
            lw[iacc - 1] = lw_t[id];
            ls[iacc - 1] = ls_t[id];
            lb[iacc - 1] = lb_t[id];
            lpr[iacc - 1] = lpr_t[id];
            ue[iacc - 1] = ue_t[id];
            un[iacc - 1] = un_t[id];
            ut[iacc - 1] = ut_t[id];
        }
    }
}

// sip_classic_mod.F90:17-127 sip_classic_init (one grid)
void sip_classic_lu(int kk, int jj, int ii, double* lw, double* ls, double* lb, double* lpr,
                    double* ue, double* un, double* ut, const double* aw, const double* ae,
                    const double* as, const double* an, const double* ab, const double* at,
                    const double* ap, const double* bp) {
    auto BP = [&](int k, int j, int i) { return bp[IX(k, j, i)]; };
    auto bu = [&](int k, int j, int i) { return BP(k, j, i) * BP(k, j, i + 1); };
    auto bv = [&](int k, int j, int i) { return BP(k, j, i) * BP(k, j + 1, i); };
    auto bw = [&](int k, int j, int i) { return BP(k, j, i) * BP(k + 1, j, i); };
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                int64_t c = IX(k, j, i);
                int64_t cim = IX(k, j, i - 1), cjm = IX(k, j - 1, i), ckm = IX(k - 1, j, i);
                lw[c] = aw[i] * bu(k, j, i - 1) / (1.0 + kAlfa * (un[cim] + ut[cim]));
                ls[c] = as[j] * bv(k, j - 1, i) / (1.0 + kAlfa * (ue[cjm] + ut[cjm]));
                lb[c] = ab[k] * bw(k - 1, j, i) / (1.0 + kAlfa * (un[ckm] + ue[ckm]));
                double p1 = kAlfa * (lb[c] * ue[ckm] + ls[c] * ue[cjm]);
                double p2 = kAlfa * (lb[c] * un[ckm] + lw[c] * un[cim]);
                double p3 = kAlfa * (lw[c] * ut[cim] + ls[c] * ut[cjm]);
                lpr[c] = 1.0 / (ap[c] + p1 + p2 + p3 - lb[c] * ut[ckm] - lw[c] * ue[cim] -
                                ls[c] * un[cjm] + kTiny);
                ue[c] = (ae[i] * bu(k, j, i) - p1) * lpr[c];
                un[c] = (an[j] * bv(k, j, i) - p2) * lpr[c];
                ut[c] = (at[k] * bw(k, j, i) - p3) * lpr[c];
            }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j) {
            for (int k = 3; k <= kk - 2; ++k) lw[IX(k, j, i)] = lw[IX(k, j, i)] * lpr[IX(k, j, i)];
            for (int k = 3; k <= kk - 2; ++k) ls[IX(k, j, i)] = ls[IX(k, j, i)] * lpr[IX(k, j, i)];
            for (int k = 3; k <= kk - 2; ++k) lb[IX(k, j, i)] = lb[IX(k, j, i)] * lpr[IX(k, j, i)];
        }
}

// pressuresolver_mod.F90:47-145 init_pressuresolver (SIP coefficient part)
int init_pressuresolver(Ctx& c) {
    for (const char* n : {"SIPLW", "SIPLS", "SIPLB", "SIPUE", "SIPUN", "SIPUT", "SIPLPR"})
        c.f3[n].assign(c.idim3d, 0.0);
    c.mip.assign(c.idim3d, 0);
    c.idxsip.assign(c.idim3d, -1);
    double* aw = c.L("GSAW"); double* ae = c.L("GSAE"); double* as = c.L("GSAS");
    double* an = c.L("GSAN"); double* ab = c.L("GSAB"); double* at = c.L("GSAT");
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        int64_t o = G.ip3;
        if (c.prm.psolver == MGLET_PSOLVER_CLASSIC) {
            sip_classic_lu(G.kk, G.jj, G.ii, c.F("SIPLW") + o, c.F("SIPLS") + o, c.F("SIPLB") + o,
                           c.F("SIPLPR") + o, c.F("SIPUE") + o, c.F("SIPUN") + o,
                           c.F("SIPUT") + o, aw + G.ipx - 1, ae + G.ipx - 1, as + G.ipy - 1,
                           an + G.ipy - 1, ab + G.ipz - 1, at + G.ipz - 1, c.F("GSAP") + o,
                           c.F("BP") + o);
        } else {
            int rc = sip_hyperplane_init_grid(G.kk, G.jj, G.ii, c.mip.data() + o,
                                              c.idxsip.data() + o);
            if (rc) return rc;
            sip_hyperplane_lu(G.kk, G.jj, G.ii, c.F("SIPLW") + o, c.F("SIPLS") + o,
                              c.F("SIPLB") + o, c.F("SIPLPR") + o, c.F("SIPUE") + o,
                              c.F("SIPUN") + o, c.F("SIPUT") + o, aw + G.ipx - 1, ae + G.ipx - 1,
                              as + G.ipy - 1, an + G.ipy - 1, ab + G.ipz - 1, at + G.ipz - 1,
                              c.F("GSAP") + o, c.F("BP") + o, c.mip.data() + o,
                              c.idxsip.data() + o);
        }
    }
    if (c.prm.psolver == MGLET_PSOLVER_SOR) {
        // sor_mod.F90:18-49 (divide0, simdfunctions_mod.F90:56-80)
        c.f3["SOR_RAP"].assign(c.idim3d, 0.0);
        for (int g = 1; g <= c.ngrid; ++g) {
            const Grid& G = c.g[g];
            const int kk = G.kk, jj = G.jj, ii = G.ii;
            double* rap = c.F("SOR_RAP") + G.ip3;
            const double* ap = c.F("GSAP") + G.ip3;
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3; k <= kk - 2; ++k) {
                        double a = ap[IX(k, j, i)];
                        rap[IX(k, j, i)] = a == 0.0 ? 0.0 : 1.0 / a;
                    }
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// laplacephi_mod.F90:134-165 laplacephi_grid
void laplacephi_grid(Ctx& c, int g, double* RES, const double* PHI) {
    const Grid& G = c.g[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    double* res = RES + G.ip3;
    const double* phi = PHI + G.ip3;
    const double* ap = c.F("GSAP") + G.ip3;
    const double* bp = c.F("BP") + G.ip3;
    const double* aw = c.L("GSAW") + G.ipx - 1; const double* ae = c.L("GSAE") + G.ipx - 1;
    const double* as = c.L("GSAS") + G.ipy - 1; const double* an = c.L("GSAN") + G.ipy - 1;
    const double* ab = c.L("GSAB") + G.ipz - 1; const double* at = c.L("GSAT") + G.ipz - 1;
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k)
                res[IX(k, j, i)] =
                    -aw[i] * phi[IX(k, j, i - 1)] * bp[IX(k, j, i - 1)] * bp[IX(k, j, i)] -
                    ae[i] * phi[IX(k, j, i + 1)] * bp[IX(k, j, i)] * bp[IX(k, j, i + 1)] -
                    as[j] * phi[IX(k, j - 1, i)] * bp[IX(k, j - 1, i)] * bp[IX(k, j, i)] -
                    an[j] * phi[IX(k, j + 1, i)] * bp[IX(k, j, i)] * bp[IX(k, j + 1, i)] -
                    ab[k] * phi[IX(k - 1, j, i)] * bp[IX(k - 1, j, i)] * bp[IX(k, j, i)] -
                    at[k] * phi[IX(k + 1, j, i)] * bp[IX(k, j, i)] * bp[IX(k + 1, j, i)] -
                    ap[IX(k, j, i)] * phi[IX(k, j, i)];
}

void laplacephi_level(Ctx& c, int ilevel, double* res, const double* phi) {
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g)
        if (ilevel <= 0 || c.g[g].level == ilevel) laplacephi_grid(c, g, res, phi);
}

// sip_hyperplane_mod.F90:450-505 sipiter1
void sipiter1_hp(int kk, int jj, int ii, const double* rhs, double* res, const double* lw,
                 const double* ls, const double* lb, const double* lpr, const int64_t* mip,
                 const int64_t* idxsip) {
    const int n3dmin = 9, n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    for (int m = n3dmin; m <= n3dmax; ++m) {
        int64_t lm = mip[m - 1], lp = mip[m] - lm;
        for (int64_t ip = 1; ip <= lp; ++ip) {
            int64_t iacc = lm + ip - 1;            // 0-based
            int64_t id = idxsip[iacc] - 1;         // 0-based
            int64_t km = id - 1, jm = id - kk, im = id - (int64_t)kk * jj;
            res[id] = (rhs[id] + res[id]) * lpr[iacc];
            res[id] = res[id] - lb[iacc] * res[km] - ls[iacc] * res[jm] - lw[iacc] * res[im];
        }
    }
}

// sip_hyperplane_mod.F90:508-569 sipiter2
void sipiter2_hp(int kk, int jj, int ii, double* phi, double* res, const double* ue,
                 const double* un, const double* ut, const int64_t* mip, const int64_t* idxsip) {
    const int n3dmin = 9, n3dmax = (ii - 2) + (jj - 2) + (kk - 2);
    for (int m = n3dmax; m >= n3dmin; --m) {
        int64_t lm = mip[m - 1], lp = mip[m] - lm;
        for (int64_t ip = 1; ip <= lp; ++ip) {
            int64_t iacc = lm + ip - 1;
            int64_t id = idxsip[iacc] - 1;
            int64_t kp = id + 1, jp = id + kk, ipp = id + (int64_t)kk * jj;
            res[id] = res[id] - ut[iacc] * res[kp] - un[iacc] * res[jp] - ue[iacc] * res[ipp];
        }
    }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) phi[IX(k, j, i)] = phi[IX(k, j, i)] + res[IX(k, j, i)];
}

// sip_classic_mod.F90:143-166 sipiter1
void sipiter1_cl(int kk, int jj, int ii, const double* rhs, double* res, const double* lw,
                 const double* ls, const double* lb, const double* lpr) {
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j) {
            for (int k = 3; k <= kk - 2; ++k) {
                int64_t c = IX(k, j, i);
                res[c] = (rhs[c] + res[c]) * lpr[c];
                res[c] = res[c] - lw[c] * res[IX(k, j, i - 1)] - ls[c] * res[IX(k, j - 1, i)];
            }
            for (int k = 3; k <= kk - 2; ++k) {
                int64_t c = IX(k, j, i);
                res[c] = res[c] - lb[c] * res[IX(k - 1, j, i)];
            }
        }
}

// sip_classic_mod.F90:169-198 sipiter2
void sipiter2_cl(int kk, int jj, int ii, double* phi, double* res, const double* ue,
                 const double* un, const double* ut) {
    for (int i = ii - 2; i >= 3; --i)
        for (int j = jj - 2; j >= 3; --j) {
            for (int k = 3; k <= kk - 2; ++k) {
                int64_t c = IX(k, j, i);
                res[c] = res[c] - un[c] * res[IX(k, j + 1, i)] - ue[c] * res[IX(k, j, i + 1)];
            }
            for (int k = kk - 2; k >= 3; --k) {
                int64_t c = IX(k, j, i);
                res[c] = res[c] - ut[c] * res[IX(k + 1, j, i)];
            }
        }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) phi[IX(k, j, i)] = phi[IX(k, j, i)] + res[IX(k, j, i)];
}

// sor_mod.F90:102-203 relax (no bp: ib type noib passes no BP)
void relax(Ctx& c, int g, double* DP, const double* RHS) {
    const Grid& G = c.g[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    double* dp = DP + G.ip3;
    const double* rhs = RHS + G.ip3;
    const double* rap = c.F("SOR_RAP") + G.ip3;
    const double* aw = c.L("GSAW") + G.ipx - 1; const double* ae = c.L("GSAE") + G.ipx - 1;
    const double* as = c.L("GSAS") + G.ipy - 1; const double* an = c.L("GSAN") + G.ipy - 1;
    const double* ab = c.L("GSAB") + G.ipz - 1; const double* at = c.L("GSAT") + G.ipz - 1;
    const double omg = c.prm.omega;
    for (int rb = 0; rb <= 1; ++rb)
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j) {
                int ks, ke;
                if ((i + j) % 2 == rb) { ks = 4; ke = kk - 2; }
                else { ks = 3; ke = kk - 3; }
                for (int k = ks; k <= ke; k += 2) {
                    double res = (aw[i] * dp[IX(k, j, i - 1)] + ae[i] * dp[IX(k, j, i + 1)] +
                                  as[j] * dp[IX(k, j - 1, i)] + an[j] * dp[IX(k, j + 1, i)] +
                                  ab[k] * dp[IX(k - 1, j, i)] + at[k] * dp[IX(k + 1, j, i)] -
                                  rhs[IX(k, j, i)]) * rap[IX(k, j, i)];
                    dp[IX(k, j, i)] = (1.0 - omg) * dp[IX(k, j, i)] - omg * res;
                }
            }
}

// pressuresolver_mod.F90:423-465 sip
void sip(Ctx& c, int ilevel, int iloop, double* dp, double* res, const double* rhs) {
    laplacephi_level(c, ilevel, res, dp);
    const bool classic = c.prm.psolver == MGLET_PSOLVER_CLASSIC;
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel) continue;
        int64_t o = G.ip3;
        if (classic)
            sipiter1_cl(G.kk, G.jj, G.ii, rhs + o, res + o, c.F("SIPLW") + o, c.F("SIPLS") + o,
                        c.F("SIPLB") + o, c.F("SIPLPR") + o);
        else
            sipiter1_hp(G.kk, G.jj, G.ii, rhs + o, res + o, c.F("SIPLW") + o, c.F("SIPLS") + o,
                        c.F("SIPLB") + o, c.F("SIPLPR") + o, c.mip.data() + o,
                        c.idxsip.data() + o);
    }
    if (iloop < c.prm.ninner)
        connect(c, ilevel, 1, nullptr, nullptr, nullptr, res, nullptr, nullptr, false, false, 0);
    else
        connect(c, ilevel, 1, nullptr, nullptr, nullptr, res, nullptr, nullptr, false, false, -1);
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel) continue;
        int64_t o = G.ip3;
        if (classic)
            sipiter2_cl(G.kk, G.jj, G.ii, dp + o, res + o, c.F("SIPUE") + o, c.F("SIPUN") + o,
                        c.F("SIPUT") + o);
        else
            sipiter2_hp(G.kk, G.jj, G.ii, dp + o, res + o, c.F("SIPUE") + o, c.F("SIPUN") + o,
                        c.F("SIPUT") + o, c.mip.data() + o, c.idxsip.data() + o);
    }
}

void bound_pressure(Ctx& c, int ilevel, const std::string& name, bool withbp);
void parent(Ctx& c, int ilevel, const char* v[3], const char* sc[3], bool normal);
void rkstep(double* p, double* dp, const double* rhsp, int64_t n, double frhs, double dtfu);
void ftoc_one(Ctx& c, int ilevel, const std::string& ff, const std::string& fc, char flag);
void ctof(Ctx& c, int ilevel, const std::string& ff, const std::string& fc);

// pressuresolver_mod.F90:361-420 mgpoisit on the field HILF (bound_pressure
// acts on PAR faces only; withbp for the ghost-cell IB, which passes bp)
void mgpoisit(Ctx& c, int ilevel, double* dp, const double* rhs, double* res, bool withbp) {
    for (int iloop = 1; iloop <= c.prm.ninner; ++iloop) {
        bound_pressure(c, ilevel, "HILF", withbp);
        if (c.prm.psolver == MGLET_PSOLVER_SOR && ilevel > c.minlevel) {
#pragma omp parallel for schedule(dynamic)
            for (int g = 1; g <= c.ngrid; ++g)
                if (c.g[g].level == ilevel) relax(c, g, dp, rhs);
        } else {
            sip(c, ilevel, iloop, dp, res, rhs);
        }
        connect(c, ilevel, 1, nullptr, nullptr, nullptr, dp, nullptr, nullptr, false, false, 0);
    }
    bound_pressure(c, ilevel, "HILF", withbp);
}

// pressuresolver_mod.F90:623-689 maxabscal
double maxabscal(Ctx& c, const double* PHI) {
    std::vector<double> mg(c.ngrid + 1, 0.0);
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const double* phi = PHI + G.ip3;
        double m = 0.0;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k) m = std::max(std::fabs(phi[IX(k, j, i)]), m);
        mg[g] = m;
    }
    double maxabs = 0.0;
    for (int g = 1; g <= c.ngrid; ++g)
        if (!c.g[g].halo)   // a copy of another rank's grid
            maxabs = std::max(std::fabs(mg[g] * std::ldexp(1.0, c.maxlevel - c.g[g].level)), maxabs);
    // MPI_Allreduce(MAX) of pressuresolver_mod.F90:295 (a failure leaves NaN)
    if (part_allreduce(c, &maxabs, 1, 1)) return std::numeric_limits<double>::quiet_NaN();
    return maxabs;
}

// pressuresolver_mod.F90:787-879 mgpcorr_grid with bp (mgpoisl always passes
// BP, line 333; for the noib BP = 1 the products are exact)
void mgpcorr(Ctx& c, double* U, double* V, double* W, double* P, const double* DP, double rfak) {
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        double* u = U + G.ip3; double* v = V + G.ip3; double* w = W + G.ip3;
        double* p = P + G.ip3;
        const double* dp = DP + G.ip3;
        const double* rdx = c.L("RDX") + G.ipx - 1;
        const double* rdy = c.L("RDY") + G.ipy - 1;
        const double* rdz = c.L("RDZ") + G.ipz - 1;
        const double* bp = c.F("BP") + G.ip3;
        for (int i = 2; i <= ii - 1; ++i)
            for (int j = 2; j <= jj - 1; ++j)
                for (int k = 2; k <= kk - 1; ++k)
                    p[IX(k, j, i)] = p[IX(k, j, i)] + dp[IX(k, j, i)] * bp[IX(k, j, i)];
        for (int i = 2; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k)
                    u[IX(k, j, i)] = u[IX(k, j, i)] + (dp[IX(k, j, i)] - dp[IX(k, j, i + 1)]) *
                                                          bp[IX(k, j, i)] * bp[IX(k, j, i + 1)] *
                                                          rdx[i] * rfak;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 2; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k)
                    v[IX(k, j, i)] = v[IX(k, j, i)] + (dp[IX(k, j, i)] - dp[IX(k, j + 1, i)]) *
                                                          bp[IX(k, j, i)] * bp[IX(k, j + 1, i)] *
                                                          rdy[j] * rfak;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 2; k <= kk - 2; ++k)
                    w[IX(k, j, i)] = w[IX(k, j, i)] + (dp[IX(k, j, i)] - dp[IX(k + 1, j, i)]) *
                                                          bp[IX(k, j, i)] * bp[IX(k + 1, j, i)] *
                                                          rdz[k] * rfak;
    }
}

// noib_mod.F90:253-354 divcal (noib: no bp, no sdiv)
void divcal(Ctx& c, double* DIV, const double* U, const double* V, const double* W, double fak) {
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        double* div = DIV + G.ip3;
        const double* u = U + G.ip3; const double* v = V + G.ip3; const double* w = W + G.ip3;
        const double* rddx = c.L("RDDX") + G.ipx - 1;
        const double* rddy = c.L("RDDY") + G.ipy - 1;
        const double* rddz = c.L("RDDZ") + G.ipz - 1;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k)
                    div[IX(k, j, i)] = fak * ((u[IX(k, j, i)] - u[IX(k, j, i - 1)]) * rddx[i] +
                                              (v[IX(k, j, i)] - v[IX(k, j - 1, i)]) * rddy[j] +
                                              (w[IX(k, j, i)] - w[IX(k - 1, j, i)]) * rddz[k]);
        if (c.ibtype == 1) {
            // gc_mod.F90:278-347 passes sdiv and bp to divcal_grid (noib_mod.F90:328-353)
            const double* sdiv = c.F("SDIV") + G.ip3;
            const double* bp = c.F("BP") + G.ip3;
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3; k <= kk - 2; ++k)
                        div[IX(k, j, i)] = div[IX(k, j, i)] + fak * sdiv[IX(k, j, i)];
            for (int64_t q = 0; q < (int64_t)kk * jj * ii; ++q) div[q] = bp[q] * div[q];
        }
    }
}

// pressuresolver_mod.F90:160-357 mgpoisl over every level of the hierarchy
// (one level: ftoc, ctof, parent and bound_pressure have no work)
void bound_flow(Ctx& c, double* U, double* V, double* W, double* P, int ilevel = 0);

void mgpoisl(Ctx& c, double dt, mglet_stage_stats* st) {
    double* U = c.F("U"); double* V = c.F("V"); double* W = c.F("W"); double* P = c.F("P");
    for (const char* n : {"DP", "HILF", "RHS", "RES"}) c.f3[n].assign(c.idim3d, 0.0);
    double* dp = c.F("DP"); double* hilf = c.F("HILF");
    double* rhs = c.F("RHS"); double* res = c.F("RES");
    const double prefak = c.prm.rho / dt;
    const bool withbp = c.ibtype == 1;
    const char* none[3] = {nullptr, nullptr, nullptr};
    const char* shilf[3] = {"HILF", nullptr, nullptr};
    divcal(c, rhs, U, V, W, prefak);
    for (int l = c.maxlevel; l >= c.minlevel; --l) ftoc_one(c, l, "RHS", "RHS", 'R');
    int ipc = 0, ipcount_done = 0;
    double maxrhs = 0.0;
    for (int ipcount = 1; ipcount <= c.prm.nouter; ++ipcount) {
        for (int ilevel = c.minlevel; ilevel <= c.maxlevel; ++ilevel) {
            ctof(c, ilevel, "HILF", "HILF");
            parent(c, ilevel, none, shilf, false);
            mgpoisit(c, ilevel, hilf, rhs, res, withbp);
        }
        for (int l = c.maxlevel; l >= c.minlevel; --l) ftoc_one(c, l, "HILF", "HILF", 'P');
        connect(c, 0, 1, nullptr, nullptr, nullptr, hilf, nullptr, nullptr, false, false, 0);
        laplacephi_level(c, 0, res, hilf);
        // rescal: rhs += res on the interior
#pragma omp parallel for schedule(dynamic)
        for (int g = 1; g <= c.ngrid; ++g) {
            const Grid& G = c.g[g];
            const int kk = G.kk, jj = G.jj, ii = G.ii;
            double* r = rhs + G.ip3; const double* s = res + G.ip3;
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3; k <= kk - 2; ++k) r[IX(k, j, i)] = r[IX(k, j, i)] + s[IX(k, j, i)];
        }
        for (int l = c.maxlevel; l >= c.minlevel + 1; --l) ftoc_one(c, l, "RHS", "RHS", 'R');
        maxrhs = maxabscal(c, rhs);
        // accumulate_pcorr over the whole flat array, then hilf = 0
        for (int64_t n = 0; n < c.idim3d; ++n) dp[n] = dp[n] + hilf[n];
        std::fill(c.f3["HILF"].begin(), c.f3["HILF"].end(), 0.0);
        ipc += c.prm.ninner;
        ipcount_done = ipcount;
        if (ipcount >= c.prm.nouter_min && maxrhs / prefak < c.prm.epcorr) break;
    }
    const char* sdp[3] = {"DP", nullptr, nullptr};
    for (int l = c.minlevel; l <= c.maxlevel; ++l) {
        parent(c, l, none, sdp, false);
        bound_pressure(c, l, "DP", withbp);
    }
    mgpcorr(c, U, V, W, P, dp, dt / c.prm.rho);
    // pressuresolver_mod.F90:334-348: ftoc fine to coarse, then per level
    // parent, bound and the corner connect
    for (int l = c.maxlevel; l >= c.minlevel; --l) {
        ftoc_one(c, l, "U", "U", 'U');
        ftoc_one(c, l, "V", "V", 'V');
        ftoc_one(c, l, "W", "W", 'W');
        ftoc_one(c, l, "P", "P", 'P');
    }
    const char* vuvw[3] = {"U", "V", "W"};
    const char* sp[3] = {"P", nullptr, nullptr};
    for (int l = c.minlevel; l <= c.maxlevel; ++l) {
        parent(c, l, vuvw, sp, false);
        bound_flow(c, U, V, W, P, l);
        connect(c, l, 2, U, V, W, P, nullptr, nullptr, true, false, 0);
    }
    if (st) {
        st->ipc = ipc;
        st->nouter_done = ipcount_done;
        st->maxrhs = maxrhs;
        st->prefak = prefak;
    }
}

// ---------------------------------------------------------------------------
// bound_flow_mod.F90 bfront (:23-256), bright (:259-494), bbottom (:497-730)
// for FIX, OP1, NOS and SLI, dispatched grid by grid and face 1..6 as
// bound_t%bound does (src/core/bound_mod.F90:36-76).  Face-local layout: the
// face-normal index n (i, j or k), the two tangential indices a < b in the
// reference's loop order (k, j for x faces; k, i for y faces; j, i for z).
double fsign(double a, double b) { return std::copysign(std::fabs(a), b); }

void bound_par(Ctx& c, int g, int iface, double* U, double* V, double* W);

void bound_face(Ctx& c, int g, int iface, double* U, double* V, double* W, double* P) {
    const Grid& G = c.g[g];
    const int typ = G.bc[iface];
    if (typ == MGLET_BC_PAR) {
        bound_par(c, g, iface, U, V, W);
        return;
    }
    if (!(typ == MGLET_BC_FIX || typ == MGLET_BC_OP1 || typ == MGLET_BC_NOS || typ == MGLET_BC_SLI))
        return;
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    double* u = U + G.ip3; double* v = V + G.ip3; double* w = W + G.ip3;
    double* p = P ? P + G.ip3 : nullptr;
    const int64_t bo = c.bufoff[6 * (g - 1) + iface - 1];
    const double* ub = c.bufU.data() + bo; const double* vb = c.bufV.data() + bo;
    const double* wb = c.bufW.data() + bo;
    const double pin = c.npinf[6 * (g - 1) + iface - 1] ? c.pinf[6 * (g - 1) + iface - 1] : 0.0;
    const double rho = c.prm.rho;
    const int axis = (iface - 1) / 2;          // 0: x (bfront), 1: y (bright), 2: z (bbottom)
    const bool lo = (iface % 2) == 1;
    const int nn = axis == 0 ? ii : (axis == 1 ? jj : kk);
    const int n2 = lo ? 2 : nn - 1, n3 = lo ? 3 : nn - 2;
    const int st1 = lo ? 1 : nn - 1, st2 = lo ? 2 : nn - 2;
    const double dir = lo ? -1.0 : 1.0;
    // tangential extents of the face: a runs fastest
    const int na = axis == 2 ? jj : kk, nb = axis == 0 ? jj : ii;
    // index of (a, b, n) in the grid; a, b tangential, n normal
    auto at = [&](int a, int b, int n) -> int64_t {
        if (axis == 0) return IX(a, b, n);        // (k, j, i)
        if (axis == 1) return IX(a, n, b);        // (k, j, i) with j normal
        return IX(n, a, b);                       // k normal
    };
    auto bi = [&](int a, int b) -> int64_t { return (int64_t)(a - 1) + (int64_t)(b - 1) * na; };
    // the normal component and the two tangential ones, in the reference's order
    double* vn = axis == 0 ? u : (axis == 1 ? v : w);
    const double* bn = axis == 0 ? ub : (axis == 1 ? vb : wb);
    // tangential components t1, t2: x faces (v, w), y faces (u, w), z faces
    // (u, v); t1 is staggered along b and t2 along a, so the OP1 flag of t1
    // averages the normal velocity over (a, b), (a, b+1) and that of t2 over
    // (a, b), (a+1, b)
    double* t1 = axis == 0 ? v : u;
    double* t2 = axis == 2 ? v : w;
    const double* b1 = axis == 0 ? vb : ub;
    const double* b2 = axis == 2 ? vb : wb;
    if (typ == MGLET_BC_FIX) {
        for (int b = 1; b <= nb; ++b)
            for (int a = 1; a <= na; ++a) {
                if (axis == 0) {
                    vn[at(a, b, st2)] = bn[bi(a, b)];
                    t1[at(a, b, n2)] = 2.0 * b1[bi(a, b)] - t1[at(a, b, n3)];
                    t2[at(a, b, n2)] = 2.0 * b2[bi(a, b)] - t2[at(a, b, n3)];
                } else if (axis == 1) {
                    t1[at(a, b, n2)] = 2.0 * b1[bi(a, b)] - t1[at(a, b, n3)];
                    vn[at(a, b, st2)] = bn[bi(a, b)];
                    t2[at(a, b, n2)] = 2.0 * b2[bi(a, b)] - t2[at(a, b, n3)];
                } else {
                    t1[at(a, b, n2)] = 2.0 * b1[bi(a, b)] - t1[at(a, b, n3)];
                    t2[at(a, b, n2)] = 2.0 * b2[bi(a, b)] - t2[at(a, b, n3)];
                    vn[at(a, b, st2)] = bn[bi(a, b)];
                }
            }
    } else if (typ == MGLET_BC_OP1) {
        for (int b = 1; b <= nb - 1; ++b)
            for (int a = 1; a <= na - 1; ++a) {
                // 1 for outflow (zero gradient), 0 for inflow (prescribed)
                double f1 = fsign(1.0, dir * (vn[at(a, b, st2)] + vn[at(a, b + 1, st2)]));
                double f2 = fsign(1.0, dir * (vn[at(a, b, st2)] + vn[at(a + 1, b, st2)]));
                f1 = 0.5 * (f1 + 1.0);
                f2 = 0.5 * (f2 + 1.0);
                const double n1v = f1 * t1[at(a, b, n3)] +
                                   (1.0 - f1) * (2.0 * b1[bi(a, b)] - t1[at(a, b, n3)]);
                const double n2v = f2 * t2[at(a, b, n3)] +
                                   (1.0 - f2) * (2.0 * b2[bi(a, b)] - t2[at(a, b, n3)]);
                if (axis == 0) {
                    vn[at(a, b, st1)] = vn[at(a, b, st2)];
                    t1[at(a, b, n2)] = n1v;
                    t2[at(a, b, n2)] = n2v;
                } else if (axis == 1) {
                    t1[at(a, b, n2)] = n1v;
                    vn[at(a, b, st1)] = vn[at(a, b, st2)];
                    t2[at(a, b, n2)] = n2v;
                } else {
                    t1[at(a, b, n2)] = n1v;
                    t2[at(a, b, n2)] = n2v;
                    vn[at(a, b, st1)] = vn[at(a, b, st2)];
                }
            }
    } else if (typ == MGLET_BC_NOS) {
        for (int b = 1; b <= nb; ++b)
            for (int a = 1; a <= na; ++a) {
                vn[at(a, b, st2)] = 0.0;
                t1[at(a, b, n2)] = 0.0;
                t2[at(a, b, n2)] = 0.0;
            }
    } else {   // SLI
        for (int b = 1; b <= nb; ++b)
            for (int a = 1; a <= na; ++a) {
                vn[at(a, b, st2)] = 0.0;
                t1[at(a, b, n2)] = t1[at(a, b, n3)];
                t2[at(a, b, n2)] = t2[at(a, b, n3)];
            }
    }
    if (!p) return;
    if (typ == MGLET_BC_OP1) {
        for (int b = 2; b <= nb; ++b)
            for (int a = 2; a <= na; ++a) {
                // the two tangential components interpolated to the cell centre
                const double c1 = 0.25 * (t1[at(a, b - 1, n2)] + t1[at(a, b, n2)] +
                                          t1[at(a, b - 1, n3)] + t1[at(a, b, n3)]);
                const double c2 = 0.25 * (t2[at(a - 1, b, n2)] + t2[at(a, b, n2)] +
                                          t2[at(a - 1, b, n3)] + t2[at(a, b, n3)]);
                const double un = vn[at(a, b, st2)];
                double umagsqr;
                if (axis == 0) umagsqr = un * un + c1 * c1 + c2 * c2;
                else if (axis == 1) umagsqr = c1 * c1 + un * un + c2 * c2;
                else umagsqr = c1 * c1 + c2 * c2 + un * un;
                p[at(a, b, n2)] = pin + std::min(0.0, 0.5 * rho * fsign(umagsqr, dir * un));
            }
    } else {
        for (int b = 1; b <= nb; ++b)
            for (int a = 1; a <= na; ++a) p[at(a, b, n2)] = p[at(a, b, n3)];
    }
}

void bound_flow(Ctx& c, double* U, double* V, double* W, double* P, int ilevel) {
    for (int g = 1; g <= c.ngrid; ++g) {
        if (ilevel && c.g[g].level != ilevel) continue;
        for (int f = 1; f <= 6; ++f) bound_face(c, g, f, U, V, W, P);
    }
}

// ---------------------------------------------------------------------------
// Multi-level operators (no IB restriction operator; BP enters bound_flow and
// the bp form of bound_pressure).

const double kPoint1 = (double)0.1f;   // the default-kind literal 0.1 of the PAR branches

std::vector<double>& buffer_of(Ctx& c, const std::string& n) {
    if (n == "U") return c.bufU;
    if (n == "V") return c.bufV;
    if (n == "W") return c.bufW;
    std::vector<double>& b = c.bufx[n];
    if (b.empty()) b.assign(c.bufU.size(), 0.0);
    return b;
}

// bound_flow_mod.F90:139-256 (bfront), :377-494 (bright), :613-730 (bbottom):
// the PAR branch.  Tangential components from the buffer with the
// interior's slope, the normal one as the buffer's coarse flux minus the
// fine flux of blocked faces.  Written per orientation: the three routines
// differ in operand order (x faces multiply by the b spacing first, y and z
// faces by the a spacing first) and the y faces take the tangential w slope
// from the ghost plane.
void bound_par(Ctx& c, int g, int iface, double* U, double* V, double* W) {
    const Grid& G = c.g[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    double* u = U + G.ip3; double* v = V + G.ip3; double* w = W + G.ip3;
    const double* bp = c.F("BP") + G.ip3;
    const int64_t bo = c.bufoff[6 * (g - 1) + iface - 1];
    const double* ub = c.bufU.data() + bo; const double* vb = c.bufV.data() + bo;
    const double* wb = c.bufW.data() + bo;
    const double* ddx = c.L("DDX") + G.ipx - 1;   // 1-based
    const double* ddy = c.L("DDY") + G.ipy - 1;
    const double* ddz = c.L("DDZ") + G.ipz - 1;
    const int axis = (iface - 1) / 2;
    const bool lo = (iface % 2) == 1;
    const int nn = axis == 0 ? ii : (axis == 1 ? jj : kk);
    const int n2 = lo ? 2 : nn - 1, n3 = lo ? 3 : nn - 2, n4 = lo ? 4 : nn - 3;
    const int st2 = lo ? 2 : nn - 2;
    const int na = axis == 2 ? jj : kk, nb = axis == 0 ? jj : ii;
    auto at = [&](int a, int b, int n) -> int64_t {
        if (axis == 0) return IX(a, b, n);
        if (axis == 1) return IX(a, n, b);
        return IX(n, a, b);
    };
    auto bi = [&](int a, int b) -> int64_t { return (int64_t)(a - 1) + (int64_t)(b - 1) * na; };
    const double* da = axis == 2 ? ddy : ddz;     // spacing along a
    const double* db = axis == 0 ? ddy : ddx;     // spacing along b
    double* vn = axis == 0 ? u : (axis == 1 ? v : w);
    const double* bn = axis == 0 ? ub : (axis == 1 ? vb : wb);
    double* t1 = axis == 0 ? v : u;               // staggered along b
    double* t2 = axis == 2 ? v : w;               // staggered along a
    const double* b1 = axis == 0 ? vb : ub;
    const double* b2 = axis == 2 ? vb : wb;
    // tangential components
    for (int b = 2; b <= nb - 1; ++b)
        for (int a = 2; a <= na - 1; ++a) {
            const double s1 = bp[at(a, b, n2)] * bp[at(a, b + 1, n2)];
            const double s2 = bp[at(a, b, n2)] * bp[at(a + 1, b, n2)];
            t1[at(a, b, n2)] = (b1[bi(a, b)] - 0.5 * (t1[at(a, b, n3)] - t1[at(a, b, n4)])) * s1 +
                               (1.0 - s1) * t1[at(a, b, n2)];
            const double slope2 = axis == 1 ? (t2[at(a, b, n2)] - t2[at(a, b, n4)])
                                            : (t2[at(a, b, n3)] - t2[at(a, b, n4)]);
            t2[at(a, b, n2)] = (b2[bi(a, b)] - 0.5 * slope2) * s2 + (1.0 - s2) * t2[at(a, b, n2)];
        }
    // face-normal component, 2x2 fine faces per coarse face
    auto prod = [&](double s, double x, double y) { return s * x * y; };
    for (int b = 3; b <= nb - 2; b += 2)
        for (int a = 3; a <= na - 2; a += 2) {
            const double sbn = bp[at(a, b, n2)];
            // the four fine faces (a, b), (a, b+1), (a+1, b), (a+1, b+1)
            const int fa[4] = {a, a, a + 1, a + 1}, fb[4] = {b, b + 1, b, b + 1};
            double sb[4];
            for (int q = 0; q < 4; ++q) {
                const int a1 = fa[q], b1q = fb[q];
                if (sbn > 0.5)
                    sb[q] = bp[at(a1, b1q, n2)] * bp[at(a1, b1q, n3)];
                else
                    sb[q] = std::min(bp[at(a1, b1q, n3)] + bp[at(a1, b1q, n2)] + bp[at(a1, b1q, n4)] +
                                         bp[at(a1, b1q - 1, n3)] + bp[at(a1, b1q + 1, n3)] +
                                         bp[at(a1 - 1, b1q, n3)] + bp[at(a1 + 1, b1q, n3)],
                                     1.0);
            }
            double fak, fine;
            const double area = axis == 0 ? (db[b] + db[b + 1]) * (da[a] + da[a + 1])
                                          : (da[a] + da[a + 1]) * (db[b] + db[b + 1]);
            if (axis == 0) {
                fak = 1.0 / area * (prod(sb[0], db[b], da[a]) + prod(sb[1], db[b + 1], da[a]) +
                                    prod(sb[2], db[b], da[a + 1]) + prod(sb[3], db[b + 1], da[a + 1]));
            } else {
                fak = 1.0 / area * (prod(sb[0], da[a], db[b]) + prod(sb[1], da[a], db[b + 1]) +
                                    prod(sb[2], da[a + 1], db[b]) + prod(sb[3], da[a + 1], db[b + 1]));
            }
            if (fak < kPoint1) fak = 1.0;
            fak = 1.0 / fak;
            double f[4];
            for (int q = 0; q < 4; ++q) {
                const double x = vn[at(fa[q], fb[q], st2)] * (1.0 - sb[q]);
                f[q] = axis == 0 ? x * db[fb[q]] * da[fa[q]] : x * da[fa[q]] * db[fb[q]];
            }
            fine = (f[0] + f[1] + f[2] + f[3]) / area;
            for (int q = 0; q < 4; ++q) {
                double& x = vn[at(fa[q], fb[q], st2)];
                x = (bn[bi(fa[q], fb[q])] - fine) * fak * sb[q] + (1.0 - sb[q]) * x * sbn;
            }
        }
}

// parent_core_mod.F90:190-255 start_and_stop: the coarse slab (1-based,
// inclusive) that the PAR face iface of fine grid igrid is prolonged from
void par_slab(const Ctx& c, int igrid, int iface, int icomp, int r[6]) {
    const Grid& G = c.g[igrid];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int ipos = c.pos[igrid][0], jpos = c.pos[igrid][1], kpos = c.pos[igrid][2];
    int ks = kpos - 2, js = jpos - 2, is = ipos - 2;
    int ke = ks + kk / 2 + 1, je = js + jj / 2 + 1, ie = is + ii / 2 + 1;
    if (iface == 1) { is = ipos - 1; ie = ipos - 1; }
    else if (iface == 2) { is = ipos + (ii - 4) / 2; if (icomp == 1) is -= 1; ie = is; }
    else if (iface == 3) { js = jpos - 1; je = jpos - 1; }
    else if (iface == 4) { js = jpos + (jj - 4) / 2; if (icomp == 2) js -= 1; je = js; }
    else if (iface == 5) { ks = kpos - 1; ke = kpos - 1; }
    else { ks = kpos + (kk - 4) / 2; if (icomp == 3) ks -= 1; ke = ks; }
    r[0] = is; r[1] = ie; r[2] = js; r[3] = je; r[4] = ks; r[5] = ke;
}

// parent1_mod.F90 (pack_single :287-325, read_buffer :345-470, prolong1
// :515-547, prolong2 :550-584): for every PAR face of the grids of ilevel,
// the parent's boundary slab is prolonged piecewise constant (staggered
// directions: the first fine point averages two coarse ones) into the fine
// grid's boundary buffer of the field.  comp: 1/2/3 for the vector
// components (staggered along x / y / z), 0 for scalars.
void parent_field(Ctx& c, int igrid, int iface, const std::string& name, int comp) {
    const Grid& G = c.g[igrid];
    const Grid& P = c.g[c.iparent[igrid]];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    int icomp = 0;
    if ((iface == 1 || iface == 2) && comp == 1) icomp = 1;
    if ((iface == 3 || iface == 4) && comp == 2) icomp = 2;
    if ((iface == 5 || iface == 6) && comp == 3) icomp = 3;
    int r[6];
    par_slab(c, igrid, iface, icomp, r);
    const double* fc = c.F(name.c_str()) + P.ip3;
    std::vector<double> in;
    {
        const int kk_ = P.kk, jj_ = P.jj;
        for (int i = r[0]; i <= r[1]; ++i)
            for (int j = r[2]; j <= r[3]; ++j)
                for (int k = r[4]; k <= r[5]; ++k)
                    in.push_back(fc[(int64_t)(i - 1) * kk_ * jj_ + (int64_t)(j - 1) * kk_ + (k - 1)]);
    }
    // idx2d (parent_core_mod.F90:154-183) and stag (:186-210)
    const int kkc = kk / 2 + 2, jjc = jj / 2 + 2, iic = ii / 2 + 2;
    int jj2d, ii2d, jjc2d, iic2d, st1 = 0, st2 = 0;
    if (iface <= 2) { ii2d = jj; jj2d = kk; iic2d = jjc; jjc2d = kkc; }
    else if (iface <= 4) { ii2d = ii; jj2d = kk; iic2d = iic; jjc2d = kkc; }
    else { ii2d = ii; jj2d = jj; iic2d = iic; jjc2d = jjc; }
    if (iface <= 2) { if (comp == 2) st2 = 1; if (comp == 3) st1 = 1; }
    else if (iface <= 4) { if (comp == 1) st2 = 1; if (comp == 3) st1 = 1; }
    else { if (comp == 1) st2 = 1; if (comp == 2) st1 = 1; }
    if ((int)in.size() != jjc2d * iic2d) throw std::runtime_error("parent: slab size");
    // prolong1: first direction
    std::vector<double> tmp((size_t)jj2d * iic2d);
    for (int ic = 1; ic <= iic2d; ++ic)
        for (int j = 1; j <= jj2d; j += 2) {
            const int jc = 2 + (j - 1) / 2;
            const double x = in[(jc - 1) + (size_t)(ic - 1) * jjc2d];
            tmp[(j - 1) + (size_t)(ic - 1) * jj2d] =
                st1 ? 0.5 * (x + in[(jc - 2) + (size_t)(ic - 1) * jjc2d]) : x;
            tmp[j + (size_t)(ic - 1) * jj2d] = x;
        }
    // prolong2: second direction, into the buffer
    double* out = buffer_of(c, name).data() + c.bufoff[6 * (igrid - 1) + iface - 1];
    for (int i = 1; i <= ii2d; i += 2) {
        const int ic = 2 + (i - 1) / 2;
        for (int j = 1; j <= jj2d; ++j) {
            const double x = tmp[(j - 1) + (size_t)(ic - 1) * jj2d];
            out[(j - 1) + (size_t)(i - 1) * jj2d] =
                st2 ? 0.5 * (x + tmp[(j - 1) + (size_t)(ic - 2) * jj2d]) : x;
            out[(j - 1) + (size_t)i * jj2d] = x;
        }
    }
}

// parent1_mod.F90:24-71 parent1: vector components (v1, v2, v3; with normal
// only the face-normal one) and scalars, PAR faces of the grids of ilevel
void parent(Ctx& c, int ilevel, const char* v[3], const char* sc[3], bool normal) {
    for (int g = 1; g <= c.ngrid; ++g) {
        if (c.g[g].level != ilevel || !c.iparent[g]) continue;
        for (int f = 1; f <= 6; ++f) {
            if (c.g[g].bc[f] != MGLET_BC_PAR) continue;
            const bool ex[3] = {!normal || f < 3, !normal || (f > 2 && f < 5), !normal || f > 4};
            for (int q = 0; q < 3; ++q)
                if (v[q] && ex[q]) parent_field(c, g, f, v[q], q + 1);
            for (int q = 0; q < 3; ++q)
                if (sc[q]) parent_field(c, g, f, sc[q], 0);
        }
    }
}

// bound_pressure_mod.F90:534-609 pressureftocone_A / _B: volume- (and bp-)
// weighted mean of the 2x2x2 fine cells starting at (k, j, i)
void pressureftocone(const Grid& G, int k, int j, int i, const double* p, const double* bp,
                     const double* ddx, const double* ddy, const double* ddz, double& pc,
                     double& bpc) {
    const int kk = G.kk, jj = G.jj;
    if (!bp) {
        bpc = 1.0;
        double sump = 0.0, sumvol = 0.0;
        for (int l = 0; l <= 1; ++l)
            for (int m = 0; m <= 1; ++m)
                for (int n = 0; n <= 1; ++n) {
                    const double vol = ddz[k + n] * ddy[j + m] * ddx[i + l];
                    sump = sump + p[IX(k + n, j + m, i + l)] * vol;
                    sumvol = sumvol + vol;
                }
        pc = sump / sumvol;
        return;
    }
    double sumbp = 0.0;
    for (int l = 0; l <= 1; ++l)
        for (int m = 0; m <= 1; ++m)
            for (int n = 0; n <= 1; ++n) sumbp = sumbp + bp[IX(k + n, j + m, i + l)];
    bpc = std::min(sumbp, 1.0);
    if (bpc < 0.5) {
        pc = 0.0;
        return;
    }
    double sump = 0.0, sumvol = 0.0;
    for (int l = 0; l <= 1; ++l)
        for (int m = 0; m <= 1; ++m)
            for (int n = 0; n <= 1; ++n) {
                const double vol = bp[IX(k + n, j + m, i + l)] * ddz[k + n] * ddy[j + m] * ddx[i + l];
                sump = sump + p[IX(k + n, j + m, i + l)] * vol;
                sumvol = sumvol + vol;
            }
    pc = sump / sumvol;
}

// bound_pressure_mod.F90:106-533: PAR faces of the grids of ilevel; the
// ghost plane of dp from the buffer (the parent's value) minus the fine
// mean next to the face, per 2x2 block.  withbp: the _bp forms.
void bound_pressure(Ctx& c, int ilevel, const std::string& name, bool withbp) {
    const std::vector<double>& buf = buffer_of(c, name);
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel) continue;
        for (int iface = 1; iface <= 6; ++iface) {
            if (G.bc[iface] != MGLET_BC_PAR) continue;
            const int kk = G.kk, jj = G.jj, ii = G.ii;
            double* p = c.F(name.c_str()) + G.ip3;
            const double* bp = withbp ? c.F("BP") + G.ip3 : nullptr;
            const double* pb = buf.data() + c.bufoff[6 * (g - 1) + iface - 1];
            const double* ddx = c.L("DDX") + G.ipx - 1;
            const double* ddy = c.L("DDY") + G.ipy - 1;
            const double* ddz = c.L("DDZ") + G.ipz - 1;
            const int axis = (iface - 1) / 2;
            const bool lo = (iface % 2) == 1;
            const int nn = axis == 0 ? ii : (axis == 1 ? jj : kk);
            const int n2 = lo ? 2 : nn - 1, n3 = lo ? 3 : nn - 2, n4 = lo ? 4 : nn - 3;
            const int st2 = lo ? 2 : nn - 2;
            const int nmin = std::min(n3, n4);
            const int na = axis == 2 ? jj : kk, nb = axis == 0 ? jj : ii;
            const double* dn = axis == 0 ? ddx : (axis == 1 ? ddy : ddz);
            const double* dstag = axis == 0 ? c.L("DX") + G.ipx - 1
                                            : (axis == 1 ? c.L("DY") + G.ipy - 1 : c.L("DZ") + G.ipz - 1);
            const double* da = axis == 2 ? ddy : ddz;
            const double* db = axis == 0 ? ddy : ddx;
            auto at = [&](int a, int b, int n) -> int64_t {
                if (axis == 0) return IX(a, b, n);
                if (axis == 1) return IX(a, n, b);
                return IX(n, a, b);
            };
            for (int b = 3; b <= nb - 2; b += 2)
                for (int a = 3; a <= na - 2; a += 2) {
                    // (k, j, i) of the 2x2x2 block at the face
                    int k, j, i;
                    if (axis == 0) { k = a; j = b; i = nmin; }
                    else if (axis == 1) { k = a; j = nmin; i = b; }
                    else { k = nmin; j = a; i = b; }
                    double pcnew, bpc;
                    pressureftocone(G, k, j, i, p, bp, ddx, ddy, ddz, pcnew, bpc);
                    const double pbv = pb[(a - 1) + (int64_t)(b - 1) * na];
                    double fak = 1.0;
                    if (withbp) {
                        if (bpc < 0.5) pcnew = pbv;
                        const double s11 = bp[at(a, b, n2)] * bp[at(a, b, n3)];
                        const double s12 = bp[at(a, b + 1, n2)] * bp[at(a, b + 1, n3)];
                        const double s13 = bp[at(a + 1, b, n2)] * bp[at(a + 1, b, n3)];
                        const double s14 = bp[at(a + 1, b + 1, n2)] * bp[at(a + 1, b + 1, n3)];
                        fak = (s11 * db[b] * da[a] + s12 * db[b + 1] * da[a] + s13 * db[b] * da[a + 1] +
                               s14 * db[b + 1] * da[a + 1]) /
                              ((db[b] + db[b + 1]) * (da[a] + da[a + 1]));
                        if (fak < kPoint1) fak = 1.0;
                        fak = 1.0 / fak;
                    }
                    for (int l = 0; l <= 1; ++l)
                        for (int n = 0; n <= 1; ++n) {
                            // the two tangential offsets: b outer, a inner
                            const int64_t dst = at(a + n, b + l, n2), src = at(a + n, b + l, n3);
                            if (withbp)
                                p[dst] = p[src] + fak * dstag[st2] / (dn[n3] + dn[n2]) * (pbv - pcnew);
                            else
                                p[dst] = p[src] + dstag[st2] / (dn[n3] + dn[n2]) * (pbv - pcnew);
                        }
                }
        }
    }
}

// noib_restrict_mod.F90:40-124 start_and_stop: the fine loop ranges, stride 2
void restrict_range(const Grid& G, char flag, int r[6]) {
    int is = 3, ie = 3, js = 3, je = 3, ks = 3, ke = 3;
    if (flag == 'U') { is = 2; ie = 2; }
    else if (flag == 'V') { js = 2; je = 2; }
    else if (flag == 'W') { ks = 2; ke = 2; }
    r[0] = is; r[1] = G.ii - ie; r[2] = js; r[3] = G.jj - je; r[4] = ks; r[5] = G.kk - ke;
}

// noib_restrict_mod.F90:126-298 restrict_u/v/w/s (area- or volume-weighted
// fine means) and ftoc_mod.F90:581-626 restrict_recieve_open (the coarse
// index of every fine block): fine grids of ilevel into their parents
//
// With the ghost-cell IB (gc_restrict_t, gc_restrict_mod.F90:8-17) P and R
// take the BP-weighted forms; U, V, W and S stay the no-IB means.
void ftoc_one(Ctx& c, int ilevel, const std::string& ff, const std::string& fc, char flag) {
    const char f = (flag == 'P' || flag == 'R' || flag == 'S' || flag == 'T') ? 'P' : flag;
    // restrict_p weighs P by BP and T by BT (gc_restrict_mod.F90:85-89)
    const bool gcp = c.ibtype == 1 && (flag == 'P' || flag == 'T'), gcr = c.ibtype == 1 && flag == 'R';
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel || !c.iparent[g]) continue;
        const Grid& P = c.g[c.iparent[g]];
        const int kk = G.kk, jj = G.jj;
        const double* bp = c.F(flag == 'T' && c.ibtype == 1 ? "BT" : "BP") + G.ip3;
        const double* fv = c.F(ff.c_str()) + G.ip3;
        double* cv = c.F(fc.c_str()) + P.ip3;
        const double* ddx = c.L("DDX") + G.ipx - 1;
        const double* ddy = c.L("DDY") + G.ipy - 1;
        const double* ddz = c.L("DDZ") + G.ipz - 1;
        int r[6];
        restrict_range(G, f, r);
        const int ic0 = f == 'U', jc0 = f == 'V', kc0 = f == 'W';
        const int ipos = c.pos[g][0], jpos = c.pos[g][1], kpos = c.pos[g][2];
        for (int i = r[0]; i <= r[1]; i += 2)
            for (int j = r[2]; j <= r[3]; j += 2)
                for (int k = r[4]; k <= r[5]; k += 2) {
                    double val;
                    if (f == 'U') {
                        const double s = fv[IX(k, j, i)] * ddy[j] * ddz[k] + fv[IX(k, j + 1, i)] * ddy[j + 1] * ddz[k] +
                                         fv[IX(k + 1, j, i)] * ddy[j] * ddz[k + 1] +
                                         fv[IX(k + 1, j + 1, i)] * ddy[j + 1] * ddz[k + 1];
                        val = s / ((ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
                    } else if (f == 'V') {
                        const double s = fv[IX(k, j, i)] * ddx[i] * ddz[k] + fv[IX(k, j, i + 1)] * ddx[i + 1] * ddz[k] +
                                         fv[IX(k + 1, j, i)] * ddx[i] * ddz[k + 1] +
                                         fv[IX(k + 1, j, i + 1)] * ddx[i + 1] * ddz[k + 1];
                        val = s / ((ddx[i] + ddx[i + 1]) * (ddz[k] + ddz[k + 1]));
                    } else if (f == 'W') {
                        const double s = fv[IX(k, j, i)] * ddx[i] * ddy[j] + fv[IX(k, j, i + 1)] * ddx[i + 1] * ddy[j] +
                                         fv[IX(k, j + 1, i)] * ddx[i] * ddy[j + 1] +
                                         fv[IX(k, j + 1, i + 1)] * ddx[i + 1] * ddy[j + 1];
                        val = s / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]));
                    } else if (gcp) {
                        // gc_restrict_mod.F90:59-171 restrict_p: BP-weighted volume mean
                        double vol[4][2], pv[4][2];
                        const int cj[4] = {j, j, j + 1, j + 1}, ci[4] = {i, i + 1, i, i + 1};
                        for (int m = 0; m < 4; ++m)
                            for (int l = 0; l < 2; ++l) {
                                vol[m][l] = bp[IX(k + l, cj[m], ci[m])] * ddz[k + l] * ddy[cj[m]] * ddx[ci[m]];
                                pv[m][l] = fv[IX(k + l, cj[m], ci[m])] * vol[m][l];
                            }
                        const double sum_pv = pv[0][0] + pv[1][0] + pv[2][0] + pv[3][0] + pv[0][1] + pv[1][1] +
                                              pv[2][1] + pv[3][1];
                        const double sum_v = vol[0][0] + vol[1][0] + vol[2][0] + vol[3][0] + vol[0][1] +
                                             vol[1][1] + vol[2][1] + vol[3][1];
                        val = sum_v > 0.0 ? sum_pv / sum_v : 0.0;
                    } else if (gcr) {
                        // gc_restrict_mod.F90:174-259 restrict_r: BP-weighted sum over the full volume
                        double pv[4][2];
                        const int cj[4] = {j, j, j + 1, j + 1}, ci[4] = {i, i + 1, i, i + 1};
                        for (int m = 0; m < 4; ++m)
                            for (int l = 0; l < 2; ++l)
                                pv[m][l] = fv[IX(k + l, cj[m], ci[m])] * bp[IX(k + l, cj[m], ci[m])] * ddz[k + l] *
                                           ddy[cj[m]] * ddx[ci[m]];
                        const double sum_pv = pv[0][0] + pv[1][0] + pv[2][0] + pv[3][0] + pv[0][1] + pv[1][1] +
                                              pv[2][1] + pv[3][1];
                        const double sum_v = (ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]);
                        val = sum_pv / sum_v;
                    } else {
                        const double s = fv[IX(k, j, i)] * ddz[k] * ddy[j] * ddx[i] +
                                         fv[IX(k, j, i + 1)] * ddz[k] * ddy[j] * ddx[i + 1] +
                                         fv[IX(k, j + 1, i)] * ddz[k] * ddy[j + 1] * ddx[i] +
                                         fv[IX(k, j + 1, i + 1)] * ddz[k] * ddy[j + 1] * ddx[i + 1] +
                                         fv[IX(k + 1, j, i)] * ddz[k + 1] * ddy[j] * ddx[i] +
                                         fv[IX(k + 1, j, i + 1)] * ddz[k + 1] * ddy[j] * ddx[i + 1] +
                                         fv[IX(k + 1, j + 1, i)] * ddz[k + 1] * ddy[j + 1] * ddx[i] +
                                         fv[IX(k + 1, j + 1, i + 1)] * ddz[k + 1] * ddy[j + 1] * ddx[i + 1];
                        val = s / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1]));
                    }
                    const int ic = ipos + (i - 3 + ic0) / 2 - ic0;
                    const int jc = jpos + (j - 3 + jc0) / 2 - jc0;
                    const int kc = kpos + (k - 3 + kc0) / 2 - kc0;
                    cv[(int64_t)(ic - 1) * P.kk * P.jj + (int64_t)(jc - 1) * P.kk + (kc - 1)] = val;
                }
    }
}

// ctof1_mod.F90:167-211 write_buffer + :308-331 unpack_single: every point
// of the fine grids of ilevel (ghosts included) takes the value of the
// parent cell it lies in
void ctof(Ctx& c, int ilevel, const std::string& ff, const std::string& fc) {
    if (ilevel == c.minlevel) return;
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel || !c.iparent[g]) continue;
        const Grid& P = c.g[c.iparent[g]];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        double* fv = c.F(ff.c_str()) + G.ip3;
        const double* cv = c.F(fc.c_str()) + P.ip3;
        const int is = c.pos[g][0] - 1, js = c.pos[g][1] - 1, ks = c.pos[g][2] - 1;
        for (int i = 1; i <= ii; ++i)
            for (int j = 1; j <= jj; ++j)
                for (int k = 1; k <= kk; ++k) {
                    const int ic = is + (i - 1) / 2, jc = js + (j - 1) / 2, kc = ks + (k - 1) / 2;
                    fv[IX(k, j, i)] = cv[(int64_t)(ic - 1) * P.kk * P.jj + (int64_t)(jc - 1) * P.kk + (kc - 1)];
                }
    }
}

// par_ftoc_mod.F90:36-64 par_ftoc_norm with init_par_ftoc :513-779: on every
// PAR face of the grids of ilevel the face-normal velocity, as the area mean
// of 2x2 fine faces (pack_single :226-318; the plain sum when sum is set),
// goes to the parent -- inside it (front at ipos-1, back at the last covered
// face) or onto its own boundary face when the PAR lies on a coarse face,
// and in that case also onto the opposite face of the parent's neighbour
// across that face (unpack_single :366-469).
void par_ftoc_norm(Ctx& c, int ilevel, double* U, double* V, double* W, bool sum) {
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel || !c.iparent[g]) continue;
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const double* ddx = c.L("DDX") + G.ipx - 1;
        const double* ddy = c.L("DDY") + G.ipy - 1;
        const double* ddz = c.L("DDZ") + G.ipz - 1;
        const int par = c.iparent[g];
        const Grid& P = c.g[par];
        const int ipos = c.pos[g][0], jpos = c.pos[g][1], kpos = c.pos[g][2];
        for (int iface = 1; iface <= 6; ++iface) {
            if (G.bc[iface] != MGLET_BC_PAR) continue;
            double* field = iface <= 2 ? U : (iface <= 4 ? V : W);
            const double* ff = field + G.ip3;
            // start_and_stop (:760-810) of the fine face
            int ks = 3, ke = kk - 2, js = 3, je = jj - 2, is = 3, ie = ii - 2;
            switch (iface) {
            case 1: is = ie = 2; break;
            case 2: is = ie = ii - 2; break;
            case 3: js = je = 2; break;
            case 4: js = je = jj - 2; break;
            case 5: ks = ke = 2; break;
            case 6: ks = ke = kk - 2; break;
            }
            std::vector<double> buf;
            auto F = [&](int k, int j, int i) { return ff[IX(k, j, i)]; };
            if (iface <= 2) {
                const int i = is;
                for (int j = js; j <= je; j += 2)
                    for (int k = ks; k <= ke; k += 2) {
                        if (sum) { buf.push_back(F(k, j, i) + F(k, j + 1, i) + F(k + 1, j, i) + F(k + 1, j + 1, i)); continue; }
                        const double sua = F(k, j, i) * ddy[j] * ddz[k] + F(k, j + 1, i) * ddy[j + 1] * ddz[k] +
                                           F(k + 1, j, i) * ddy[j] * ddz[k + 1] + F(k + 1, j + 1, i) * ddy[j + 1] * ddz[k + 1];
                        buf.push_back(sua / ((ddy[j] + ddy[j + 1]) * (ddz[k] + ddz[k + 1])));
                    }
            } else if (iface <= 4) {
                const int j = js;
                for (int i = is; i <= ie; i += 2)
                    for (int k = ks; k <= ke; k += 2) {
                        if (sum) { buf.push_back(F(k, j, i) + F(k, j, i + 1) + F(k + 1, j, i) + F(k + 1, j, i + 1)); continue; }
                        const double sua = F(k, j, i) * ddx[i] * ddz[k] + F(k, j, i + 1) * ddx[i + 1] * ddz[k] +
                                           F(k + 1, j, i) * ddx[i] * ddz[k + 1] + F(k + 1, j, i + 1) * ddx[i + 1] * ddz[k + 1];
                        buf.push_back(sua / ((ddx[i] + ddx[i + 1]) * (ddz[k] + ddz[k + 1])));
                    }
            } else {
                const int k = ks;
                for (int i = is; i <= ie; i += 2)
                    for (int j = js; j <= je; j += 2) {
                        if (sum) { buf.push_back(F(k, j, i) + F(k, j + 1, i) + F(k, j, i + 1) + F(k, j + 1, i + 1)); continue; }
                        const double sua = F(k, j, i) * ddx[i] * ddy[j] + F(k, j + 1, i) * ddx[i] * ddy[j + 1] +
                                           F(k, j, i + 1) * ddx[i + 1] * ddy[j] + F(k, j + 1, i + 1) * ddx[i + 1] * ddy[j + 1];
                        buf.push_back(sua / ((ddx[i] + ddx[i + 1]) * (ddy[j] + ddy[j + 1])));
                    }
            }
            // the destinations (init_par_ftoc :566-690)
            const int pos = iface <= 2 ? ipos : (iface <= 4 ? jpos : kpos);
            const int nf = iface <= 2 ? ii : (iface <= 4 ? jj : kk);
            const int nc = iface <= 2 ? P.ii : (iface <= 4 ? P.jj : P.kk);
            const bool one_connect = !(nf > nc);
            const bool odd = iface % 2 == 1;
            int recv1 = iface;
            if (pos == 3 && one_connect) {
                if (!odd) recv1 = -1;
            } else if (pos > 3) {
                if (odd) recv1 = -1;
            }
            auto unpack = [&](int gc, int ifr) {
                const Grid& C = c.g[gc];
                int ista = ipos, isto = ipos + (ii - 4) / 2 - 1;
                int jsta = jpos, jsto = jpos + (jj - 4) / 2 - 1;
                int ksta = kpos, ksto = kpos + (kk - 4) / 2 - 1;
                if (ifr < 0) {
                    switch (iface) {
                    case 1: ista = isto = ipos - 1; break;
                    case 2: ista = isto; break;
                    case 3: jsta = jsto = jpos - 1; break;
                    case 4: jsta = jsto; break;
                    case 5: ksta = ksto = kpos - 1; break;
                    case 6: ksta = ksto; break;
                    }
                } else {
                    switch (ifr) {
                    case 1: ista = isto = 2; break;
                    case 2: ista = isto = C.ii - 2; break;
                    case 3: jsta = jsto = 2; break;
                    case 4: jsta = jsto = C.jj - 2; break;
                    case 5: ksta = ksto = 2; break;
                    case 6: ksta = ksto = C.kk - 2; break;
                    }
                }
                double* fc = field + C.ip3;
                size_t n = 0;
                for (int i = ista; i <= isto; ++i)
                    for (int j = jsta; j <= jsto; ++j)
                        for (int k = ksta; k <= ksto; ++k)
                            fc[(int64_t)(i - 1) * C.kk * C.jj + (int64_t)(j - 1) * C.kk + (k - 1)] = buf[n++];
            };
            unpack(par, recv1);
            if (recv1 < 0) continue;
            const int nbr = P.nbr[iface];
            if (nbr <= 0) continue;
            unpack(nbr, odd ? iface + 1 : iface - 1);
        }
    }
}

// lesmodel_mod.F90:573-764 bfront / bright / bbottom, the bound of the
// viscosity G on the grids of ilevel, faces in the order of bound_mod.F90:
// 36-76: NOS and SLI put -EPSILON*gmol into the first ghost plane, FIX and
// OP1 copy the first interior plane there, PAR takes its buffer (rows
// 2..n-1) where BP is open.
void bound_g(Ctx& c, int ilevel) {
    double* Gf = c.F("G");
    const double* BP = c.F("BP");
    const std::vector<double>& buf = buffer_of(c, "G");
    const double geps = -std::numeric_limits<double>::epsilon() * c.prm.gmol;
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel) continue;
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        double* gv = Gf + G.ip3;
        const double* bp = BP + G.ip3;
        for (int f = 1; f <= 6; ++f) {
            const int t = G.bc[f];
            const bool wall = t == MGLET_BC_NOS || t == MGLET_BC_SLI;
            const bool copy = t == MGLET_BC_FIX || t == MGLET_BC_OP1;
            const bool par = t == MGLET_BC_PAR;
            if (!wall && !copy && !par) continue;
            const int d = (f - 1) / 2;
            const int n = d == 0 ? ii : (d == 1 ? jj : kk);
            const int p2 = f % 2 == 1 ? 2 : n - 1, p3 = f % 2 == 1 ? 3 : n - 2;
            const double* b = buf.data() + c.bufoff[6 * (g - 1) + f - 1];
            // the plane's two directions (a outer, q inner) and the flat index
            const int na = d == 2 ? ii : (d == 1 ? ii : jj), nq = d == 2 ? jj : kk;
            auto at = [&](int p, int a, int q) -> int64_t {
                if (d == 0) return IX(q, a, p);
                if (d == 1) return IX(q, p, a);
                return IX(p, q, a);
            };
            const int lo = par ? 2 : 1, ahi = par ? na - 1 : na, qhi = par ? nq - 1 : nq;
            for (int a = lo; a <= ahi; ++a)
                for (int q = lo; q <= qhi; ++q) {
                    const int64_t x = at(p2, a, q);
                    if (wall) {
                        gv[x] = geps;
                    } else if (copy) {
                        gv[x] = gv[at(p3, a, q)];
                    } else {
                        const double sbp = bp[x];
                        gv[x] = b[(q - 1) + (int64_t)(a - 1) * nq] * sbp + (1.0 - sbp) * gv[x];
                    }
                }
        }
    }
}

// lesmodel_mod.F90:63-80 init_lesmodel for the model "none": G = gmol inside
// every grid and 0 on its ghost layers (zero_ghostlayers, mgletmath_mod.F90:
// 27-44), connected with corners; on the finer levels the PAR buffers from
// the parent (parent, s1 = G) and the bound above.  The coarsest level's
// wall faces keep G = 0 in their ghosts, so no viscous flux crosses them.
void init_viscosity(Ctx& c) {
    double* Gf = c.F("G");
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        double* gv = Gf + G.ip3;
        for (int i = 1; i <= ii; ++i)
            for (int j = 1; j <= jj; ++j)
                for (int k = 1; k <= kk; ++k) {
                    const bool in = i >= 3 && i <= ii - 2 && j >= 3 && j <= jj - 2 && k >= 3 && k <= kk - 2;
                    gv[IX(k, j, i)] = in ? c.prm.gmol : 0.0;
                }
    }
    connect(c, 0, 2, nullptr, nullptr, nullptr, Gf, nullptr, nullptr, true, false, 0);
    const char* none[3] = {nullptr, nullptr, nullptr};
    const char* sg[3] = {"G", nullptr, nullptr};
    for (int l = c.minlevel + 1; l <= c.maxlevel; ++l) {
        parent(c, l, none, sg, false);
        bound_g(c, l);
    }
}

// wernerwengle_mod.F90:13-28 init_wernerwengle: the constants of the
// Werner-Wengle wall function for gmol and rho
struct WernerWengle {
    double rho, gmol, cwb, cpo4, cpo5, cpo6, cpo8;
};

WernerWengle werner_wengle(double gmol, double rho) {
    WernerWengle q;
    const double cwa = 8.3;
    q.rho = rho;
    q.gmol = gmol;
    q.cwb = 1.0 / 7.0;
    const double cpo1 = 1.0 - q.cwb;
    const double cpo2 = 1.0 + q.cwb;
    q.cpo4 = cpo2 / cwa * std::pow(gmol / rho, q.cwb);
    q.cpo5 = 0.5 * cpo1 * std::pow(cwa, cpo2 / cpo1) * std::pow(gmol / rho, cpo2);
    q.cpo6 = 0.5 * gmol / rho * std::pow(cwa, 2.0 / cpo1);
    q.cpo8 = 2.0 / cpo2;
    return q;
}

// ---- LES models (lesmodel_mod.F90:93-570) ---------------------------------

// the default-kind literal of a model constant, widened: Cm = 0.1 is the
// single-precision 0.1
double les_default_cm(int model) {
    return model == 1 ? (double)0.1f : (model == 2 ? 0.5 : (double)1.35f);
}

double sabs(double dudx, double dudy, double dudz, double dvdx, double dvdy, double dvdz,
            double dwdx, double dwdy, double dwdz) {
    // lesmodel_mod.F90:520-540
    return std::sqrt(dudx * dudx + dvdy * dvdy + dwdz * dwdz + 0.5 * ((dvdx + dudy) * (dvdx + dudy)) +
                     0.5 * ((dwdx + dudz) * (dwdx + dudz)) + 0.5 * ((dwdy + dvdz) * (dwdy + dvdz)));
}

// lesmodel_mod.F90:368-390 smagorinsky: Cm^2 sqrt(2) |S|
double les_smagorinsky(double cm, const double* gr) {
    return cm * cm * std::sqrt(2.0) * sabs(gr[0], gr[1], gr[2], gr[3], gr[4], gr[5], gr[6], gr[7], gr[8]);
}

// lesmodel_mod.F90:393-487 wale; x**5 as x^3 x^2, the expansion of an
// integer power by repeated products
double les_wale(double cm, double tol, const double* gr) {
    const double dudx = gr[0], dudy = gr[1], dudz = gr[2], dvdx = gr[3], dvdy = gr[4], dvdz = gr[5];
    const double dwdx = gr[6], dwdy = gr[7], dwdz = gr[8];
    const double third = (double)(1.0f / 3.0f);   // (1.0/3.0) of default-kind literals
    const double tr = dudx * dudx + dudy * dvdx + dudz * dwdx + dvdx * dudy + dvdy * dvdy + dvdz * dwdy +
                      dwdx * dudz + dwdy * dvdz + dwdz * dwdz;
    const double sd00 = 0.5 * (dudx * dudx + dudy * dvdx + dudz * dwdx + dudx * dudx + dudy * dvdx + dudz * dwdx) -
                        third * tr;
    const double sd01 = 0.5 * (dudx * dudy + dudy * dvdy + dudz * dwdy + dvdx * dudx + dvdy * dvdx + dvdz * dwdx);
    const double sd02 = 0.5 * (dudx * dudz + dudy * dvdz + dudz * dwdz + dwdx * dudx + dwdy * dvdx + dwdz * dwdx);
    const double sd11 = 0.5 * (dvdx * dudy + dvdy * dvdy + dvdz * dwdy + dvdx * dudy + dvdy * dvdy + dvdz * dwdy) -
                        third * tr;
    const double sd12 = 0.5 * (dvdx * dudz + dvdy * dvdz + dvdz * dwdz + dwdx * dudy + dwdy * dvdy + dwdz * dwdy);
    const double sd22 = 0.5 * (dwdx * dudz + dwdy * dvdz + dwdz * dwdz + dwdx * dudz + dwdy * dvdz + dwdz * dwdz) -
                        third * tr;
    const double sdabs = std::sqrt(sd00 * sd00 + 2 * (sd01 * sd01) + 2 * (sd02 * sd02) + sd11 * sd11 +
                                   2 * (sd12 * sd12) + sd22 * sd22);
    const double sa = sabs(dudx, dudy, dudz, dvdx, dvdy, dvdz, dwdx, dwdy, dwdz);
    const double root = std::sqrt(sdabs);
    if (root < tol * sa) return 0.0;
    const double x = root == 0.0 ? 0.0 : sa / root;
    const double x2 = x * x, x3 = x2 * x;
    return cm * cm * root / (x3 * x2 + 1.0);
}

// lesmodel_mod.F90:490-517 sigma with tensormath_mod.F90 (t, multiply, sqr,
// trace, det) and eig_b :221-268 (the analytic eigenvalues of Hasan et al.):
// the singular values of the velocity gradient; the C library's pow, acos
// and cos as the reference calls them
double les_sigma(double cm, const double* gr) {
    double g[3][3];   // g[c][r] = gij%g(r+1, c+1): columns dudx..dudz, dvdx.., dwdx..
    for (int cc = 0; cc < 3; ++cc)
        for (int r = 0; r < 3; ++r) g[cc][r] = gr[3 * cc + r];
    // G = gij^T gij: G(j,i) = sum_k gij(i,k) gij(j,k), from 0 in k order
    double G[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double a = 0.0;
            for (int k = 0; k < 3; ++k) a = a + g[k][i] * g[k][j];
            G[i][j] = a;   // G[i][j] = G%g(j+1, i+1)
        }
    auto at = [&](int r, int cc) { return G[cc - 1][r - 1]; };   // G%g(r, c)
    double sq[3][3];
    for (int i = 1; i <= 3; ++i)
        for (int j = 1; j <= 3; ++j)
            sq[i - 1][j - 1] = at(1, i) * at(j, 1) + at(2, i) * at(j, 2) + at(3, i) * at(j, 3);
    const double i1 = at(1, 1) + at(2, 2) + at(3, 3);
    const double i2 = 0.5 * (i1 * i1 - (sq[0][0] + sq[1][1] + sq[2][2]));
    const double i3 = at(1, 1) * (at(2, 2) * at(3, 3) - at(3, 2) * at(2, 3)) -
                      at(2, 1) * (at(1, 2) * at(3, 3) - at(3, 2) * at(1, 3)) +
                      at(3, 1) * (at(1, 2) * at(2, 3) - at(2, 2) * at(1, 3));
    double a1 = i1 * i1 / 9.0 - i2 / 3.0;
    const double a2 = i1 * i1 * i1 / 27.0 - (i1 * i2) / 6.0 + i3 / 2.0;
    a1 = std::max(a1, 0.0);
    const double den = std::pow(a1, 3.0 / 2.0);
    double arg = den == 0.0 ? 0.0 : a2 / den;
    arg = std::max(std::min(arg, 1.0), -1.0);
    const double a3 = (1.0 / 3.0) * std::acos(arg);
    const double pi = 4.0 * std::atan(1.0);
    double e1 = i1 / 3.0 + 2.0 * std::sqrt(a1) * std::cos(a3);
    double e2 = i1 / 3.0 - 2.0 * std::sqrt(a1) * std::cos(pi / 3.0 + a3);
    double e3 = i1 / 3.0 - 2.0 * std::sqrt(a1) * std::cos(pi / 3.0 - a3);
    e1 = std::max(e1, 0.0); e2 = std::max(e2, 0.0); e3 = std::max(e3, 0.0);
    const double s1 = std::sqrt(e1), s2 = std::sqrt(e2), s3 = std::sqrt(e3);
    const double num = s3 * (s1 - s2) * (s2 - s3), d1 = s1 * s1;
    return cm * cm * (d1 == 0.0 ? 0.0 : num / d1);
}

// the Werner-Wengle gradient dds/2 from the wall (wernerwengle_mod.F90:36-61)
double gradp2(const WernerWengle& q, double cpo11, double cpo12, double uquer, double dds) {
    const double uquern = std::fabs(uquer);
    const double vz = std::copysign(1.0, uquer);
    const double rdds = 1.0 / dds;
    if (uquern >= q.cpo6 * rdds) return rdds * (cpo12 * uquern + cpo11 * rdds) * vz;
    return 2.0 * uquern / dds * vz;
}

// efvisc_gc (lesmodel_mod.F90:200-365) of one grid: G inside from the
// velocity gradients, the filter width cbrt(cell volume) * BP, and the NOS
// wall-model gradients
void efvisc_grid(Ctx& c, int g) {
    const Grid& G = c.g[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int64_t o = G.ip3;
    const double* u = c.F("U") + o; const double* v = c.F("V") + o; const double* w = c.F("W") + o;
    const double* bp = c.F("BP") + o;
    double* gv = c.F("G") + o;
    const double* dx = c.L("DX") + G.ipx - 1; const double* dy = c.L("DY") + G.ipy - 1;
    const double* dz = c.L("DZ") + G.ipz - 1;
    const double* ddx = c.L("DDX") + G.ipx - 1; const double* ddy = c.L("DDY") + G.ipy - 1;
    const double* ddz = c.L("DDZ") + G.ipz - 1;
    const double* rddx = c.L("RDDX") + G.ipx - 1; const double* rddy = c.L("RDDY") + G.ipy - 1;
    const double* rddz = c.L("RDDZ") + G.ipz - 1;
    const double gmol = c.prm.gmol, rho = c.prm.rho;
    const WernerWengle q = werner_wengle(gmol, rho);
    const double cwb = q.cwb, cpo1 = 1.0 - cwb, cpo2 = 1.0 + cwb;
    const double cpo11 = 2.0 * q.cpo6 * cwb * cpo1 / std::pow(2.0, cwb);
    const double cpo12 = cwb * cpo2 / std::pow(2.0, cwb - 1.0);
    const double tol = 1.0 / std::pow(std::numeric_limits<double>::max(), 1.0 / 6.0);
    const int nfro = G.bc[1], nbac = G.bc[2], nrgt = G.bc[3], nlft = G.bc[4], nbot = G.bc[5], ntop = G.bc[6];
#define A(a, k, j, i) a[IX(k, j, i)]
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                double gr[9];
                const double dxf = 0.25 * dx[i - 1] * rddx[i];
                gr[0] = (A(u, k, j, i) - A(u, k, j, i - 1)) * rddx[i];
                gr[1] = ((A(u, k, j + 1, i) - A(u, k, j - 1, i)) * dxf +
                         (A(u, k, j + 1, i - 1) - A(u, k, j - 1, i - 1)) * (0.5 - dxf)) * rddy[j];
                gr[2] = ((A(u, k + 1, j, i) - A(u, k - 1, j, i)) * dxf +
                         (A(u, k + 1, j, i - 1) - A(u, k - 1, j, i - 1)) * (0.5 - dxf)) * rddz[k];
                const double dyf = 0.25 * dy[j - 1] * rddy[j];
                gr[3] = ((A(v, k, j, i + 1) - A(v, k, j, i - 1)) * dyf +
                         (A(v, k, j - 1, i + 1) - A(v, k, j - 1, i - 1)) * (0.5 - dyf)) * rddx[i];
                gr[4] = (A(v, k, j, i) - A(v, k, j - 1, i)) * rddy[j];
                gr[5] = ((A(v, k + 1, j, i) - A(v, k - 1, j, i)) * dyf +
                         (A(v, k + 1, j - 1, i) - A(v, k - 1, j - 1, i)) * (0.5 - dyf)) * rddz[k];
                const double dzf = 0.25 * dz[k - 1] * rddz[k];
                gr[6] = ((A(w, k, j, i + 1) - A(w, k, j, i - 1)) * dzf +
                         (A(w, k - 1, j, i + 1) - A(w, k - 1, j, i - 1)) * (0.5 - dzf)) * rddx[i];
                gr[7] = ((A(w, k, j + 1, i) - A(w, k, j - 1, i)) * dzf +
                         (A(w, k - 1, j + 1, i) - A(w, k - 1, j - 1, i)) * (0.5 - dzf)) * rddy[j];
                gr[8] = (A(w, k, j, i) - A(w, k - 1, j, i)) * rddz[k];
                double delta = std::cbrt(ddx[i] * ddy[j] * ddz[k]);
                delta = delta * A(bp, k, j, i);
                // NOS corrections (:261-330), in the reference's order
                const double dyf2 = 0.5 * dy[j - 1] * rddy[j], dzf2 = 0.5 * dz[k - 1] * rddz[k];
                const double dxf2 = 0.5 * dx[i - 1] * rddx[i];
                const double vm = dyf2 * A(v, k, j, i) + (1.0 - dyf2) * A(v, k, j - 1, i);
                const double wm = dzf2 * A(w, k, j, i) + (1.0 - dzf2) * A(w, k - 1, j, i);
                const double um = dxf2 * A(u, k, j, i) + (1.0 - dxf2) * A(u, k, j, i - 1);
                if (nfro == 5 && i == 3) { gr[3] = gradp2(q, cpo11, cpo12, vm, ddx[i]); gr[6] = gradp2(q, cpo11, cpo12, wm, ddx[i]); }
                if (nbac == 5 && i == ii - 2) { gr[3] = -gradp2(q, cpo11, cpo12, vm, ddx[i]); gr[6] = -gradp2(q, cpo11, cpo12, wm, ddx[i]); }
                if (nrgt == 5 && j == 3) { gr[1] = gradp2(q, cpo11, cpo12, um, ddy[j]); gr[7] = gradp2(q, cpo11, cpo12, wm, ddy[j]); }
                if (nlft == 5 && j == jj - 2) { gr[1] = -gradp2(q, cpo11, cpo12, um, ddy[j]); gr[7] = -gradp2(q, cpo11, cpo12, wm, ddy[j]); }
                if (nbot == 5 && k == 3) { gr[2] = gradp2(q, cpo11, cpo12, um, ddz[k]); gr[5] = gradp2(q, cpo11, cpo12, vm, ddz[k]); }
                if (ntop == 5 && k == kk - 2) { gr[2] = -gradp2(q, cpo11, cpo12, um, ddz[k]); gr[5] = -gradp2(q, cpo11, cpo12, vm, ddz[k]); }
                const double dm = c.ilesmodel == 1 ? les_smagorinsky(c.cm, gr)
                                   : (c.ilesmodel == 2 ? les_wale(c.cm, tol, gr) : les_sigma(c.cm, gr));
                A(gv, k, j, i) = rho * (delta * delta) * dm + gmol;
            }
#undef A
}

// setginbody (lesmodel_mod.F90:543-570): in blocked cells G is the mean of
// the open neighbours, in place and in loop order
void setginbody(Ctx& c, int g) {
    const Grid& G = c.g[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    double* gv = c.F("G") + G.ip3;
    const double* bp = c.F("BP") + G.ip3;
#define A(a, k, j, i) a[IX(k, j, i)]
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                double nn = A(bp, k, j, i + 1) + A(bp, k, j, i - 1) + A(bp, k, j + 1, i) + A(bp, k, j - 1, i) +
                            A(bp, k + 1, j, i) + A(bp, k - 1, j, i);
                nn = std::max(nn, 1.0);
                const double gbpn = (A(gv, k, j, i + 1) * A(bp, k, j, i + 1) + A(gv, k, j, i - 1) * A(bp, k, j, i - 1) +
                                     A(gv, k, j + 1, i) * A(bp, k, j + 1, i) + A(gv, k, j - 1, i) * A(bp, k, j - 1, i) +
                                     A(gv, k + 1, j, i) * A(bp, k + 1, j, i) + A(gv, k - 1, j, i) * A(bp, k - 1, j, i)) /
                                    nn;
                A(gv, k, j, i) = A(bp, k, j, i) * A(gv, k, j, i) + (1.0 - A(bp, k, j, i)) * gbpn;
            }
#undef A
}

// lesmodel / lesmodel_gc (lesmodel_mod.F90:93-197): efvisc level by level
// (finest first), then per level parent, bound and connect of G, setginbody,
// and the corner connect tstle4 needs
void lesmodel(Ctx& c) {
    if (c.ilesmodel == 0) return;
    for (int l = c.maxlevel; l >= c.minlevel; --l)
        for (int g = 1; g <= c.ngrid; ++g)
            if (c.g[g].level == l) efvisc_grid(c, g);
    double* Gf = c.F("G");
    const char* none[3] = {nullptr, nullptr, nullptr};
    const char* sg[3] = {"G", nullptr, nullptr};
    for (int l = c.minlevel; l <= c.maxlevel; ++l) {
        parent(c, l, none, sg, false);
        bound_g(c, l);
        connect(c, l, 1, nullptr, nullptr, nullptr, Gf, nullptr, nullptr, false, false, 0);
    }
    for (int g = 1; g <= c.ngrid; ++g) setginbody(c, g);
    connect(c, 0, 1, nullptr, nullptr, nullptr, Gf, nullptr, nullptr, true, false, 0);
}

// ---- momentum source terms after tstle4 (timeintegration_mod.F90:102-103) --

// boussinesqterm_grid (boussinesqterm_mod.F90:92-181): -gravity beta T_old at
// the velocity points, over tstle4's ranges, per component with gravity
void boussinesqterm(Ctx& c) {
    if (!c.buoyancy) return;
    const std::string nm = "T" + std::to_string(c.buoyancy_scalar) + "_OLD";
    const double* T = c.F(nm.c_str());
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const int64_t o = G.ip3;
        double* uo = c.F("UO") + o; double* vo = c.F("VO") + o; double* wo = c.F("WO") + o;
        const double* t = T + o;
        const int nfro = G.bc[1], nbac = G.bc[2], nrgt = G.bc[3], nlft = G.bc[4], nbot = G.bc[5], ntop = G.bc[6];
        const int nbu = (nbac == 7 || nbac == 3), nlv = (nlft == 7 || nlft == 3), ntw = (ntop == 7 || ntop == 3);
        const int nfu = nfro == 3, nrv = nrgt == 3, nbw = nbot == 3;
        if (std::fabs(c.gravity[0]) > 0.0)
            for (int i = 3 - nfu; i <= ii - 3 + nbu; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3; k <= kk - 2; ++k)
                        uo[IX(k, j, i)] = uo[IX(k, j, i)] + -c.gravity[0] * c.beta * (0.5 * (t[IX(k, j, i)] + t[IX(k, j, i + 1)]));
        if (std::fabs(c.gravity[1]) > 0.0)
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3 - nrv; j <= jj - 3 + nlv; ++j)
                    for (int k = 3; k <= kk - 2; ++k)
                        vo[IX(k, j, i)] = vo[IX(k, j, i)] + -c.gravity[1] * c.beta * (0.5 * (t[IX(k, j, i)] + t[IX(k, j + 1, i)]));
        if (std::fabs(c.gravity[2]) > 0.0)
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3 - nbw; k <= kk - 3 + ntw; ++k)
                        wo[IX(k, j, i)] = wo[IX(k, j, i)] + -c.gravity[2] * c.beta * (0.5 * (t[IX(k, j, i)] + t[IX(k + 1, j, i)]));
    }
}

// coriolis_grid (coriolisterm_mod.F90:100-189): -2 omega x u with the other
// components averaged to the velocity point
void coriolisterm(Ctx& c) {
    if (!c.coriolis) return;
    const double* om = c.omega;
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const int64_t o = G.ip3;
        double* uo = c.F("UO") + o; double* vo = c.F("VO") + o; double* wo = c.F("WO") + o;
        const double* u = c.F("U") + o; const double* v = c.F("V") + o; const double* w = c.F("W") + o;
        const int nfro = G.bc[1], nbac = G.bc[2], nrgt = G.bc[3], nlft = G.bc[4], nbot = G.bc[5], ntop = G.bc[6];
        const int nbu = (nbac == 7 || nbac == 3), nlv = (nlft == 7 || nlft == 3), ntw = (ntop == 7 || ntop == 3);
        const int nfu = nfro == 3, nrv = nrgt == 3, nbw = nbot == 3;
#define A(a, k, j, i) a[IX(k, j, i)]
        if (std::fabs(om[1]) + std::fabs(om[2]) > 0.0)
            for (int i = 3 - nfu; i <= ii - 3 + nbu; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3; k <= kk - 2; ++k) {
                        const double v2 = 0.25 * (A(v, k, j - 1, i) + A(v, k, j - 1, i + 1) + A(v, k, j, i) + A(v, k, j, i + 1));
                        const double v3 = 0.25 * (A(w, k - 1, j, i) + A(w, k - 1, j, i + 1) + A(w, k, j, i) + A(w, k, j, i + 1));
                        A(uo, k, j, i) = A(uo, k, j, i) + -2.0 * (om[1] * v3 - om[2] * v2);
                    }
        if (std::fabs(om[0]) + std::fabs(om[2]) > 0.0)
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3 - nrv; j <= jj - 3 + nlv; ++j)
                    for (int k = 3; k <= kk - 2; ++k) {
                        const double v1 = 0.25 * (A(u, k, j, i - 1) + A(u, k, j + 1, i - 1) + A(u, k, j, i) + A(u, k, j + 1, i));
                        const double v3 = 0.25 * (A(w, k - 1, j, i) + A(w, k - 1, j + 1, i) + A(w, k, j, i) + A(w, k, j + 1, i));
                        A(vo, k, j, i) = A(vo, k, j, i) + -2.0 * (om[2] * v1 - om[0] * v3);
                    }
        if (std::fabs(om[0]) + std::fabs(om[1]) > 0.0)
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3 - nbw; k <= kk - 3 + ntw; ++k) {
                        const double v1 = 0.25 * (A(u, k, j, i - 1) + A(u, k + 1, j, i - 1) + A(u, k, j, i) + A(u, k + 1, j, i));
                        const double v2 = 0.25 * (A(v, k, j - 1, i) + A(v, k + 1, j - 1, i) + A(v, k, j, i) + A(v, k + 1, j, i));
                        A(wo, k, j, i) = A(wo, k, j, i) + -2.0 * (om[0] * v2 - om[1] * v1);
                    }
#undef A
    }
}

// ---- scalar transport (src/scalar/timeintegrate_scalar_mod.F90) -----------

// scacore_mod.F90:232-262 prt: the turbulent Prandtl number (default-kind
// literals of the Kays/Crawford fit widened)
double prt(const Ctx& c, const Ctx::ScalarDef& s, double gtgmol) {
    if (s.kayscrawford == 0) return c.prturb;
    if (gtgmol > 0.0)
        return (double)0.5882f + (double)0.228f * gtgmol -
               (double)0.0441f * (gtgmol * gtgmol) * (1.0 - std::exp((double)(-5.165f) / gtgmol));
    return s.prmol;
}

// timeintegrate_scalar_mod.F90:229-476 tstsca4_grid: the face fluxes QTU,
// QTV, QTW of scalar t (central convection, diffusion with the LES
// diffusivity where a model runs, the upwind correction at PAR faces)
void tstsca4_grid(Ctx& c, int g, const Ctx::ScalarDef& sd, const double* T) {
    const Grid& G = c.g[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int64_t o = G.ip3;
    double* qtu = c.F("QTU") + o; double* qtv = c.F("QTV") + o; double* qtw = c.F("QTW") + o;
    const double* t = T + o;
    const double* u = c.F("U") + o; const double* v = c.F("V") + o; const double* w = c.F("W") + o;
    const double* gg = c.F("G") + o; const double* bt = c.F("BT") + o;
    const double* ddx = c.L("DDX") + G.ipx - 1; const double* ddy = c.L("DDY") + G.ipy - 1;
    const double* ddz = c.L("DDZ") + G.ipz - 1;
    const double* rdx = c.L("RDX") + G.ipx - 1; const double* rdy = c.L("RDY") + G.ipy - 1;
    const double* rdz = c.L("RDZ") + G.ipz - 1;
    const double gmol = c.prm.gmol, rho = c.prm.rho;
    const int nfro = G.bc[1], nbac = G.bc[2], nrgt = G.bc[3], nlft = G.bc[4], nbot = G.bc[5], ntop = G.bc[6];
    const int nfu = nfro == 7, nbu = nbac == 7, nrv = nrgt == 7, nlv = nlft == 7, nbw = nbot == 7, ntw = ntop == 7;
#define A(a, k, j, i) a[IX(k, j, i)]
    for (int i = 1; i <= ii; ++i)
        for (int j = 1; j <= jj; ++j)
            for (int k = 1; k <= kk; ++k) A(qtu, k, j, i) = A(qtv, k, j, i) = A(qtw, k, j, i) = 0.0;
    auto gsca = [&](double g0, double g1) {
        const double gscamol = gmol / rho / sd.prmol;
        if (c.ilesmodel == 0) return gscamol;
        const double gtgmolp = (g0 - gmol) / gmol, gtgmoln = (g1 - gmol) / gmol;
        const double gs = gscamol + (g1 + g0 - 2.0 * gmol) / rho / (prt(c, sd, gtgmoln) + prt(c, sd, gtgmolp));
        return std::max(gscamol, gs);
    };
    for (int i = 3 - nfu; i <= ii - 3 + nbu; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                const double gs = gsca(A(gg, k, j, i), A(gg, k, j, i + 1));
                const double adv = (ddy[j] * ddz[k]) * A(u, k, j, i) * 0.5 * (A(t, k, j, i) + A(t, k, j, i + 1));
                const double area = A(bt, k, j, i) * A(bt, k, j, i + 1) * (ddy[j] * ddz[k]);
                const double diff = -gs * rdx[i] * (A(t, k, j, i + 1) - A(t, k, j, i)) * area;
                A(qtu, k, j, i) = adv + diff;
            }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3 - nrv; j <= jj - 3 + nlv; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                const double gs = gsca(A(gg, k, j, i), A(gg, k, j + 1, i));
                const double adv = (ddx[i] * ddz[k]) * A(v, k, j, i) * 0.5 * (A(t, k, j, i) + A(t, k, j + 1, i));
                const double area = A(bt, k, j, i) * A(bt, k, j + 1, i) * (ddx[i] * ddz[k]);
                const double diff = -gs * rdy[j] * (A(t, k, j + 1, i) - A(t, k, j, i)) * area;
                A(qtv, k, j, i) = adv + diff;
            }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3 - nbw; k <= kk - 3 + ntw; ++k) {
                const double gs = gsca(A(gg, k, j, i), A(gg, k + 1, j, i));
                const double adv = (ddx[i] * ddy[j]) * A(w, k, j, i) * 0.5 * (A(t, k, j, i) + A(t, k + 1, j, i));
                const double area = A(bt, k, j, i) * A(bt, k + 1, j, i) * (ddx[i] * ddy[j]);
                const double diff = -gs * rdz[k] * (A(t, k + 1, j, i) - A(t, k, j, i)) * area;
                A(qtw, k, j, i) = adv + diff;
            }
    // PAR faces: upwind in the layer next to the coarse grid
    if (nfro == 8)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                const int i = 3;
                A(qtu, k, j, i) = A(qtu, k, j, i) + (ddy[j] * ddz[k]) * (A(u, k, j, i) - std::fabs(A(u, k, j, i))) *
                                                        0.5 * 0.5 * (-A(t, k, j, i) + A(t, k, j, i + 1));
            }
    if (nbac == 8)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                const int i = ii - 3;
                A(qtu, k, j, i) = A(qtu, k, j, i) + (ddy[j] * ddz[k]) * (A(u, k, j, i) + std::fabs(A(u, k, j, i))) *
                                                        0.5 * 0.5 * (A(t, k, j, i) - A(t, k, j, i + 1));
            }
    if (nrgt == 8)
        for (int i = 3; i <= ii - 2; ++i)
            for (int k = 3; k <= kk - 2; ++k) {
                const int j = 3;
                A(qtv, k, j, i) = A(qtv, k, j, i) + (ddx[i] * ddz[k]) * (A(v, k, j, i) - std::fabs(A(v, k, j, i))) *
                                                        0.5 * 0.5 * (-A(t, k, j, i) + A(t, k, j + 1, i));
            }
    if (nlft == 8)
        for (int i = 3; i <= ii - 2; ++i)
            for (int k = 3; k <= kk - 2; ++k) {
                const int j = jj - 3;
                A(qtv, k, j, i) = A(qtv, k, j, i) + (ddx[i] * ddz[k]) * (A(v, k, j, i) + std::fabs(A(v, k, j, i))) *
                                                        0.5 * 0.5 * (A(t, k, j, i) - A(t, k, j + 1, i));
            }
    if (nbot == 8)
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j) {
                const int k = 3;
                A(qtw, k, j, i) = A(qtw, k, j, i) + (ddx[i] * ddy[j]) * (A(w, k, j, i) - std::fabs(A(w, k, j, i))) *
                                                        0.5 * 0.5 * (-A(t, k, j, i) + A(t, k + 1, j, i));
            }
    if (ntop == 8)
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j) {
                const int k = kk - 3;
                A(qtw, k, j, i) = A(qtw, k, j, i) + (ddx[i] * ddy[j]) * (A(w, k, j, i) + std::fabs(A(w, k, j, i))) *
                                                        0.5 * 0.5 * (A(t, k, j, i) - A(t, k + 1, j, i));
            }
#undef A
}

// bound_scalar_mod.F90:103-123 (and the right / bottom twins): on a PAR
// face the coarse flux of the buffer split over the four fine faces by
// their open areas
void bound_scaflux_par(Ctx& c, int ilevel) {
    const double* BT = c.F("BT");
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel) continue;
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const double* bt = BT + G.ip3;
        for (int f = 1; f <= 6; ++f) {
            if (G.bc[f] != MGLET_BC_PAR) continue;
            const int d = (f - 1) / 2;
            const char* fn = d == 0 ? "QTU" : (d == 1 ? "QTV" : "QTW");
            double* q = c.F(fn) + G.ip3;
            const double* buf = buffer_of(c, fn).data() + c.bufoff[6 * (g - 1) + f - 1];
            const int n = d == 0 ? ii : (d == 1 ? jj : kk);
            const int p3 = f % 2 == 1 ? 3 : n - 2, ps = f % 2 == 1 ? 2 : n - 2;
            const int na = d == 0 ? jj : ii, nq = d == 2 ? jj : kk;
            auto at = [&](int p, int a, int qq) -> int64_t {
                if (d == 0) return IX(qq, a, p);
                if (d == 1) return IX(qq, p, a);
                return IX(p, qq, a);
            };
            for (int a = 3; a <= na - 2; a += 2)
                for (int qq = 3; qq <= nq - 2; qq += 2) {
                    const double a1 = bt[at(p3, a, qq)], a2 = bt[at(p3, a, qq + 1)];
                    const double a3 = bt[at(p3, a + 1, qq)], a4 = bt[at(p3, a + 1, qq + 1)];
                    const double tot = a1 + a2 + a3 + a4;
                    const double qtot = buf[(qq - 1) + (int64_t)(a - 1) * nq];
                    auto d0 = [&](double x) { return tot == 0.0 ? 0.0 : x / tot; };
                    q[at(ps, a, qq)] = d0(a1) * qtot;
                    q[at(ps, a, qq + 1)] = d0(a2) * qtot;
                    q[at(ps, a + 1, qq)] = d0(a3) * qtot;
                    q[at(ps, a + 1, qq + 1)] = d0(a4) * qtot;
                }
        }
    }
}

// wernerwengle_mod.F90:92-122 qwallfix: the wall heat flux of the wall model
double qwallfix(const Ctx& c, double tbound, double tfluid, double uquer, double dds, double prmol) {
    const WernerWengle q = werner_wengle(c.prm.gmol, c.prm.rho);
    const double gmol = c.prm.gmol, rho = c.prm.rho, cwa = 8.3, cwb = q.cwb;
    const double cpo1 = 1.0 - cwb, cpo2 = 1.0 + cwb;
    const double uquern = std::fabs(uquer);
    if (uquern >= q.cpo6 / dds) {
        const double ddsb = std::pow(dds, -cwb);
        const double tauwin = rho * std::pow(ddsb * (q.cpo4 * uquern + q.cpo5 / dds), q.cpo8);
        const double sm = gmol / std::sqrt(tauwin * rho) * std::pow(cwa, 1.0 / (1.0 - cwb));
        const double fsm = 1.0 / (dds * dds) *
                           (0.5 * (sm * sm) * prmol + std::pow(std::sqrt(tauwin * rho) / gmol, -cpo1) * cwa / cpo2 *
                                                          (std::pow(dds, cpo2) - std::pow(sm, cpo2)));
        return gmol / rho * (tbound - tfluid) / dds / fsm;
    }
    return gmol / rho / prmol * (tbound - tfluid) * 2.0 / dds;
}

// bound_scalar_mod.F90:124-210 (and the right / bottom twins): the SWA and
// SIO conditions of scalar l on the grids of ilevel, from the scalar's
// boundary buffer (a wall or inflow value, or a flux)
void bound_scaflux_walls(Ctx& c, int ilevel, int l, const double* T) {
    if (c.scabc_kind.empty()) return;
    const Ctx::ScalarDef& sd = c.sca[l];
    const std::vector<double>& tb = buffer_of(c, sd.name);
    const double gmol = c.prm.gmol, rho = c.prm.rho;
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (G.level != ilevel) continue;
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const int64_t o = G.ip3;
        const double* t = T + o;
        const double* u = c.F("U") + o; const double* v = c.F("V") + o; const double* w = c.F("W") + o;
        const double* dxs[3] = {c.L("DX") + G.ipx - 1, c.L("DY") + G.ipy - 1, c.L("DZ") + G.ipz - 1};
        const double* dd[3] = {c.L("DDX") + G.ipx - 1, c.L("DDY") + G.ipy - 1, c.L("DDZ") + G.ipz - 1};
        for (int f = 1; f <= 6; ++f) {
            const int kind = c.scabc_kind[6 * (g - 1) + f - 1];
            if (kind == 0) continue;
            const int type = c.scabc_type[(6 * (g - 1) + f - 1) * 9 + l];
            const int d = (f - 1) / 2;
            const double dir = f % 2 == 1 ? -1.0 : 1.0;
            const int n = d == 0 ? ii : (d == 1 ? jj : kk);
            const int p2 = f % 2 == 1 ? 2 : n - 2, p3 = f % 2 == 1 ? 3 : n - 2;
            const int na = d == 0 ? jj : ii, nq = d == 2 ? jj : kk;
            const double* A1 = d == 0 ? dd[1] : dd[0];      // ddy (x faces) or ddx
            const double* A2 = d == 2 ? dd[1] : dd[2];      // ddz, or ddy (z faces)
            double* qf = c.F(d == 0 ? "QTU" : (d == 1 ? "QTV" : "QTW")) + o;
            const double* un = d == 0 ? u : (d == 1 ? v : w);
            const double* b = tb.data() + c.bufoff[6 * (g - 1) + f - 1];
            auto at = [&](int p, int a, int qq) -> int64_t {
                if (d == 0) return IX(qq, a, p);
                if (d == 1) return IX(qq, p, a);
                return IX(p, qq, a);
            };
            const bool les_wall = kind == 1 && type == 0 && c.ilesmodel != 0;
            for (int a = les_wall ? 2 : 1; a <= na; ++a)
                for (int qq = les_wall ? 2 : 1; qq <= nq; ++qq) {
                    const double tbv = b[(qq - 1) + (int64_t)(a - 1) * nq];
                    const double tin = t[at(p3, a, qq)];
                    double r;
                    if (type == 1) {
                        const double area = A1[a] * A2[qq];
                        r = -dir * tbv * area;
                    } else if (kind == 1 && c.ilesmodel == 0) {
                        const double gamma2dx = 2.0 * gmol / rho / sd.prmol / dxs[d][p2];
                        const double diff = gamma2dx * (tbv - tin);
                        r = -dir * diff * A1[a] * A2[qq];
                    } else if (kind == 1) {
                        // the two tangential velocities at the cell centre of the first layer
                        double s1, s2;
                        if (d == 0) {
                            const int k = qq, j = a, i = p3;
                            s1 = w[IX(k - 1, j, i)] + (w[IX(k, j, i)] - w[IX(k - 1, j, i)]) / dd[2][k] * dd[2][k - 1] * 0.5;
                            s2 = v[IX(k, j - 1, i)] + (v[IX(k, j, i)] - v[IX(k, j - 1, i)]) / dd[1][j] * dd[1][j - 1] * 0.5;
                        } else if (d == 1) {
                            const int k = qq, i = a, j = p3;
                            s1 = w[IX(k - 1, j, i)] + (w[IX(k, j, i)] - w[IX(k - 1, j, i)]) / dd[2][k] * dd[2][k - 1] * 0.5;
                            s2 = u[IX(k, j, i - 1)] + (u[IX(k, j, i)] - u[IX(k, j, i - 1)]) / dd[0][i] * dd[0][i - 1] * 0.5;
                        } else {
                            const int j = qq, i = a, k = p3;
                            s1 = u[IX(k, j, i - 1)] + (u[IX(k, j, i)] - u[IX(k, j, i - 1)]) / dd[0][i] * dd[0][i - 1] * 0.5;
                            s2 = v[IX(k, j - 1, i)] + (v[IX(k, j, i)] - v[IX(k, j - 1, i)]) / dd[1][j] * dd[1][j - 1] * 0.5;
                        }
                        const double uquer = std::sqrt(s1 * s1 + s2 * s2);
                        const double area = A1[a] * A2[qq];
                        r = -dir * qwallfix(c, tbv, tin, uquer, dd[d][p3], sd.prmol) * area;
                    } else {
                        const double gamma = gmol / rho / sd.prmol;
                        const double unv = un[at(p2, a, qq)];
                        const double tout = -dir * unv >= 0.0 ? 2.0 * tbv - tin : tin;
                        const double adv = -dir * unv * 0.5 * (tout + tin);
                        const double diff = gamma * (tout - tin) / dxs[d][p2];
                        const double area = A1[a] * A2[qq];
                        r = -dir * (adv + diff) * area;
                    }
                    qf[at(p2, a, qq)] = r;
                }
        }
    }
}

// timeintegrate_scalar (timeintegrate_scalar_mod.F90:17-108) for every
// scalar: fluxes, PAR fluxes from the parent, flux balance, source, RK
// update, restriction and the corner connect
// ---------------------------------------------------------------------------
// Ghost-cell IB of the scalars: blockbt (blockbt_mod.F90:11-208), maskbt
// (scacore_mod.F90:265-306) and set_scastencils (gc_scastencils_mod.F90:
// 949-1125).
constexpr int kScaIsize = 9, kScaRsize = 8, kScaNperi = 6;

// BT from BP: a cell is open where it or a face neighbour is fluid
// (blockbt_grid, :73-91, on 2..n-1), connected per level; on the finer levels
// the cells behind a PAR face open where the coarse cell lets a scalar flux
// through (open_scalarflux_boundary, :93-208, from ctof of BT).
int blockbt(Ctx& c) {
    double* BT = c.F("BT");
    const double* BP = c.F("BP");
    auto mx = [](double a, double b) { return a < b ? b : a; };
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const double* bp = BP + G.ip3;
        double* bt = BT + G.ip3;
        for (int i = 2; i <= ii - 1; ++i)
            for (int j = 2; j <= jj - 1; ++j)
                for (int k = 2; k <= kk - 1; ++k)
                    bt[IX(k, j, i)] = mx(mx(mx(mx(mx(mx(bp[IX(k, j, i)], bp[IX(k, j, i + 1)]), bp[IX(k, j, i - 1)]),
                                                  bp[IX(k, j + 1, i)]),
                                               bp[IX(k, j - 1, i)]),
                                            bp[IX(k + 1, j, i)]),
                                         bp[IX(k - 1, j, i)]);
    }
    for (int l = c.minlevel; l <= c.maxlevel; ++l)
        connect(c, l, 2, nullptr, nullptr, nullptr, BT, nullptr, nullptr, true, false, 0);
    c.f3["BTH"].assign(c.idim3d, 0.0);
    for (int l = c.minlevel; l <= c.maxlevel; ++l) {
        std::fill(c.f3["BTH"].begin(), c.f3["BTH"].end(), -1.0);
        if (c.minlevel != c.maxlevel) ctof(c, l, "BTH", "BT");
        const double* H = c.F("BTH");
        BT = c.F("BT");
        for (int g = 1; g <= c.ngrid; ++g) {
            const Grid& G = c.g[g];
            if (G.level != l) continue;
            const int kk = G.kk, jj = G.jj, ii = G.ii;
            const double* hf = H + G.ip3;
            double* bt = BT + G.ip3;
            // faces front, back, right, left, bottom, top: the receiver
            // layer (3 or n-2) from the ghost (2 or n-1) and itself
            for (int f = 1; f <= 6; ++f) {
                if (G.bc[f] != MGLET_BC_PAR) continue;
                const int ax = (f - 1) / 2, hi = (f - 1) % 2;
                const int n = ax == 0 ? ii : (ax == 1 ? jj : kk);
                const int p2 = hi ? n - 1 : 2, p3 = hi ? n - 2 : 3;
                const int na = ax == 0 ? jj : ii, nb = ax == 2 ? jj : kk;   // the two other axes
                for (int a = 2; a <= na - 1; ++a)
                    for (int b = 2; b <= nb - 1; ++b) {
                        int k2, j2, i2, k3, j3, i3;
                        if (ax == 0) { i2 = p2; i3 = p3; j2 = j3 = a; k2 = k3 = b; }
                        else if (ax == 1) { j2 = p2; j3 = p3; i2 = i3 = a; k2 = k3 = b; }
                        else { k2 = p2; k3 = p3; i2 = i3 = a; j2 = j3 = b; }
                        const double c2 = hf[IX(k2, j2, i2)], c3 = hf[IX(k3, j3, i3)];
                        if (c2 < -0.5 || c3 < -0.5)
                            return fail(MGLET_ERR_ARG, "blockbt: a fine cell behind a PAR face has no coarse value");
                        bt[IX(k3, j3, i3)] = mx(c2 * c3, bt[IX(k3, j3, i3)]);
                    }
            }
        }
        connect(c, l, 2, nullptr, nullptr, nullptr, BT, nullptr, nullptr, true, false, 0);
    }
    return 0;
}

// maskbt_grid (scacore_mod.F90:289-306): t *= bt on 3..n-2
void maskbt(Ctx& c, double* T) {
    const double* BT = c.F("BT");
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        double* t = T + G.ip3;
        const double* bt = BT + G.ip3;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k) t[IX(k, j, i)] = t[IX(k, j, i)] * bt[IX(k, j, i)];
    }
}

// set_scastencils(ctyp, sca, t= or qtt=) (:949-1125): per grid the cells in
// list order; t: a fixed-value body sets var(intcell) from its stencil
// cells and acoeffvel * value; qtt: a fixed-flux body adds areabyvol *
// value.  A cell without a body (body <= 0) counts as fixed flux 0.
int sca_stencils(Ctx& c, char ctyp, const Ctx::ScalarDef& sd, double* T, double* QTT) {
    for (int g = 1; g <= c.ngrid; ++g) {
        if ((int)c.scal.size() <= g) break;
        const Ctx::ScaList& L = c.scal[g];
        const std::vector<double>& xr = ctyp == 'C' ? L.xpolr : L.xpolrvel;
        double* var = (T ? T : QTT) + c.g[g].ip3;
        for (int cell = 0; cell < L.ncells; ++cell) {
            const int64_t* xi = L.xpoli.data() + (size_t)cell * kScaIsize;
            const double* r = xr.data() + (size_t)cell * kScaRsize;
            const int64_t intcell = xi[0], body = xi[1];
            int bctype = 1;
            double bcval = 0.0;
            if (body > 0) {
                if (body > (int64_t)sd.geo_flag.size())
                    return fail(MGLET_ERR_ARG, "set_scastencils: a body without a scalar condition");
                bctype = sd.geo_flag[body - 1];
                bcval = sd.geo_value[body - 1];
            }
            if (T) {
                double val = 0.0;
                for (int64_t n = 1; n <= xi[2]; ++n) val = val + var[xi[2 + n] - 1] * r[n];
                const double coeff = r[1 + kScaNperi];
                if (bctype == 0) {
                    val = val + coeff * bcval;
                    var[intcell - 1] = val;
                }
            } else if (bctype == 1) {
                var[intcell - 1] = var[intcell - 1] + r[0] * bcval;
            }
        }
    }
    return 0;
}

int timeintegrate_scalar(Ctx& c, double dt, int irk, const mglet_rk_scheme* rk) {
    double frhs, fu, dtrk, dtrki;
    if (irk > rk->nrk || irk < 1) return fail(MGLET_ERR_ARG, "timeintegrate_scalar: irk out of range");
    frhs = rk->a[irk - 1];
    fu = rk->b[irk - 1];
    dtrk = irk < rk->nrk ? rk->c[irk] : 1.0;
    dtrki = dtrk - rk->c[irk - 1];
    (void)dtrki;
    const char* qn[3] = {"QTU", "QTV", "QTW"};
    const char* none[3] = {nullptr, nullptr, nullptr};
    for (size_t l = 0; l < c.sca.size(); ++l) {
        const Ctx::ScalarDef& sd = c.sca[l];
        double* T = c.F(sd.name.c_str());
        double* DT = c.F(("D" + sd.name).c_str());
        c.f3[sd.name + "_OLD"] = c.f3[sd.name];   // :56-57, for the Boussinesq term
        T = c.F(sd.name.c_str());
        DT = c.F(("D" + sd.name).c_str());
        for (int g = 1; g <= c.ngrid; ++g) tstsca4_grid(c, g, sd, T);
        for (int lv = c.minlevel; lv <= c.maxlevel; ++lv) {
            parent(c, lv, qn, none, false);
            bound_scaflux_par(c, lv);
            bound_scaflux_walls(c, lv, (int)l, T);
        }
        double* qtt = c.F("QTT");
        std::fill(c.f3["QTT"].begin(), c.f3["QTT"].end(), 0.0);
        std::vector<const double*> srcf;
        for (const auto& src : sd.sources) srcf.push_back(src.first.empty() ? nullptr : c.F(src.first.c_str()));
        for (int g = 1; g <= c.ngrid; ++g) {
            const Grid& G = c.g[g];
            const int kk = G.kk, jj = G.jj, ii = G.ii;
            const int64_t o = G.ip3;
            const double* qtu = c.F("QTU") + o; const double* qtv = c.F("QTV") + o;
            const double* qtw = c.F("QTW") + o;
            const double* rddx = c.L("RDDX") + G.ipx - 1; const double* rddy = c.L("RDDY") + G.ipy - 1;
            const double* rddz = c.L("RDDZ") + G.ipz - 1;
            for (int i = 3; i <= ii - 2; ++i)
                for (int j = 3; j <= jj - 2; ++j)
                    for (int k = 3; k <= kk - 2; ++k) {
                        const double net = qtu[IX(k, j, i - 1)] - qtu[IX(k, j, i)] + qtv[IX(k, j - 1, i)] -
                                           qtv[IX(k, j, i)] + qtw[IX(k - 1, j, i)] - qtw[IX(k, j, i)];
                        double q = rddz[k] * rddy[j] * rddx[i] * net;
                        // sourceterm (:549-634), the sources in order
                        for (size_t s = 0; s < srcf.size(); ++s)
                            q = srcf[s] ? q + sd.sources[s].second * srcf[s][o + IX(k, j, i)]
                                        : q + sd.sources[s].second;
                        qtt[o + IX(k, j, i)] = q;
                    }
        }
        // timeintegrate_scalar_mod.F90:71-73: the flux condition of the bodies
        if (c.ibtype == 1)
            if (int rc = sca_stencils(c, 'P', sd, nullptr, qtt)) return rc;
        rkstep(T, DT, qtt, c.idim3d, frhs, dt * fu);
        maskbt(c, T);   // :84 (BT = 1 without the ghost-cell IB)
        if (c.ibtype == 1) {   // :87-90: the value condition of the bodies
            connect(c, 0, 2, nullptr, nullptr, nullptr, T, nullptr, nullptr, true, false, 0);
            if (int rc = sca_stencils(c, 'P', sd, T, nullptr)) return rc;
        }
        for (int l = c.maxlevel; l > c.minlevel; --l) ftoc_one(c, l, sd.name, sd.name, 'T');
        connect(c, 0, 2, nullptr, nullptr, nullptr, T, nullptr, nullptr, true, false, 0);
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Ghost-cell IB runtime (gc_flowstencils_mod.F90:922-1604, timeintegration_mod
// :255-303).  The lists are walked cell after cell, as the reference does: a
// ghost value may feed a later stencil of the same list.
void wmxpolsol(double* var, const GcList& L, const std::vector<double>& xr) {
    size_t pi = 0, pr = 0;
    for (int cell = 0; cell < L.ncells; ++cell) {
        const int64_t intcell = L.xpoli[pi++];
        const int64_t n = L.xpoli[pi++];
        double flux = 0.0;
        for (int64_t q = 0; q < n; ++q) {
            const int64_t st = L.xpoli[pi++];
            flux = flux + var[st - 1] * xr[pr++];
        }
        flux = flux + xr[pr++];
        var[intcell - 1] = flux;
    }
}

void wmxpolsolrlx(double* var, int ncells, const std::vector<double>& oldsol,
                  const std::vector<int64_t>& poldsol) {
    for (int q = 0; q < ncells; ++q) var[poldsol[q] - 1] = oldsol[q];
}

void wmxpolsolsav(const double* var, const GcList& L, std::vector<double>& oldsol,
                  std::vector<int64_t>& poldsol) {
    oldsol.resize(L.ncells);
    poldsol.resize(L.ncells);
    size_t pi = 0;
    for (int q = 0; q < L.ncells; ++q) {
        const int64_t idx = L.xpoli[pi++];
        const int64_t n = L.xpoli[pi++];
        pi += (size_t)n;
        poldsol[q] = idx;
        oldsol[q] = var[idx - 1];
    }
}

// gc_flowstencils_mod.F90:1113-1183 wmxpolsolcorr: spread the divergence of a
// cut cell over its open face areas
int wmxpolsolcorr(const Grid& G, double* u, double* v, double* w, const double* ddx,
                  const double* ddy, const double* ddz, const GcFlux& F) {
    const int kk = G.kk, jj = G.jj;
    const int64_t ishift = (int64_t)jj * kk, jshift = kk, kshift = 1;
    size_t pi = 0, pr = 0;
    for (int cell = 0; cell < F.ncells; ++cell) {
        pi++;   // foundnr
        const int64_t intcell = F.fxpoli[pi++];
        const double ax1 = F.fxpolr[pr++], ax2 = F.fxpolr[pr++], ay1 = F.fxpolr[pr++];
        const double ay2 = F.fxpolr[pr++], az1 = F.fxpolr[pr++], az2 = F.fxpolr[pr++];
        const double acoeffstc = F.fxpolr[pr++];
        const int64_t c0 = intcell - 1;
        const int k = (int)(c0 % kk) + 1, j = (int)((c0 / kk) % jj) + 1, i = (int)(c0 / ((int64_t)kk * jj)) + 1;
        double div = ddy[j] * ddz[k] * (u[c0] - u[c0 - ishift]) +
                     ddx[i] * ddz[k] * (v[c0] - v[c0 - jshift]) +
                     ddx[i] * ddy[j] * (w[c0] - w[c0 - kshift]) + acoeffstc;
        const double sarea = ax1 + ax2 + ay1 + ay2 + az1 + az2;
        if (sarea < std::numeric_limits<double>::min())
            return fail(MGLET_ERR_ARG, "wmxpolsolcorr: cut cell without open area");
        div = div / sarea;
        u[c0] = u[c0] - ax1 * div / (ddy[j] * ddz[k]);
        u[c0 - ishift] = u[c0 - ishift] + ax2 * div / (ddy[j] * ddz[k]);
        v[c0] = v[c0] - ay1 * div / (ddx[i] * ddz[k]);
        v[c0 - jshift] = v[c0 - jshift] + ay2 * div / (ddx[i] * ddz[k]);
        w[c0] = w[c0] - az1 * div / (ddx[i] * ddy[j]);
        w[c0 - kshift] = w[c0 - kshift] + az2 * div / (ddx[i] * ddy[j]);
    }
    return 0;
}

// setibvalues_level (:1456-1485) modes F, R, S, C and wmxpolquadvel modes X,
// Y, Z (setpointvalues_all, :1370-1390)
// on the grids of ilevel (0: every grid)
int gc_level(Ctx& c, char mode, double* U, double* V, double* W, int ilevel = 0) {
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        if (ilevel && G.level != ilevel) continue;
        double* f[3] = {U + G.ip3, V + G.ip3, W + G.ip3};
        if (mode == 'C') {
            if (int rc = wmxpolsolcorr(G, f[0], f[1], f[2], c.L("DDX") + G.ipx - 1,
                                       c.L("DDY") + G.ipy - 1, c.L("DDZ") + G.ipz - 1, c.gcf[g]))
                return rc;
            continue;
        }
        for (int cmp = 0; cmp < 3; ++cmp) {
            GcList& L = c.gcl[g][cmp];
            switch (mode) {
            case 'F': wmxpolsol(f[cmp], L, L.xpolr); break;
            case 'X': wmxpolsol(f[cmp], L, L.xpolrvel); break;
            case 'R':
                if (L.poldsol.size() < (size_t)L.ncells)
                    return fail(MGLET_ERR_ARG, "gc: restore R before any save S (setibvalues first)");
                wmxpolsolrlx(f[cmp], L.ncells, L.oldsol, L.poldsol);
                break;
            case 'Y':
                if (L.poldsolvel.size() < (size_t)L.ncells)
                    return fail(MGLET_ERR_ARG, "gc: restore Y before any save Z (setpointvalues first)");
                wmxpolsolrlx(f[cmp], L.ncells, L.oldsolvel, L.poldsolvel);
                break;
            case 'S': wmxpolsolsav(f[cmp], L, L.oldsol, L.poldsol); break;
            case 'Z': wmxpolsolsav(f[cmp], L, L.oldsolvel, L.poldsolvel); break;
            default: return fail(MGLET_ERR_ARG, "gc: unknown mode");
            }
        }
    }
    return 0;
}

// setibvalues (:1393-1438) of the velocity fields U, V, W: per level
// (parent,) extrapolation F and flux correction C, each followed by
// bound_flow and connect; fine to coarse (ftoc, par_ftoc_norm); per level
// again (parent,) C and the save S
int setibvalues(Ctx& c) {
    double *U = c.F("U"), *V = c.F("V"), *W = c.F("W");
    const char* vn[3] = {"U", "V", "W"};
    const char* none[3] = {nullptr, nullptr, nullptr};
    const bool ml = c.minlevel != c.maxlevel;
    auto bound = [&](int l) { bound_flow(c, U, V, W, nullptr, ml ? l : 0); };
    auto conn = [&](int l, int layers, bool corners) {
        connect(c, ml ? l : 0, layers, U, V, W, nullptr, nullptr, nullptr, corners, false, 0);
    };
    for (int l = c.minlevel; l <= c.maxlevel; ++l) {
        if (ml) parent(c, l, vn, none, false);
        bound(l);
        conn(l, 2, false);
        if (int rc = gc_level(c, 'F', U, V, W, l)) return rc;
        bound(l);
        conn(l, 1, true);
        if (int rc = gc_level(c, 'C', U, V, W, l)) return rc;
        bound(l);
        conn(l, 1, true);
    }
    for (int l = c.maxlevel; l > c.minlevel; --l) {
        for (int q = 0; q < 3; ++q) ftoc_one(c, l, vn[q], vn[q], "UVW"[q]);
        par_ftoc_norm(c, l, U, V, W, false);
    }
    for (int l = c.minlevel; l <= c.maxlevel; ++l) {
        if (ml) parent(c, l, vn, none, false);
        bound(l);
        conn(l, 1, true);
        if (int rc = gc_level(c, 'C', U, V, W, l)) return rc;
        bound(l);
        conn(l, 1, true);
        if (int rc = gc_level(c, 'S', U, V, W, l)) return rc;
    }
    return 0;
}

// setpointvalues (:1323-1367): point values = velocities with the ghost
// cells extrapolated ('X', new) or restored ('Y'), connected and bounded
int setpointvalues(Ctx& c, bool comp_new) {
    c.f3["PWU"] = c.f3["U"];
    c.f3["PWV"] = c.f3["V"];
    c.f3["PWW"] = c.f3["W"];
    // pwu%buffers = u%buffers: bound_flow takes the U, V, W boundary buffers
    double *pu = c.F("PWU"), *pv = c.F("PWV"), *pw = c.F("PWW");
    if (int rc = gc_level(c, comp_new ? 'X' : 'Y', pu, pv, pw)) return rc;
    const bool ml = c.minlevel != c.maxlevel;
    for (int l = c.minlevel; l <= c.maxlevel; ++l) {
        connect(c, ml ? l : 0, 1, pu, pv, pw, nullptr, nullptr, nullptr, false, false, 0);
        bound_flow(c, pu, pv, pw, nullptr, ml ? l : 0);
    }
    if (comp_new) return gc_level(c, 'Z', pu, pv, pw);
    return 0;
}

// timeintegration_mod.F90:277-303 maskbp_grid
void maskbp(Ctx& c, double* U, double* V, double* W, double* P) {
    const double* BP = c.F("BP");
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        double* u = U + G.ip3; double* v = V + G.ip3; double* w = W + G.ip3; double* p = P + G.ip3;
        const double* bp = BP + G.ip3;
        for (int i = 1; i <= ii - 1; ++i)
            for (int j = 1; j <= jj - 1; ++j) {
                for (int k = 1; k <= kk - 1; ++k)
                    u[IX(k, j, i)] = u[IX(k, j, i)] * bp[IX(k, j, i)] * bp[IX(k, j, i + 1)];
                for (int k = 1; k <= kk - 1; ++k)
                    v[IX(k, j, i)] = v[IX(k, j, i)] * bp[IX(k, j, i)] * bp[IX(k, j + 1, i)];
                for (int k = 1; k <= kk - 1; ++k)
                    w[IX(k, j, i)] = w[IX(k, j, i)] * bp[IX(k, j, i)] * bp[IX(k + 1, j, i)];
                for (int k = 1; k <= kk - 1; ++k) p[IX(k, j, i)] = p[IX(k, j, i)] * bp[IX(k, j, i)];
            }
    }
}

// setsdivfield (:1488-1572): the flux-correction constants as a source
// field, connected, and written back so that both sides of a connected face
// correct alike
void setsdivfield(Ctx& c) {
    double* S = c.F("SDIV");
    std::fill(c.f3["SDIV"].begin(), c.f3["SDIV"].end(), 0.0);
    auto walk = [&](bool put) {
        for (int g = 1; g <= c.ngrid; ++g) {
            const Grid& G = c.g[g];
            const int kk = G.kk, jj = G.jj;
            const double* ddx = c.L("DDX") + G.ipx - 1;
            const double* ddy = c.L("DDY") + G.ipy - 1;
            const double* ddz = c.L("DDZ") + G.ipz - 1;
            GcFlux& F = c.gcf[g];
            size_t pi = 0, pr = 0;
            for (int cell = 0; cell < F.ncells; ++cell) {
                pi++;
                const int64_t c0 = F.fxpoli[pi++] - 1;
                pr += 6;
                const int k = (int)(c0 % kk) + 1, j = (int)((c0 / kk) % jj) + 1;
                const int i = (int)(c0 / ((int64_t)kk * jj)) + 1;
                if (put) S[G.ip3 + c0] = F.fxpolr[pr] / (ddx[i] * ddy[j] * ddz[k]);
                else F.fxpolr[pr] = S[G.ip3 + c0] * ddx[i] * ddy[j] * ddz[k];
                pr++;
            }
        }
    };
    walk(true);
    for (int l = c.maxlevel; l > c.minlevel; --l) ftoc_one(c, l, "SDIV", "SDIV", 'S');
    connect(c, 0, 2, nullptr, nullptr, nullptr, S, nullptr, nullptr, true, false, 0);
    walk(false);
}

// ---------------------------------------------------------------------------

// tstle4_mod.F90:532-1753 tstle4_par, a loop-by-loop transcription: on PAR
// faces (code 8) the upwind correction of the second-to-last layer, then the
// momentum-conserving convective fluxes of the coarse velocities,
// redistributed onto the fine cells (back, front, top, bottom, left, right).
// The work arrays start as NaN: a read of an entry the reference does not
// write would reach the result.
void tstle4_par(int kk, int jj, int ii, double* uo, double* vo, double* wo, const double* u,
                const double* v, const double* w, const double* ut, const double* vt,
                const double* wt, const double* dx, const double* dy, const double* dz,
                const double* ddx, const double* ddy, const double* ddz, const double* rdx,
                const double* rdy, const double* rdz, const double* rddx, const double* rddy,
                const double* rddz, int nfro, int nbac, int nrgt, int nlft, int nbot, int ntop) {
    if (nfro != 8 && nbac != 8 && nrgt != 8 && nlft != 8 && nbot != 8 && ntop != 8) return;
    const double wkon = 1.0;
    const int64_t n3 = (int64_t)kk * jj * ii;
    const double nan = std::numeric_limits<double>::quiet_NaN();
    std::vector<double> wcu_(n3, nan), wcv_(n3, nan), wcw_(n3, nan);
    double* wcu = wcu_.data(); double* wcv = wcv_.data(); double* wcw = wcw_.data();
#define A(a, k, j, i) a[IX(k, j, i)]
    double fkdtu, fkdtv, fkdtw, dxi, ddxi, dyj, ddyj, dzk, ddzk, rdzk, rddzk;
    double auy, auz, avx, avz, awx, awy;
    // ---- upwind in the second-to-last layer
    if (nfro == 8) {
        const int i = 4;
        for (int j = 3; j <= jj - 2; ++j) {
            dyj = dy[j]; ddyj = ddy[j];
            fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            for (int k = 3; k <= kk - 2; ++k) {
                dzk = dz[k]; rdzk = rdz[k]; ddzk = ddz[k]; rddzk = rddz[k];
                avx = dyj * ddzk;
                awx = ddyj * dzk;
                const double fvw = avx * (A(ut, k, j, i - 1) + A(ut, k, j + 1, i - 1)) * 0.5;
                const double qv = 0.5 * (fvw - std::fabs(fvw)) *
                                  (0.5 * A(v, k, j, i) - 1.5 * A(v, k, j, i - 1) + A(v, k, j, i - 2)) * 0.5 * 0.5;
                A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (-qv);
                A(vo, k, j, i - 1) = A(vo, k, j, i - 1) + fkdtv * rddzk * (+qv);
                const double fww = awx * (A(ut, k, j, i - 1) + A(ut, k + 1, j, i - 1)) * 0.5;
                const double qw = 0.5 * (fww - std::fabs(fww)) *
                                  (0.5 * A(w, k, j, i) - 1.5 * A(w, k, j, i - 1) + A(w, k, j, i - 2)) * 0.5 * 0.5;
                A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (-qw);
                A(wo, k, j, i - 1) = A(wo, k, j, i - 1) + fkdtw * rdzk * (+qw);
            }
        }
    }
    if (nbac == 8) {
        const int i = ii - 2;
        for (int j = 3; j <= jj - 2; ++j) {
            dyj = dy[j]; ddyj = ddy[j];
            fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            for (int k = 3; k <= kk - 2; ++k) {
                dzk = dz[k]; rdzk = rdz[k]; ddzk = ddz[k]; rddzk = rddz[k];
                avx = dyj * ddzk;
                awx = ddyj * dzk;
                const double fvw = avx * (A(ut, k, j, i - 1) + A(ut, k, j + 1, i - 1)) * 0.5;
                const double qv = 0.5 * (fvw + std::fabs(fvw)) *
                                  (0.5 * A(v, k, j, i - 1) - 1.5 * A(v, k, j, i) + A(v, k, j, i + 1)) * 0.5 * 0.5;
                A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (-qv);
                A(vo, k, j, i - 1) = A(vo, k, j, i - 1) + fkdtv * rddzk * (+qv);
                const double fww = awx * (A(ut, k, j, i - 1) + A(ut, k + 1, j, i - 1)) * 0.5;
                const double qw = 0.5 * (fww + std::fabs(fww)) *
                                  (0.5 * A(w, k, j, i - 1) - 1.5 * A(w, k, j, i) + A(w, k, j, i + 1)) * 0.5 * 0.5;
                A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (-qw);
                A(wo, k, j, i - 1) = A(wo, k, j, i - 1) + fkdtw * rdzk * (+qw);
            }
        }
    }
    if (nrgt == 8) {
        for (int i = 3; i <= ii - 2; ++i) {
            const int j = 4;
            dxi = dx[i]; ddxi = ddx[i];
            fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            for (int k = 3; k <= kk - 2; ++k) {
                dzk = dz[k]; rdzk = rdz[k]; ddzk = ddz[k]; rddzk = rddz[k];
                auy = dxi * ddzk;
                awy = ddxi * dzk;
                const double fus = auy * (A(vt, k, j - 1, i) + A(vt, k, j - 1, i + 1)) * 0.5;
                const double qu = 0.5 * (fus - std::fabs(fus)) *
                                  (0.5 * A(u, k, j, i) - 1.5 * A(u, k, j - 1, i) + A(u, k, j - 2, i)) * 0.5 * 0.5;
                A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (-qu);
                A(uo, k, j - 1, i) = A(uo, k, j - 1, i) + fkdtu * rddzk * (+qu);
                const double fws = awy * (A(vt, k, j - 1, i) + A(vt, k + 1, j - 1, i)) * 0.5;
                const double qw = 0.5 * (fws - std::fabs(fws)) *
                                  (0.5 * A(w, k, j, i) - 1.5 * A(w, k, j - 1, i) + A(w, k, j - 2, i)) * 0.5 * 0.5;
                A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (-qw);
                A(wo, k, j - 1, i) = A(wo, k, j - 1, i) + fkdtw * rdzk * (+qw);
            }
        }
    }
    if (nlft == 8) {
        for (int i = 3; i <= ii - 2; ++i) {
            const int j = jj - 2;
            dxi = dx[i]; ddxi = ddx[i];
            fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            for (int k = 3; k <= kk - 2; ++k) {
                dzk = dz[k]; rdzk = rdz[k]; ddzk = ddz[k]; rddzk = rddz[k];
                auy = dxi * ddzk;
                awy = ddxi * dzk;
                const double fus = auy * (A(vt, k, j - 1, i) + A(vt, k, j - 1, i + 1)) * 0.5;
                const double qu = 0.5 * (fus + std::fabs(fus)) *
                                  (0.5 * A(u, k, j - 1, i) - 1.5 * A(u, k, j, i) + A(u, k, j + 1, i)) * 0.5 * 0.5;
                A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (-qu);
                A(uo, k, j - 1, i) = A(uo, k, j - 1, i) + fkdtu * rddzk * (+qu);
                const double fws = awy * (A(vt, k, j - 1, i) + A(vt, k + 1, j - 1, i)) * 0.5;
                const double qw = 0.5 * (fws + std::fabs(fws)) *
                                  (0.5 * A(w, k, j - 1, i) - 1.5 * A(w, k, j, i) + A(w, k, j + 1, i)) * 0.5 * 0.5;
                A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (-qw);
                A(wo, k, j - 1, i) = A(wo, k, j - 1, i) + fkdtw * rdzk * (+qw);
            }
        }
    }
    if (nbot == 8) {
        for (int i = 3; i <= ii - 2; ++i) {
            dxi = dx[i]; ddxi = ddx[i];
            for (int j = 3; j <= jj - 2; ++j) {
                const int k = 4;
                fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
                fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
                fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
                dyj = dy[j]; ddyj = ddy[j];
                auz = dxi * ddyj;
                avz = ddxi * dyj;
                rdzk = rdz[k]; rddzk = rddz[k];
                const double fub = auz * (A(wt, k - 1, j, i) + A(wt, k - 1, j, i + 1)) * 0.5;
                const double qu = 0.5 * (fub - std::fabs(fub)) *
                                  (0.5 * A(u, k, j, i) - 1.5 * A(u, k - 1, j, i) + A(u, k - 2, j, i)) * 0.5 * 0.5;
                A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (-qu);
                A(uo, k - 1, j, i) = A(uo, k - 1, j, i) + fkdtu * rddzk * (+qu);
                const double fvb = avz * (A(wt, k - 1, j, i) + A(wt, k - 1, j + 1, i)) * 0.5;
                const double qv = 0.5 * (fvb - std::fabs(fvb)) *
                                  (0.5 * A(v, k, j, i) - 1.5 * A(v, k - 1, j, i) + A(v, k - 2, j, i)) * 0.5 * 0.5;
                A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (-qv);
                A(vo, k - 1, j, i) = A(vo, k - 1, j, i) + fkdtv * rddzk * (+qv);
            }
        }
    }
    if (ntop == 8) {
        for (int i = 3; i <= ii - 2; ++i) {
            dxi = dx[i]; ddxi = ddx[i];
            for (int j = 3; j <= jj - 2; ++j) {
                const int k = kk - 2;
                fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
                fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
                fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
                dyj = dy[j]; ddyj = ddy[j];
                auz = dxi * ddyj;
                avz = ddxi * dyj;
                rdzk = rdz[k]; rddzk = rddz[k];
                const double fub = auz * (A(wt, k - 1, j, i) + A(wt, k - 1, j, i + 1)) * 0.5;
                const double qu = 0.5 * (fub + std::fabs(fub)) *
                                  (0.5 * A(u, k - 1, j, i) - 1.5 * A(u, k, j, i) + A(u, k + 1, j, i)) * 0.5 * 0.5;
                A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (-qu);
                A(uo, k - 1, j, i) = A(uo, k - 1, j, i) + fkdtu * rddzk * (+qu);
                const double fvb = avz * (A(wt, k - 1, j, i) + A(wt, k - 1, j + 1, i)) * 0.5;
                const double qv = 0.5 * (fvb + std::fabs(fvb)) *
                                  (0.5 * A(v, k - 1, j, i) - 1.5 * A(v, k, j, i) + A(v, k + 1, j, i)) * 0.5 * 0.5;
                A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (-qv);
                A(vo, k - 1, j, i) = A(vo, k - 1, j, i) + fkdtv * rddzk * (+qv);
            }
        }
    }
    (void)fkdtu;
    // ---- momentum-conserving fluxes: BACK
    if (nbac == 8) {
        int i = ii - 2;
        // w cell: standard flux, then the flux of every coarse velocity
        for (int j = 3; j <= jj - 2; ++j) {
            ddyj = ddy[j];
            for (int k = 2; k <= kk - 2; ++k) {
                dzk = dz[k];
                awx = ddyj * dzk;
                const double fwe = awx * (A(ut, k, j, i) + A(ut, k + 1, j, i)) * 0.5;
                A(wcw, k, j, i + 1) = 0.5 * fwe * (A(w, k, j, i) + A(w, k, j, i + 1));
            }
        }
        for (int j = 3; j <= jj - 2; j += 2) {
            ddyj = ddy[j];
            int k = 2;
            dzk = dz[k];
            awx = ddyj * dzk;
            double fwe = awx * (2 * A(ut, k, j, i) + 2 * A(ut, k, j + 1, i) + A(ut, k + 1, j, i) +
                                A(ut, k + 1, j + 1, i) + A(ut, k + 2, j, i) + A(ut, k + 2, j + 1, i)) * 0.125;
            A(wcw, k, j, i) = 0.5 * fwe * (A(w, k, j, i) + A(w, k, j, i + 1));
            A(wcw, k, j + 1, i) = 0.5 * fwe * (A(w, k, j + 1, i) + A(w, k, j + 1, i + 1));
            for (k = 4; k <= kk - 4; k += 2) {
                dzk = dz[k];
                awx = ddyj * dzk;
                fwe = awx * (A(ut, k - 1, j, i) + A(ut, k - 1, j + 1, i) + A(ut, k, j, i) + A(ut, k, j + 1, i) +
                             A(ut, k + 1, j, i) + A(ut, k + 1, j + 1, i) + A(ut, k + 2, j, i) +
                             A(ut, k + 2, j + 1, i)) * 0.125;
                A(wcw, k, j, i) = 0.5 * fwe * (A(w, k, j, i) + A(w, k, j, i + 1));
                A(wcw, k, j + 1, i) = 0.5 * fwe * (A(w, k, j + 1, i) + A(w, k, j + 1, i + 1));
            }
            k = kk - 2;
            dzk = dz[k];
            awx = ddyj * dzk;
            fwe = awx * (A(ut, k - 1, j, i) + A(ut, k - 1, j + 1, i) + A(ut, k, j, i) + A(ut, k, j + 1, i) +
                         2 * A(ut, k + 1, j, i) + 2 * A(ut, k + 1, j + 1, i)) * 0.125;
            A(wcw, k, j, i) = 0.5 * fwe * (A(w, k, j, i) + A(w, k, j, i + 1));
            A(wcw, k, j + 1, i) = 0.5 * fwe * (A(w, k, j + 1, i) + A(w, k, j + 1, i + 1));
        }
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 2; k <= kk - 4; k += 2)
                A(wcw, k + 1, j, i) = 0.5 * (A(wcw, k, j, i) + A(wcw, k + 2, j, i));
        for (int j = 3; j <= jj - 2; ++j) {
            fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            for (int k = 2; k <= kk - 2; ++k) {
                rdzk = rdz[k];
                A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (-A(wcw, k, j, i + 1) + A(wcw, k, j, i));
            }
        }
        // v cell
        for (int j = 2; j <= jj - 2; ++j) {
            dyj = dy[j];
            for (int k = 3; k <= kk - 2; ++k) {
                ddzk = ddz[k];
                avx = ddzk * dyj;
                const double fve = avx * (A(ut, k, j, i) + A(ut, k, j + 1, i)) * 0.5;
                A(wcv, k, j, i + 1) = 0.5 * fve * (A(v, k, j, i) + A(v, k, j, i + 1));
            }
        }
        {
            int j = 2;
            dyj = dy[j];
            for (int k = 3; k <= kk - 2; k += 2) {
                ddzk = ddz[k];
                avx = ddzk * dyj;
                const double fve = avx * (2 * A(ut, k, j, i) + 2 * A(ut, k + 1, j, i) + A(ut, k, j + 1, i) +
                                          A(ut, k + 1, j + 1, i) + A(ut, k, j + 2, i) + A(ut, k + 1, j + 2, i)) * 0.125;
                A(wcv, k, j, i) = 0.5 * fve * (A(v, k, j, i) + A(v, k, j, i + 1));
                A(wcv, k + 1, j, i) = 0.5 * fve * (A(v, k + 1, j, i) + A(v, k + 1, j, i + 1));
            }
            for (j = 4; j <= jj - 4; j += 2) {
                dyj = dy[j];
                for (int k = 3; k <= kk - 2; k += 2) {
                    ddzk = ddz[k];
                    avx = ddzk * dyj;
                    const double fve = avx * (A(ut, k, j - 1, i) + A(ut, k + 1, j - 1, i) + A(ut, k, j, i) +
                                              A(ut, k + 1, j, i) + A(ut, k, j + 1, i) + A(ut, k + 1, j + 1, i) +
                                              A(ut, k, j + 2, i) + A(ut, k + 1, j + 2, i)) * 0.125;
                    A(wcv, k, j, i) = 0.5 * fve * (A(v, k, j, i) + A(v, k, j, i + 1));
                    A(wcv, k + 1, j, i) = 0.5 * fve * (A(v, k + 1, j, i) + A(v, k + 1, j, i + 1));
                }
            }
            j = jj - 2;
            dyj = dy[j];
            for (int k = 3; k <= kk - 2; k += 2) {
                ddzk = ddz[k];
                avx = ddzk * dyj;
                const double fve = avx * (A(ut, k, j - 1, i) + A(ut, k + 1, j - 1, i) + A(ut, k, j, i) +
                                          A(ut, k + 1, j, i) + 2 * A(ut, k, j + 1, i) + 2 * A(ut, k + 1, j + 1, i)) * 0.125;
                A(wcv, k, j, i) = 0.5 * fve * (A(v, k, j, i) + A(v, k, j, i + 1));
                A(wcv, k + 1, j, i) = 0.5 * fve * (A(v, k + 1, j, i) + A(v, k + 1, j, i + 1));
            }
        }
        for (int j = 2; j <= jj - 4; j += 2)
            for (int k = 3; k <= kk - 2; ++k)
                A(wcv, k, j + 1, i) = 0.5 * (A(wcv, k, j, i) + A(wcv, k, j + 2, i));
        for (int j = 2; j <= jj - 2; ++j) {
            fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            for (int k = 3; k <= kk - 2; ++k) {
                rddzk = rddz[k];
                A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (A(wcv, k, j, i) - A(wcv, k, j, i + 1));
            }
        }
    }
    // ---- FRONT
    if (nfro == 8) {
        int i = 3;
        for (int j = 3; j <= jj - 2; ++j) {
            ddyj = ddy[j];
            for (int k = 2; k <= kk - 2; ++k) {
                dzk = dz[k];
                awx = ddyj * dzk;
                const double fww = awx * (A(ut, k, j, i - 1) + A(ut, k + 1, j, i - 1)) * 0.5;
                A(wcw, k, j, i - 1) = 0.5 * fww * (A(w, k, j, i) + A(w, k, j, i - 1));
            }
        }
        for (int j = 3; j <= jj - 2; j += 2) {
            ddyj = ddy[j];
            int k = 2;
            dzk = dz[k];
            awx = ddyj * dzk;
            double fww = awx * (2 * A(ut, k, j, i - 1) + 2 * A(ut, k, j + 1, i - 1) + A(ut, k + 1, j, i - 1) +
                                A(ut, k + 1, j + 1, i - 1) + A(ut, k + 2, j, i - 1) + A(ut, k + 2, j + 1, i - 1)) * 0.125;
            A(wcw, k, j, i) = 0.5 * fww * (A(w, k, j, i) + A(w, k, j, i - 1));
            A(wcw, k, j + 1, i) = 0.5 * fww * (A(w, k, j + 1, i) + A(w, k, j + 1, i - 1));
            for (k = 4; k <= kk - 4; k += 2) {
                dzk = dz[k];
                awx = ddyj * dzk;
                fww = awx * (A(ut, k - 1, j, i - 1) + A(ut, k - 1, j + 1, i - 1) + A(ut, k, j, i - 1) +
                             A(ut, k, j + 1, i - 1) + A(ut, k + 1, j, i - 1) + A(ut, k + 1, j + 1, i - 1) +
                             A(ut, k + 2, j, i - 1) + A(ut, k + 2, j + 1, i - 1)) * 0.125;
                A(wcw, k, j, i) = 0.5 * fww * (A(w, k, j, i) + A(w, k, j, i - 1));
                A(wcw, k, j + 1, i) = 0.5 * fww * (A(w, k, j + 1, i) + A(w, k, j + 1, i - 1));
            }
            k = kk - 2;
            dzk = dz[k];
            awx = ddyj * dzk;
            fww = awx * (A(ut, k - 1, j, i - 1) + A(ut, k - 1, j + 1, i - 1) + A(ut, k, j, i - 1) +
                         A(ut, k, j + 1, i - 1) + 2 * A(ut, k + 1, j, i - 1) + 2 * A(ut, k + 1, j + 1, i - 1)) * 0.125;
            A(wcw, k, j, i) = 0.5 * fww * (A(w, k, j, i) + A(w, k, j, i - 1));
            A(wcw, k, j + 1, i) = 0.5 * fww * (A(w, k, j + 1, i) + A(w, k, j + 1, i - 1));
        }
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 2; k <= kk - 4; k += 2)
                A(wcw, k + 1, j, i) = 0.5 * (A(wcw, k, j, i) + A(wcw, k + 2, j, i));
        for (int j = 3; j <= jj - 2; ++j) {
            fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            for (int k = 2; k <= kk - 2; ++k) {
                rdzk = rdz[k];
                A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (A(wcw, k, j, i - 1) - A(wcw, k, j, i));
            }
        }
        for (int j = 2; j <= jj - 2; ++j) {
            dyj = dy[j];
            for (int k = 3; k <= kk - 2; ++k) {
                ddzk = ddz[k];
                avx = ddzk * dyj;
                const double fvw = avx * (A(ut, k, j, i - 1) + A(ut, k, j + 1, i - 1)) * 0.5;
                A(wcv, k, j, i - 1) = 0.5 * fvw * (A(v, k, j, i) + A(v, k, j, i - 1));
            }
        }
        {
            int j = 2;
            dyj = dy[j];
            for (int k = 3; k <= kk - 2; k += 2) {
                ddzk = ddz[k];
                avx = ddzk * dyj;
                const double fvw = avx * (2 * A(ut, k, j, i - 1) + 2 * A(ut, k + 1, j, i - 1) + A(ut, k, j + 1, i - 1) +
                                          A(ut, k + 1, j + 1, i - 1) + A(ut, k, j + 2, i - 1) + A(ut, k + 1, j + 2, i - 1)) * 0.125;
                A(wcv, k, j, i) = 0.5 * fvw * (A(v, k, j, i) + A(v, k, j, i - 1));
                A(wcv, k + 1, j, i) = 0.5 * fvw * (A(v, k + 1, j, i) + A(v, k + 1, j, i - 1));
            }
            for (j = 4; j <= jj - 4; j += 2) {
                dyj = dy[j];
                for (int k = 3; k <= kk - 2; k += 2) {
                    ddzk = ddz[k];
                    avx = ddzk * dyj;
                    const double fvw = avx * (A(ut, k, j - 1, i - 1) + A(ut, k + 1, j - 1, i - 1) + A(ut, k, j, i - 1) +
                                              A(ut, k + 1, j, i - 1) + A(ut, k, j + 1, i - 1) + A(ut, k + 1, j + 1, i - 1) +
                                              A(ut, k, j + 2, i - 1) + A(ut, k + 1, j + 2, i - 1)) * 0.125;
                    A(wcv, k, j, i) = 0.5 * fvw * (A(v, k, j, i) + A(v, k, j, i - 1));
                    A(wcv, k + 1, j, i) = 0.5 * fvw * (A(v, k + 1, j, i) + A(v, k + 1, j, i - 1));
                }
            }
            j = jj - 2;
            dyj = dy[j];
            for (int k = 3; k <= kk - 2; k += 2) {
                ddzk = ddz[k];
                avx = ddzk * dyj;
                const double fvw = avx * (A(ut, k, j - 1, i - 1) + A(ut, k + 1, j - 1, i - 1) + A(ut, k, j, i - 1) +
                                          A(ut, k + 1, j, i - 1) + 2 * A(ut, k, j + 1, i - 1) + 2 * A(ut, k + 1, j + 1, i - 1)) * 0.125;
                A(wcv, k, j, i) = 0.5 * fvw * (A(v, k, j, i) + A(v, k, j, i - 1));
                A(wcv, k + 1, j, i) = 0.5 * fvw * (A(v, k + 1, j, i) + A(v, k + 1, j, i - 1));
            }
        }
        for (int j = 2; j <= jj - 4; j += 2)
            for (int k = 3; k <= kk - 2; ++k)
                A(wcv, k, j + 1, i) = 0.5 * (A(wcv, k, j, i) + A(wcv, k, j + 2, i));
        for (int j = 2; j <= jj - 2; ++j) {
            fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
            for (int k = 3; k <= kk - 2; ++k) {
                rddzk = rddz[k];
                A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (-A(wcv, k, j, i) + A(wcv, k, j, i - 1));
            }
        }
    }
    // ---- TOP and BOTTOM: u cell (pairs in j, distribution in i), v cell
    // (pairs in i, distribution in j); kq the plane of the fine fluxes, kc
    // that of the standard flux, ks the transporting layer, sgn the order of
    // the two w-flux planes in the update
    for (int side = 0; side < 2; ++side) {
        const bool top = side == 0;
        if ((top ? ntop : nbot) != 8) continue;
        const int k = top ? kk - 2 : 3;
        const int kw = top ? k : k - 1;          // wt plane
        const int kn = top ? k + 1 : k - 1;      // the other u/v plane of the flux
        const int kc = top ? k + 1 : k - 1;      // standard-flux plane of wcu / wcv
        for (int i = 2; i <= ii - 2; ++i) {
            dxi = dx[i];
            for (int j = 3; j <= jj - 2; ++j) {
                ddyj = ddy[j];
                auz = dxi * ddyj;
                const double f = auz * (A(wt, kw, j, i) + A(wt, kw, j, i + 1)) * 0.5;
                A(wcu, kc, j, i) = 0.5 * f * (A(u, k, j, i) + A(u, kn, j, i));
            }
        }
        {
            int i = 2;
            dxi = dx[i];
            for (int j = 3; j <= jj - 2; j += 2) {
                ddyj = ddy[j];
                auz = dxi * ddyj;
                const double f = auz * (2 * A(wt, kw, j, i) + 2 * A(wt, kw, j + 1, i) + A(wt, kw, j, i + 1) +
                                        A(wt, kw, j + 1, i + 1) + A(wt, kw, j, i + 2) + A(wt, kw, j + 1, i + 2)) * 0.125;
                A(wcu, k, j, i) = 0.5 * f * (A(u, k, j, i) + A(u, kn, j, i));
                A(wcu, k, j + 1, i) = 0.5 * f * (A(u, k, j + 1, i) + A(u, kn, j + 1, i));
            }
            for (i = 4; i <= ii - 4; i += 2) {
                dxi = dx[i];
                for (int j = 3; j <= jj - 2; j += 2) {
                    ddyj = ddy[j];
                    auz = dxi * ddyj;
                    const double f = auz * (A(wt, kw, j, i - 1) + A(wt, kw, j + 1, i - 1) + A(wt, kw, j, i) +
                                            A(wt, kw, j + 1, i) + A(wt, kw, j, i + 1) + A(wt, kw, j + 1, i + 1) +
                                            A(wt, kw, j, i + 2) + A(wt, kw, j + 1, i + 2)) * 0.125;
                    A(wcu, k, j, i) = 0.5 * f * (A(u, k, j, i) + A(u, kn, j, i));
                    A(wcu, k, j + 1, i) = 0.5 * f * (A(u, k, j + 1, i) + A(u, kn, j + 1, i));
                }
            }
            i = ii - 2;
            dxi = dx[i];
            for (int j = 3; j <= jj - 2; j += 2) {
                ddyj = ddy[j];
                auz = dxi * ddyj;
                const double f = auz * (A(wt, kw, j, i - 1) + A(wt, kw, j + 1, i - 1) + A(wt, kw, j, i) +
                                        A(wt, kw, j + 1, i) + 2 * A(wt, kw, j, i + 1) + 2 * A(wt, kw, j + 1, i + 1)) * 0.125;
                A(wcu, k, j, i) = 0.5 * f * (A(u, k, j, i) + A(u, kn, j, i));
                A(wcu, k, j + 1, i) = 0.5 * f * (A(u, k, j + 1, i) + A(u, kn, j + 1, i));
            }
        }
        for (int i = 2; i <= ii - 4; i += 2)
            for (int j = 3; j <= jj - 2; ++j)
                A(wcu, k, j, i + 1) = 0.5 * (A(wcu, k, j, i) + A(wcu, k, j, i + 2));
        rddzk = rddz[k];
        for (int i = 2; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j) {
                fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
                if (top)
                    A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (A(wcu, k, j, i) - A(wcu, k + 1, j, i));
                else
                    A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (-A(wcu, k, j, i) + A(wcu, k - 1, j, i));
            }
        for (int i = 3; i <= ii - 2; ++i) {
            ddxi = ddx[i];
            for (int j = 2; j <= jj - 2; ++j) {
                dyj = dy[j];
                avz = ddxi * dyj;
                const double f = avz * (A(wt, kw, j, i) + A(wt, kw, j + 1, i)) * 0.5;
                A(wcv, kc, j, i) = 0.5 * f * (A(v, k, j, i) + A(v, kn, j, i));
            }
        }
        for (int i = 3; i <= ii - 2; i += 2) {
            ddxi = ddx[i];
            int j = 2;
            dyj = dy[j];
            avz = ddxi * dyj;
            double f = avz * (2 * A(wt, kw, j, i) + 2 * A(wt, kw, j, i + 1) + A(wt, kw, j + 1, i) +
                              A(wt, kw, j + 1, i + 1) + A(wt, kw, j + 2, i) + A(wt, kw, j + 2, i + 1)) * 0.125;
            A(wcv, k, j, i) = 0.5 * f * (A(v, k, j, i) + A(v, kn, j, i));
            A(wcv, k, j, i + 1) = 0.5 * f * (A(v, k, j, i + 1) + A(v, kn, j, i + 1));
            for (j = 4; j <= jj - 4; j += 2) {
                dyj = dy[j];
                avz = ddxi * dyj;
                f = avz * (A(wt, kw, j - 1, i) + A(wt, kw, j - 1, i + 1) + A(wt, kw, j, i) + A(wt, kw, j, i + 1) +
                           A(wt, kw, j + 1, i) + A(wt, kw, j + 1, i + 1) + A(wt, kw, j + 2, i) +
                           A(wt, kw, j + 2, i + 1)) * 0.125;
                A(wcv, k, j, i) = 0.5 * f * (A(v, k, j, i) + A(v, kn, j, i));
                A(wcv, k, j, i + 1) = 0.5 * f * (A(v, k, j, i + 1) + A(v, kn, j, i + 1));
            }
            j = jj - 2;
            dyj = dy[j];
            avz = ddxi * dyj;
            f = avz * (A(wt, kw, j - 1, i) + A(wt, kw, j - 1, i + 1) + A(wt, kw, j, i) + A(wt, kw, j, i + 1) +
                       2 * A(wt, kw, j + 1, i) + 2 * A(wt, kw, j + 1, i + 1)) * 0.125;
            A(wcv, k, j, i) = 0.5 * f * (A(v, k, j, i) + A(v, kn, j, i));
            A(wcv, k, j, i + 1) = 0.5 * f * (A(v, k, j, i + 1) + A(v, kn, j, i + 1));
        }
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 2; j <= jj - 4; j += 2)
                A(wcv, k, j + 1, i) = 0.5 * (A(wcv, k, j, i) + A(wcv, k, j + 2, i));
        rddzk = rddz[k];
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 2; j <= jj - 2; ++j) {
                fkdtv = -1.0 * rddx[i] * rdy[j] * wkon;
                if (top)
                    A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (A(wcv, k, j, i) - A(wcv, k + 1, j, i));
                else
                    A(vo, k, j, i) = A(vo, k, j, i) + fkdtv * rddzk * (-A(wcv, k, j, i) + A(wcv, k - 1, j, i));
            }
    }
    // ---- LEFT and RIGHT: u cell (pairs in k, distribution in i), w cell
    // (pairs in i, distribution in k)
    for (int side = 0; side < 2; ++side) {
        const bool left = side == 0;
        if ((left ? nlft : nrgt) != 8) continue;
        const int j = left ? jj - 2 : 3;
        const int jv = left ? j : j - 1;          // vt plane
        const int jn = left ? j + 1 : j - 1;      // the other u/w plane of the flux
        const int jc = left ? j + 1 : j - 1;      // standard-flux plane
        for (int i = 2; i <= ii - 2; ++i) {
            dxi = dx[i];
            for (int k = 3; k <= kk - 2; ++k) {
                ddzk = ddz[k];
                auy = dxi * ddzk;
                const double f = auy * (A(vt, k, jv, i) + A(vt, k, jv, i + 1)) * 0.5;
                A(wcu, k, jc, i) = 0.5 * f * (A(u, k, j, i) + A(u, k, jn, i));
            }
        }
        {
            int i = 2;
            dxi = dx[i];
            for (int k = 3; k <= kk - 2; k += 2) {
                ddzk = ddz[k];
                auy = dxi * ddzk;
                const double f = auy * (2 * A(vt, k, jv, i) + 2 * A(vt, k + 1, jv, i) + A(vt, k, jv, i + 1) +
                                        A(vt, k + 1, jv, i + 1) + A(vt, k, jv, i + 2) + A(vt, k + 1, jv, i + 2)) * 0.125;
                A(wcu, k, j, i) = 0.5 * f * (A(u, k, j, i) + A(u, k, jn, i));
                A(wcu, k + 1, j, i) = 0.5 * f * (A(u, k + 1, j, i) + A(u, k + 1, jn, i));
            }
            for (i = 4; i <= ii - 4; i += 2) {
                dxi = dx[i];
                for (int k = 3; k <= kk - 2; k += 2) {
                    ddzk = ddz[k];
                    auy = dxi * ddzk;
                    const double f = auy * (A(vt, k, jv, i - 1) + A(vt, k + 1, jv, i - 1) + A(vt, k, jv, i) +
                                            A(vt, k + 1, jv, i) + A(vt, k, jv, i + 1) + A(vt, k + 1, jv, i + 1) +
                                            A(vt, k, jv, i + 2) + A(vt, k + 1, jv, i + 2)) * 0.125;
                    A(wcu, k, j, i) = 0.5 * f * (A(u, k, j, i) + A(u, k, jn, i));
                    A(wcu, k + 1, j, i) = 0.5 * f * (A(u, k + 1, j, i) + A(u, k + 1, jn, i));
                }
            }
            i = ii - 2;
            dxi = dx[i];
            for (int k = 3; k <= kk - 2; k += 2) {
                ddzk = ddz[k];
                auy = dxi * ddzk;
                const double f = auy * (A(vt, k, jv, i - 1) + A(vt, k + 1, jv, i - 1) + A(vt, k, jv, i) +
                                        A(vt, k + 1, jv, i) + 2 * A(vt, k, jv, i + 1) + 2 * A(vt, k + 1, jv, i + 1)) * 0.125;
                A(wcu, k, j, i) = 0.5 * f * (A(u, k, j, i) + A(u, k, jn, i));
                A(wcu, k + 1, j, i) = 0.5 * f * (A(u, k + 1, j, i) + A(u, k + 1, jn, i));
            }
        }
        for (int i = 2; i <= ii - 4; i += 2)
            for (int k = 3; k <= kk - 2; ++k)
                A(wcu, k, j, i + 1) = 0.5 * (A(wcu, k, j, i) + A(wcu, k, j, i + 2));
        for (int i = 2; i <= ii - 2; ++i) {
            fkdtu = -1.0 * rddy[j] * rdx[i] * wkon;
            for (int k = 3; k <= kk - 2; ++k) {
                rddzk = rddz[k];
                if (left)
                    A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (A(wcu, k, j, i) - A(wcu, k, j + 1, i));
                else
                    A(uo, k, j, i) = A(uo, k, j, i) + fkdtu * rddzk * (-A(wcu, k, j, i) + A(wcu, k, j - 1, i));
            }
        }
        for (int i = 3; i <= ii - 2; ++i) {
            ddxi = ddx[i];
            for (int k = 2; k <= kk - 2; ++k) {
                dzk = dz[k];
                awy = ddxi * dzk;
                const double f = awy * (A(vt, k, jv, i) + A(vt, k + 1, jv, i)) * 0.5;
                A(wcw, k, jc, i) = 0.5 * f * (A(w, k, j, i) + A(w, k, jn, i));
            }
        }
        for (int i = 3; i <= ii - 2; i += 2) {
            ddxi = ddx[i];
            int k = 2;
            dzk = dz[k];
            awy = ddxi * dzk;
            double f = awy * (2 * A(vt, k, jv, i) + 2 * A(vt, k, jv, i + 1) + A(vt, k + 1, jv, i) +
                              A(vt, k + 1, jv, i + 1) + A(vt, k + 2, jv, i) + A(vt, k + 2, jv, i + 1)) * 0.125;
            A(wcw, k, j, i) = 0.5 * f * (A(w, k, j, i) + A(w, k, jn, i));
            A(wcw, k, j, i + 1) = 0.5 * f * (A(w, k, j, i + 1) + A(w, k, jn, i + 1));
            for (k = 4; k <= kk - 4; ++k) {   // every k, as the reference runs it
                dzk = dz[k];
                awy = ddxi * dzk;
                f = awy * (A(vt, k - 1, jv, i) + A(vt, k - 1, jv, i + 1) + A(vt, k, jv, i) + A(vt, k, jv, i + 1) +
                           A(vt, k + 1, jv, i) + A(vt, k + 1, jv, i + 1) + A(vt, k + 2, jv, i) +
                           A(vt, k + 2, jv, i + 1)) * 0.125;
                A(wcw, k, j, i) = 0.5 * f * (A(w, k, j, i) + A(w, k, jn, i));
                A(wcw, k, j, i + 1) = 0.5 * f * (A(w, k, j, i + 1) + A(w, k, jn, i + 1));
            }
            k = kk - 2;
            dzk = dz[k];
            awy = ddxi * dzk;
            f = awy * (A(vt, k - 1, jv, i) + A(vt, k - 1, jv, i + 1) + A(vt, k, jv, i) + A(vt, k, jv, i + 1) +
                       2 * A(vt, k + 1, jv, i) + 2 * A(vt, k + 1, jv, i + 1)) * 0.125;
            A(wcw, k, j, i) = 0.5 * f * (A(w, k, j, i) + A(w, k, jn, i));
            A(wcw, k, j, i + 1) = 0.5 * f * (A(w, k, j, i + 1) + A(w, k, jn, i + 1));
        }
        for (int i = 3; i <= ii - 2; ++i)
            for (int k = 2; k <= kk - 4; k += 2)
                A(wcw, k + 1, j, i) = 0.5 * (A(wcw, k, j, i) + A(wcw, k + 2, j, i));
        for (int i = 3; i <= ii - 2; ++i) {
            fkdtw = -1.0 * rddx[i] * rddy[j] * wkon;
            for (int k = 2; k <= kk - 2; ++k) {
                rdzk = rdz[k];
                if (left)
                    A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (-A(wcw, k, j + 1, i) + A(wcw, k, j, i));
                else
                    A(wo, k, j, i) = A(wo, k, j, i) + fkdtw * rdzk * (A(wcw, k, j - 1, i) - A(wcw, k, j, i));
            }
        }
    }
#undef A
}

// tstle4_mod.F90:139-265 tstle4_kon, :268-458 tstle4_diff, :461-529 tstle4_gradp,
// :532-1753 tstle4_par
// wernerwengle_mod.F90:64-87 tauwin and tstle4_mod.F90:1832-1844
// swcle3d_one: the wall shear over rho and the wall-normal width dds
double swcle3d_one(const WernerWengle& q, double dds, double u) {
    const double vz = std::copysign(1.0, u);
    const double uquern = std::fabs(u);
    double tauwin;
    if (uquern >= q.cpo6 / dds) {
        const double ddsb = std::pow(dds, -q.cwb);
        tauwin = vz * q.rho * std::pow(ddsb * (q.cpo4 * uquern + q.cpo5 / dds), q.cpo8);
    } else {
        tauwin = vz * 2.0 * q.gmol * uquern / dds;
    }
    return tauwin / q.rho / dds;
}

// tstle4_mod.F90:1756-1829 swcle3d: on NOS (code 5) faces the wall shear of
// the two tangential components is taken from uo, vo, wo in the layer next to
// the wall, over the whole face including its ghost rows (2..n-1)
void swcle3d(const WernerWengle& q, int kk, int jj, int ii, double* uo, double* vo, double* wo,
             const double* u, const double* v, const double* w, const double* ddx,
             const double* ddy, const double* ddz, int nfro, int nbac, int nrgt, int nlft, int nbot,
             int ntop) {
#define A(a, k, j, i) a[IX(k, j, i)]
    for (int side = 0; side < 2; ++side) {       // FRONT, BACK
        if ((side ? nbac : nfro) != 5) continue;
        const int i = side ? ii - 2 : 3;
        for (int j = 2; j <= jj - 1; ++j)
            for (int k = 2; k <= kk - 1; ++k) {
                A(vo, k, j, i) = A(vo, k, j, i) - swcle3d_one(q, ddx[i], A(v, k, j, i));
                A(wo, k, j, i) = A(wo, k, j, i) - swcle3d_one(q, ddx[i], A(w, k, j, i));
            }
    }
    for (int side = 0; side < 2; ++side) {       // RIGHT, LEFT
        if ((side ? nlft : nrgt) != 5) continue;
        const int j = side ? jj - 2 : 3;
        for (int i = 2; i <= ii - 1; ++i)
            for (int k = 2; k <= kk - 1; ++k) {
                A(uo, k, j, i) = A(uo, k, j, i) - swcle3d_one(q, ddy[j], A(u, k, j, i));
                A(wo, k, j, i) = A(wo, k, j, i) - swcle3d_one(q, ddy[j], A(w, k, j, i));
            }
    }
    for (int side = 0; side < 2; ++side) {       // BOTTOM, TOP
        if ((side ? ntop : nbot) != 5) continue;
        const int k = side ? kk - 2 : 3;
        for (int i = 2; i <= ii - 1; ++i)
            for (int j = 2; j <= jj - 1; ++j) {
                A(uo, k, j, i) = A(uo, k, j, i) - swcle3d_one(q, ddz[k], A(u, k, j, i));
                A(vo, k, j, i) = A(vo, k, j, i) - swcle3d_one(q, ddz[k], A(v, k, j, i));
            }
    }
#undef A
}

void tstle4_grid(Ctx& c, int g) {
    const Grid& G = c.g[g];
    const int kk = G.kk, jj = G.jj, ii = G.ii;
    const int64_t o = G.ip3;
    double* uo = c.F("UO") + o; double* vo = c.F("VO") + o; double* wo = c.F("WO") + o;
    // tstle4(uo, vo, wo, pwu, pwv, pww, u, v, w, p, g) (timeintegration_mod.F90:101):
    // the transported velocities are the point values PWU.. for the
    // ghost-cell IB and U.. otherwise; the transporting ones are always U..
    const bool gc = c.ibtype == 1;
    const double* u = c.F(gc ? "PWU" : "U") + o;
    const double* v = c.F(gc ? "PWV" : "V") + o;
    const double* w = c.F(gc ? "PWW" : "W") + o;
    const double* ut = c.F("U") + o; const double* vt = c.F("V") + o; const double* wt = c.F("W") + o;
    const double* p = c.F("P") + o; const double* gg = c.F("G") + o;
    const double* dx = c.L("DX") + G.ipx - 1; const double* dy = c.L("DY") + G.ipy - 1;
    const double* dz = c.L("DZ") + G.ipz - 1;
    const double* ddx = c.L("DDX") + G.ipx - 1; const double* ddy = c.L("DDY") + G.ipy - 1;
    const double* ddz = c.L("DDZ") + G.ipz - 1;
    const double* rdx = c.L("RDX") + G.ipx - 1; const double* rdy = c.L("RDY") + G.ipy - 1;
    const double* rdz = c.L("RDZ") + G.ipz - 1;
    const double* rddx = c.L("RDDX") + G.ipx - 1; const double* rddy = c.L("RDDY") + G.ipy - 1;
    const double* rddz = c.L("RDDZ") + G.ipz - 1;
    const int nfro = G.bc[1], nbac = G.bc[2], nrgt = G.bc[3], nlft = G.bc[4], nbot = G.bc[5],
              ntop = G.bc[6];
    int nfu = 0, nbu = 0, nrv = 0, nlv = 0, nbw = 0, ntw = 0;
    if (nbac == 7) nbu = 1;
    if (nlft == 7) nlv = 1;
    if (ntop == 7) ntw = 1;
    if (nfro == 3) nfu = 1;
    if (nbac == 3) nbu = 1;
    if (nrgt == 3) nrv = 1;
    if (nlft == 3) nlv = 1;
    if (nbot == 3) nbw = 1;
    if (ntop == 3) ntw = 1;
    const double gmol = c.prm.gmol, rho = c.prm.rho;
    const double iles = c.ilesmodel == 0 ? 0.0 : 1.0;
#define A(a, k, j, i) a[IX(k, j, i)]
    // ---- kon
    for (int i = 3 - nfu; i <= ii - 3 + nbu; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                double ax = ddy[j] * ddz[k], ay = dx[i] * ddz[k], az = dx[i] * ddy[j];
                double fe = ax * (A(ut, k, j, i) + (A(ut, k, j, i + 1) - A(ut, k, j, i)) * 0.5 * dx[i] / ddx[i + 1]);
                double fw = ax * (A(ut, k, j, i - 1) + (A(ut, k, j, i) - A(ut, k, j, i - 1)) * 0.5 * dx[i - 1] / ddx[i]);
                double fn = ay * (A(vt, k, j, i) + A(vt, k, j, i + 1)) * 0.5;
                double fs = ay * (A(vt, k, j - 1, i) + A(vt, k, j - 1, i + 1)) * 0.5;
                double ft = az * (A(wt, k, j, i) + A(wt, k, j, i + 1)) * 0.5;
                double fb = az * (A(wt, k - 1, j, i) + A(wt, k - 1, j, i + 1)) * 0.5;
                double qe = 0.5 * fe * (A(u, k, j, i) + A(u, k, j, i + 1));
                double qw = 0.5 * fw * (A(u, k, j, i - 1) + A(u, k, j, i));
                double qn = 0.5 * fn * (A(u, k, j, i) + A(u, k, j + 1, i));
                double qs = 0.5 * fs * (A(u, k, j - 1, i) + A(u, k, j, i));
                double qt = 0.5 * ft * (A(u, k, j, i) + A(u, k + 1, j, i));
                double qb = 0.5 * fb * (A(u, k - 1, j, i) + A(u, k, j, i));
                A(uo, k, j, i) = -(qe - qw + qn - qs + qt - qb) * rdx[i] * rddy[j] * rddz[k];
            }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3 - nrv; j <= jj - 3 + nlv; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                double ax = dy[j] * ddz[k], ay = ddx[i] * ddz[k], az = ddx[i] * dy[j];
                double fe = ax * (A(ut, k, j, i) + A(ut, k, j + 1, i)) * 0.5;
                double fw = ax * (A(ut, k, j, i - 1) + A(ut, k, j + 1, i - 1)) * 0.5;
                double fn = ay * (A(vt, k, j, i) + (A(vt, k, j + 1, i) - A(vt, k, j, i)) * 0.5 * dy[j] / ddy[j + 1]);
                double fs = ay * (A(vt, k, j - 1, i) + (A(vt, k, j, i) - A(vt, k, j - 1, i)) * 0.5 * dy[j - 1] / ddy[j]);
                double ft = az * (A(wt, k, j, i) + A(wt, k, j + 1, i)) * 0.5;
                double fb = az * (A(wt, k - 1, j, i) + A(wt, k - 1, j + 1, i)) * 0.5;
                double qe = 0.5 * fe * (A(v, k, j, i) + A(v, k, j, i + 1));
                double qw = 0.5 * fw * (A(v, k, j, i - 1) + A(v, k, j, i));
                double qn = 0.5 * fn * (A(v, k, j, i) + A(v, k, j + 1, i));
                double qs = 0.5 * fs * (A(v, k, j - 1, i) + A(v, k, j, i));
                double qt = 0.5 * ft * (A(v, k, j, i) + A(v, k + 1, j, i));
                double qb = 0.5 * fb * (A(v, k - 1, j, i) + A(v, k, j, i));
                A(vo, k, j, i) = -(qe - qw + qn - qs + qt - qb) * rddx[i] * rdy[j] * rddz[k];
            }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3 - nbw; k <= kk - 3 + ntw; ++k) {
                double ax = ddy[j] * dz[k], ay = ddx[i] * dz[k], az = ddx[i] * ddy[j];
                double fe = ax * (A(ut, k, j, i) + A(ut, k + 1, j, i)) * 0.5;
                double fw = ax * (A(ut, k, j, i - 1) + A(ut, k + 1, j, i - 1)) * 0.5;
                double fn = ay * (A(vt, k, j, i) + A(vt, k + 1, j, i)) * 0.5;
                double fs = ay * (A(vt, k, j - 1, i) + A(vt, k + 1, j - 1, i)) * 0.5;
                double ft = az * (A(wt, k, j, i) + (A(wt, k + 1, j, i) - A(wt, k, j, i)) * 0.5 * dz[k] / ddz[k + 1]);
                double fb = az * (A(wt, k - 1, j, i) + (A(wt, k, j, i) - A(wt, k - 1, j, i)) * 0.5 * dz[k - 1] / ddz[k]);
                double qe = 0.5 * fe * (A(w, k, j, i) + A(w, k, j, i + 1));
                double qw = 0.5 * fw * (A(w, k, j, i - 1) + A(w, k, j, i));
                double qn = 0.5 * fn * (A(w, k, j, i) + A(w, k, j + 1, i));
                double qs = 0.5 * fs * (A(w, k, j - 1, i) + A(w, k, j, i));
                double qt = 0.5 * ft * (A(w, k, j, i) + A(w, k + 1, j, i));
                double qb = 0.5 * fb * (A(w, k - 1, j, i) + A(w, k, j, i));
                A(wo, k, j, i) = -(qe - qw + qn - qs + qt - qb) * rddx[i] * rddy[j] * rdz[k];
            }
    // ---- diff: swcle3d (tstle4_mod.F90:315-316), then the viscous fluxes
    swcle3d(werner_wengle(gmol, rho), kk, jj, ii, uo, vo, wo, u, v, w, ddx, ddy, ddz, nfro, nbac,
            nrgt, nlft, nbot, ntop);
    auto hm = [&](double a, double b) { return a * b / std::max(a + b, gmol); };
    for (int i = 3 - nfu; i <= ii - 3 + nbu; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                double ax = ddy[j] * ddz[k], ay = dx[i] * ddz[k], az = dx[i] * ddy[j];
                double ge = A(gg, k, j, i + 1);
                double gw = A(gg, k, j, i);
                double gn = hm(A(gg, k, j, i), A(gg, k, j + 1, i)) + hm(A(gg, k, j, i + 1), A(gg, k, j + 1, i + 1));
                double gs = hm(A(gg, k, j - 1, i), A(gg, k, j, i)) + hm(A(gg, k, j - 1, i + 1), A(gg, k, j, i + 1));
                double gt = hm(A(gg, k, j, i), A(gg, k + 1, j, i)) + hm(A(gg, k, j, i + 1), A(gg, k + 1, j, i + 1));
                double gb = hm(A(gg, k - 1, j, i), A(gg, k, j, i)) + hm(A(gg, k - 1, j, i + 1), A(gg, k, j, i + 1));
                double qe = -ge * ax * rddx[i + 1] * (A(u, k, j, i + 1) - A(u, k, j, i));
                double qw = -gw * ax * rddx[i] * (A(u, k, j, i) - A(u, k, j, i - 1));
                double qn = -gn * ay * rdy[j] * (A(u, k, j + 1, i) - A(u, k, j, i));
                double qs = -gs * ay * rdy[j - 1] * (A(u, k, j, i) - A(u, k, j - 1, i));
                double qt = -gt * az * rdz[k] * (A(u, k + 1, j, i) - A(u, k, j, i));
                double qb = -gb * az * rdz[k - 1] * (A(u, k, j, i) - A(u, k - 1, j, i));
                double st = ((ge * (A(u, k, j, i + 1) - A(u, k, j, i)) * rddx[i + 1]) -
                             (gw * (A(u, k, j, i) - A(u, k, j, i - 1)) * rddx[i])) * ax +
                            ((gn * (A(v, k, j, i + 1) - A(v, k, j, i))) -
                             (gs * (A(v, k, j - 1, i + 1) - A(v, k, j - 1, i)))) * ddz[k] +
                            ((gt * (A(w, k, j, i + 1) - A(w, k, j, i))) -
                             (gb * (A(w, k - 1, j, i + 1) - A(w, k - 1, j, i)))) * ddy[j];
                double qc = st * iles;
                double fak = 1.0 / rho * rddy[j] * rdx[i] * rddz[k];
                A(uo, k, j, i) = A(uo, k, j, i) - fak * (qe - qw + qn - qs + qt - qb - qc);
            }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3 - nrv; j <= jj - 3 + nlv; ++j)
            for (int k = 3; k <= kk - 2; ++k) {
                double ax = dy[j] * ddz[k], ay = ddx[i] * ddz[k], az = ddx[i] * dy[j];
                double ge = hm(A(gg, k, j, i), A(gg, k, j, i + 1)) + hm(A(gg, k, j + 1, i), A(gg, k, j + 1, i + 1));
                double gw = hm(A(gg, k, j, i - 1), A(gg, k, j, i)) + hm(A(gg, k, j + 1, i - 1), A(gg, k, j + 1, i));
                double gn = A(gg, k, j + 1, i);
                double gs = A(gg, k, j, i);
                double gt = hm(A(gg, k, j, i), A(gg, k + 1, j, i)) + hm(A(gg, k, j + 1, i), A(gg, k + 1, j + 1, i));
                double gb = hm(A(gg, k - 1, j, i), A(gg, k, j, i)) + hm(A(gg, k - 1, j + 1, i), A(gg, k, j + 1, i));
                double qe = -ge * ax * rdx[i] * (A(v, k, j, i + 1) - A(v, k, j, i));
                double qw = -gw * ax * rdx[i - 1] * (A(v, k, j, i) - A(v, k, j, i - 1));
                double qn = -gn * ay * rddy[j + 1] * (A(v, k, j + 1, i) - A(v, k, j, i));
                double qs = -gs * ay * rddy[j] * (A(v, k, j, i) - A(v, k, j - 1, i));
                double qt = -gt * az * rdz[k] * (A(v, k + 1, j, i) - A(v, k, j, i));
                double qb = -gb * az * rdz[k - 1] * (A(v, k, j, i) - A(v, k - 1, j, i));
                double st = ((ge * (A(u, k, j + 1, i) - A(u, k, j, i))) -
                             (gw * (A(u, k, j + 1, i - 1) - A(u, k, j, i - 1)))) * ddz[k] +
                            ((gn * (A(v, k, j + 1, i) - A(v, k, j, i)) * rddy[j + 1]) -
                             (gs * (A(v, k, j, i) - A(v, k, j - 1, i)) * rddy[j])) * ay +
                            ((gt * (A(w, k, j + 1, i) - A(w, k, j, i))) -
                             (gb * (A(w, k - 1, j + 1, i) - A(w, k - 1, j, i)))) * ddx[i];
                double qc = st * iles;
                double fak = 1.0 / rho * rddx[i] * rdy[j] * rddz[k];
                A(vo, k, j, i) = A(vo, k, j, i) - fak * (qe - qw + qn - qs + qt - qb - qc);
            }
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3 - nbw; k <= kk - 3 + ntw; ++k) {
                double ax = ddy[j] * dz[k], ay = ddx[i] * dz[k], az = ddx[i] * ddy[j];
                double ge = hm(A(gg, k, j, i), A(gg, k, j, i + 1)) + hm(A(gg, k + 1, j, i), A(gg, k + 1, j, i + 1));
                double gw = hm(A(gg, k, j, i - 1), A(gg, k, j, i)) + hm(A(gg, k + 1, j, i - 1), A(gg, k + 1, j, i));
                double gn = hm(A(gg, k, j, i), A(gg, k, j + 1, i)) + hm(A(gg, k + 1, j, i), A(gg, k + 1, j + 1, i));
                double gs = hm(A(gg, k, j - 1, i), A(gg, k, j, i)) + hm(A(gg, k + 1, j - 1, i), A(gg, k + 1, j, i));
                double gt = A(gg, k + 1, j, i);
                double gb = A(gg, k, j, i);
                double qe = -ge * ax * rdx[i] * (A(w, k, j, i + 1) - A(w, k, j, i));
                double qw = -gw * ax * rdx[i - 1] * (A(w, k, j, i) - A(w, k, j, i - 1));
                double qn = -gn * ay * rdy[j] * (A(w, k, j + 1, i) - A(w, k, j, i));
                double qs = -gs * ay * rdy[j - 1] * (A(w, k, j, i) - A(w, k, j - 1, i));
                double qt = -gt * az * rddz[k + 1] * (A(w, k + 1, j, i) - A(w, k, j, i));
                double qb = -gb * az * rddz[k] * (A(w, k, j, i) - A(w, k - 1, j, i));
                double st = ((ge * (A(u, k + 1, j, i) - A(u, k, j, i))) -
                             (gw * (A(u, k + 1, j, i - 1) - A(u, k, j, i - 1)))) * ddy[j] +
                            ((gn * (A(v, k + 1, j, i) - A(v, k, j, i))) -
                             (gs * (A(v, k + 1, j - 1, i) - A(v, k, j - 1, i)))) * ddx[i] +
                            ((gt * (A(w, k + 1, j, i) - A(w, k, j, i)) * rddz[k + 1]) -
                             (gb * (A(w, k, j, i) - A(w, k - 1, j, i)) * rddz[k])) * az;
                double qc = st * iles;
                double fak = 1.0 / rho * rddx[i] * rddy[j] * rdz[k];
                A(wo, k, j, i) = A(wo, k, j, i) - fak * (qe - qw + qn - qs + qt - qb - qc);
            }
    // ---- gradp
    const double gpx = c.prm.gradp[0] * G.gradpflag, gpy = c.prm.gradp[1] * G.gradpflag,
                 gpz = c.prm.gradp[2] * G.gradpflag;
    for (int i = 3 - nfu; i <= ii - 3 + nbu; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3; k <= kk - 2; ++k)
                A(uo, k, j, i) = A(uo, k, j, i) - 1.0 / (rho * dx[i]) * (A(p, k, j, i + 1) - A(p, k, j, i) + gpx * dx[i]);
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3 - nrv; j <= jj - 3 + nlv; ++j)
            for (int k = 3; k <= kk - 2; ++k)
                A(vo, k, j, i) = A(vo, k, j, i) - 1.0 / (rho * dy[j]) * (A(p, k, j + 1, i) - A(p, k, j, i) + gpy * dy[j]);
    for (int i = 3; i <= ii - 2; ++i)
        for (int j = 3; j <= jj - 2; ++j)
            for (int k = 3 - nbw; k <= kk - 3 + ntw; ++k)
                A(wo, k, j, i) = A(wo, k, j, i) - 1.0 / (rho * dz[k]) * (A(p, k + 1, j, i) - A(p, k, j, i) + gpz * dz[k]);
    // the steady body force (a source term the reference does not have):
    // added after gradp over the same ranges
    if (c.bodyforce) {
        const double* fx = c.F("FBX") + o; const double* fy = c.F("FBY") + o; const double* fz = c.F("FBZ") + o;
        for (int i = 3 - nfu; i <= ii - 3 + nbu; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k) A(uo, k, j, i) = A(uo, k, j, i) + A(fx, k, j, i);
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3 - nrv; j <= jj - 3 + nlv; ++j)
                for (int k = 3; k <= kk - 2; ++k) A(vo, k, j, i) = A(vo, k, j, i) + A(fy, k, j, i);
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3 - nbw; k <= kk - 3 + ntw; ++k) A(wo, k, j, i) = A(wo, k, j, i) + A(fz, k, j, i);
    }
#undef A
    tstle4_par(kk, jj, ii, uo, vo, wo, u, v, w, ut, vt, wt, dx, dy, dz, ddx, ddy, ddz, rdx, rdy, rdz,
               rddx, rddy, rddz, nfro, nbac, nrgt, nlft, nbot, ntop);
}

void tstle4(Ctx& c) {
    for (const char* n : {"UO", "VO", "WO"}) c.f3[n].assign(c.idim3d, 0.0);
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g) tstle4_grid(c, g);
}

// rungekutta_mod.F90:315-333 rkstep
void rkstep(double* p, double* dp, const double* rhsp, int64_t n, double frhs, double dtfu) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        dp[i] = frhs * dp[i] + rhsp[i];
        p[i] = p[i] + dtfu * dp[i];
    }
}

// rungekutta_mod.F90:70-95,98-237 (init_*), :288-309 comp_c
int rk_init(const char* name, mglet_rk_scheme* rk) {
    std::memset(rk, 0, sizeof(*rk));
    std::string n(name ? name : "");
    for (auto& ch : n) ch = (char)std::tolower((unsigned char)ch);
    auto comp_c = [&]() {
        for (int q = 0; q < 6; ++q) rk->c[q] = 0.0;
        for (int i = 1; i <= rk->nrk; ++i)
            for (int j = 1; j <= i - 1; ++j) {
                double fak = 1.0;
                for (int k = 2; k <= j; ++k) fak = rk->a[k - 1] * fak + 1.0;
                rk->c[i - 1] = rk->c[i - 1] + rk->b[j - 1] * fak;
            }
    };
    if (n == "williamson") {
        rk->nrk = 3;
        rk->cflmax = (1.0 - 2.220446049250313e-16) * std::sqrt(3.0);
        double c[3] = {0.0, 1.0 / 3.0, 3.0 / 4.0}, a[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0},
               b[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
        for (int q = 0; q < 3; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; rk->c[q] = c[q]; }
    } else if (n == "berland") {
        rk->nrk = 6;
        rk->cflmax = (double)(3.80f - 0.01f);
        double a[6] = {0.0, -0.737101392796, -1.634740794341, -0.744739003780, -1.469897351522, -2.813971388035};
        double b[6] = {0.032918605146, 0.823256998200, 0.381530948900, 0.200092213184, 1.718581042715, 0.27};
        for (int q = 0; q < 6; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; }
        comp_c();
    } else if (n == "carpenter") {
        rk->nrk = 5;
        rk->cflmax = (double)(3.34f - 0.01f);
        double a[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                       -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
        double b[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                       1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                       2277821191437.0 / 14882151754819.0};
        for (int q = 0; q < 5; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; }
        comp_c();
    } else if (n == "bernardini") {
        rk->nrk = 5;
        rk->cflmax = (double)(3.47f - 0.01f);
        const double eps = -3.88856487394645e-7;
        double a[5] = {0.0, -1.0, -1.55798 + eps, -1.0, -0.45031 + eps};
        double b[5] = {0.2, 0.83204 + eps, 0.6, 0.35394 + eps, 0.2};
        for (int q = 0; q < 5; ++q) { rk->a[q] = a[q]; rk->b[q] = b[q]; }
        comp_c();
    } else {
        return fail(MGLET_ERR_ARG, "rk_init: invalid scheme " + n);
    }
    return 0;
}

// timeintegration_mod.F90:306-452 compcflmax, compdivmax, enerfg
void itinfo(Ctx& c, double dt, mglet_itinfo* out) {
    std::vector<double> cfl(c.ngrid + 1), dmx(c.ngrid + 1), es(c.ngrid + 1), vs(c.ngrid + 1);
#pragma omp parallel for schedule(dynamic)
    for (int g = 1; g <= c.ngrid; ++g) {
        const Grid& G = c.g[g];
        const int kk = G.kk, jj = G.jj, ii = G.ii;
        const double* u = c.F("U") + G.ip3; const double* v = c.F("V") + G.ip3;
        const double* w = c.F("W") + G.ip3; const double* bp = c.F("BP") + G.ip3;
        const double* sdiv = c.F("SDIV") + G.ip3;
        const double* dx = c.L("DX") + G.ipx - 1; const double* dy = c.L("DY") + G.ipy - 1;
        const double* dz = c.L("DZ") + G.ipz - 1;
        const double* ddx = c.L("DDX") + G.ipx - 1; const double* ddy = c.L("DDY") + G.ipy - 1;
        const double* ddz = c.L("DDZ") + G.ipz - 1;
        const double* rddx = c.L("RDDX") + G.ipx - 1; const double* rddy = c.L("RDDY") + G.ipy - 1;
        const double* rddz = c.L("RDDZ") + G.ipz - 1;
#define A(a, k, j, i) a[IX(k, j, i)]
        double cmax = 0.0;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k) {
                    double cflu = std::fabs(2.0 * A(u, k, j, i - 1) + (A(u, k, j, i) - A(u, k, j, i - 1)) * dx[i - 1] / ddx[i]) / ddx[i] +
                                  std::fabs(2.0 * A(u, k, j, i) + (A(u, k, j, i + 1) - A(u, k, j, i)) * dx[i] / ddx[i + 1]) / ddx[i] +
                                  std::fabs(A(v, k, j, i) + A(v, k, j, i + 1)) / ddy[j] +
                                  std::fabs(A(v, k, j - 1, i) + A(v, k, j - 1, i + 1)) / ddy[j] +
                                  std::fabs(A(w, k, j, i) + A(w, k, j, i + 1)) / ddz[k] +
                                  std::fabs(A(w, k - 1, j, i) + A(w, k - 1, j, i + 1)) / ddz[k];
                    cflu = cflu * A(bp, k, j, i) * A(bp, k, j, i + 1);
                    double cflv = std::fabs(A(u, k, j, i) + A(u, k, j + 1, i)) / ddx[i] +
                                  std::fabs(A(u, k, j, i - 1) + A(u, k, j + 1, i - 1)) / ddx[i] +
                                  std::fabs(2.0 * A(v, k, j - 1, i) + (A(v, k, j, i) - A(v, k, j - 1, i)) * dy[j - 1] / ddy[j]) / ddy[j] +
                                  std::fabs(2.0 * A(v, k, j, i) + (A(v, k, j + 1, i) - A(v, k, j, i)) * dy[j] / ddy[j + 1]) / ddy[j] +
                                  std::fabs(A(w, k, j, i) + A(w, k, j + 1, i)) / ddz[k] +
                                  std::fabs(A(w, k - 1, j, i) + A(w, k - 1, j + 1, i)) / ddz[k];
                    cflv = cflv * A(bp, k, j, i) * A(bp, k, j + 1, i);
                    double cflw = std::fabs(A(u, k, j, i) + A(u, k + 1, j, i)) / ddx[i] +
                                  std::fabs(A(u, k, j, i - 1) + A(u, k + 1, j, i - 1)) / ddx[i] +
                                  std::fabs(A(v, k, j, i) + A(v, k + 1, j, i)) / ddy[j] +
                                  std::fabs(A(v, k, j - 1, i) + A(v, k + 1, j - 1, i)) / ddy[j] +
                                  std::fabs(2.0 * A(w, k - 1, j, i) + (A(w, k, j, i) - A(w, k - 1, j, i)) * dz[k - 1] / ddz[k]) / ddz[k] +
                                  std::fabs(2.0 * A(w, k, j, i) + (A(w, k + 1, j, i) - A(w, k, j, i)) * dz[k] / ddz[k + 1]) / ddz[k];
                    cflw = cflw * A(bp, k, j, i) * A(bp, k + 1, j, i);
                    double m = std::max(cflu, std::max(cflv, cflw));
                    if (m > cmax) cmax = m;
                }
        cfl[g] = cmax * 0.25 * dt;
        double dm = 0.0;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k) {
                    double div = A(sdiv, k, j, i) + (A(u, k, j, i) - A(u, k, j, i - 1)) * rddx[i] +
                                 (A(v, k, j, i) - A(v, k, j - 1, i)) * rddy[j] +
                                 (A(w, k, j, i) - A(w, k - 1, j, i)) * rddz[k];
                    div = A(bp, k, j, i) * div;
                    if (std::fabs(div) > dm) dm = std::fabs(div);
                }
        dmx[g] = dm;
        double esum = 0.0, vsum = 0.0;
        for (int i = 3; i <= ii - 2; ++i)
            for (int j = 3; j <= jj - 2; ++j)
                for (int k = 3; k <= kk - 2; ++k) {
                    double up = A(u, k, j, i - 1) + (A(u, k, j, i) - A(u, k, j, i - 1)) * 0.5 * dx[i - 1] / ddx[i];
                    double vp = A(v, k, j - 1, i) + (A(v, k, j, i) - A(v, k, j - 1, i)) * 0.5 * dy[j - 1] / ddy[j];
                    double wp = A(w, k - 1, j, i) + (A(w, k, j, i) - A(w, k - 1, j, i)) * 0.5 * dz[k - 1] / ddz[k];
                    double vol = ddx[i] * ddy[j] * ddz[k];
                    esum = esum + vol * 0.5 * (up * up + vp * vp + wp * wp);
                    vsum = vsum + vol;
                }
        es[g] = esum / vsum;
        vs[g] = vsum;
#undef A
    }
    // itinfo_mod.F90:204-226: maxima over grids; energy as the running
    // volume-weighted mean of the per-grid means, in grid order.
    double cm = 0.0, dm = 0.0, esum = 0.0, vol = 0.0;
    bool nan = false;
    for (int g = 1; g <= c.ngrid; ++g) {
        if (c.g[g].halo) continue;   // another rank's grid
        cm = std::max(cm, cfl[g]);
        dm = std::max(dm, dmx[g]);
        if (vol + vs[g] > 0.0) esum = (esum * vol + es[g] * vs[g]) / (vol + vs[g]);
        else esum = 0.0;
        vol = vol + vs[g];
        if (!std::isfinite(cfl[g]) || !std::isfinite(dmx[g]) || !std::isfinite(es[g])) nan = true;
    }
    if (c.xfn) {
        double mx[3] = {cm, dm, nan ? 1.0 : 0.0}, sm[2] = {esum * vol, vol};
        if (part_allreduce(c, mx, 3, 1) || part_allreduce(c, sm, 2, 2)) nan = true;
        cm = mx[0];
        dm = mx[1];
        nan = nan || mx[2] != 0.0;
        esum = sm[1] > 0.0 ? sm[0] / sm[1] : 0.0;
    }
    out->cflmax = cm;
    out->divmax = dm;
    out->energy = esum;
    out->exploded = nan ? 1 : 0;
}

bool check_supported(const Ctx& c) {
    for (int g = 1; g <= c.ngrid; ++g)
        for (int f = 1; f <= 6; ++f) {
            const int t = c.g[g].bc[f];
            if (!(is_con(t) || t == MGLET_BC_FIX || t == MGLET_BC_OP1 || t == MGLET_BC_NOS ||
                  t == MGLET_BC_SLI || t == MGLET_BC_PAR))
                return false;
        }
    return true;
}

}  // namespace

// ===========================================================================
// C ABI (mirrors include/mglet_gpu.h with an oracle_ prefix)
struct oracle_ctx : Ctx {};

namespace {
// the pressure solve runs on hierarchies once their parents are known; the
// ghost-cell restriction (gc_restrict_mod.F90) is not restated
int hierarchy_ready(const Ctx& c) {
    for (int g = 1; g <= c.ngrid; ++g) {
        if (c.g[g].level == c.minlevel) continue;
        if (!c.iparent[g]) return fail(MGLET_ERR_ARG, "oracle: a fine grid without parent (set_hierarchy)");
    }
    return 0;
}

}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_rk_init(const char* name, mglet_rk_scheme* out) { return rk_init(name, out); }

int oracle_rk_get_coeffs(const mglet_rk_scheme* rk, int irk, double* frhs, double* fu,
                         double* dtrk, double* dtrki) {
    if (irk > rk->nrk || irk < 0) return fail(MGLET_ERR_ARG, "get_coeffs: irk out of range");
    *frhs = rk->a[irk - 1];
    *fu = rk->b[irk - 1];
    *dtrk = irk < rk->nrk ? rk->c[irk] : 1.0;
    *dtrki = *dtrk - rk->c[irk - 1];
    return 0;
}

int oracle_create(const mglet_grid_desc* d, const mglet_flow_params* prm, oracle_ctx** out) {
    if (!d || !prm || !out || d->ngrid <= 0) return fail(MGLET_ERR_ARG, "create: bad arguments");
    oracle_ctx* c = new oracle_ctx();
    c->ngrid = d->ngrid;
    c->prm = *prm;
    c->g.resize(d->ngrid + 1);
    int64_t o3 = 0, ox = 0, oy = 0, oz = 0;   // ipx/ipy/ipz 0-based
    c->minlevel = 1 << 30;
    c->maxlevel = -1;
    for (int g = 1; g <= d->ngrid; ++g) {
        Grid& G = c->g[g];
        G.kk = d->mgdims[3 * (g - 1) + 0];
        G.jj = d->mgdims[3 * (g - 1) + 1];
        G.ii = d->mgdims[3 * (g - 1) + 2];
        G.level = d->level[g - 1];
        for (int f = 1; f <= 6; ++f) G.bc[f] = d->bctype[6 * (g - 1) + f - 1];
        for (int f = 1; f <= 26; ++f) G.nbr[f] = d->nbrgrid[26 * (g - 1) + f - 1];
        G.gradpflag = d->gradpflag ? d->gradpflag[g - 1] : 1;
        G.ip3 = o3; G.ipx = ox; G.ipy = oy; G.ipz = oz;
        o3 += (int64_t)G.kk * G.jj * G.ii;
        ox += G.ii; oy += G.jj; oz += G.kk;
        c->minlevel = std::min(c->minlevel, G.level);
        c->maxlevel = std::max(c->maxlevel, G.level);
    }
    if (!check_supported(*c)) {
        delete c;
        return fail(MGLET_ERR_UNSUPPORTED,
                    "oracle: only CON, CO1, FIX, OP1, NOS, SLI and PAR faces are restated");
    }
    c->iparent.assign(d->ngrid + 1, 0);
    c->pos.assign(d->ngrid + 1, {0, 0, 0});
    c->idim3d = o3; c->idimx = ox; c->idimy = oy; c->idimz = oz;
    for (const char* n : {"U", "V", "W", "P", "G", "DU", "DV", "DW", "BP", "SDIV", "UO", "VO",
                          "WO", "DP", "HILF", "RHS", "RES", "GSAP", "PWU", "PWV", "PWW"})
        c->f3[n].assign(o3, 0.0);
    c->gcl.resize(d->ngrid + 1);
    c->gcf.resize(d->ngrid + 1);
    std::fill(c->f3["BP"].begin(), c->f3["BP"].end(), 1.0);       // noib_mod.F90:45-47
    auto set1 = [&](const char* n, const double* src, int64_t len) {
        c->f1[n].assign(src, src + len);
    };
    set1("X", d->x, c->idimx); set1("Y", d->y, c->idimy); set1("Z", d->z, c->idimz);
    set1("DX", d->dx, c->idimx); set1("DY", d->dy, c->idimy); set1("DZ", d->dz, c->idimz);
    set1("DDX", d->ddx, c->idimx); set1("DDY", d->ddy, c->idimy); set1("DDZ", d->ddz, c->idimz);
    // corefields_mod.F90:139-173 calc_reciprocal with divide0
    auto recip = [&](const char* r, const char* s) {
        const std::vector<double>& a = c->f1[s];
        std::vector<double>& b = c->f1[r];
        b.resize(a.size());
        for (size_t q = 0; q < a.size(); ++q) b[q] = a[q] == 0.0 ? 0.0 : 1.0 / a[q];
    };
    recip("RDDX", "DDX"); recip("RDDY", "DDY"); recip("RDDZ", "DDZ");
    recip("RDX", "DX"); recip("RDY", "DY"); recip("RDZ", "DZ");
    for (const char* n : {"GSAW", "GSAE"}) c->f1[n].assign(c->idimx, 0.0);
    for (const char* n : {"GSAS", "GSAN"}) c->f1[n].assign(c->idimy, 0.0);
    for (const char* n : {"GSAB", "GSAT"}) c->f1[n].assign(c->idimz, 0.0);
    // boundary buffers (zero until set) and OP1 parameters
    c->bufoff.assign(6 * (size_t)d->ngrid, 0);
    int64_t nb = 0;
    for (int g = 1; g <= d->ngrid; ++g) {
        const Grid& G = c->g[g];
        const int64_t sz[3] = {(int64_t)G.kk * G.jj, (int64_t)G.kk * G.ii, (int64_t)G.jj * G.ii};
        for (int f = 1; f <= 6; ++f) {
            c->bufoff[6 * (g - 1) + f - 1] = nb;
            nb += sz[(f - 1) / 2];
        }
    }
    c->bufU.assign(nb, 0.0); c->bufV.assign(nb, 0.0); c->bufW.assign(nb, 0.0);
    c->pinf.assign(6 * (size_t)d->ngrid, 0.0);
    c->npinf.assign(6 * (size_t)d->ngrid, 0);
    init_connect_core(*c);
    init_viscosity(*c);
    giteig(*c);
    int rc = init_pressuresolver(*c);
    if (rc) {
        delete c;
        return rc;
    }
    *out = c;
    return 0;
}

int oracle_destroy(oracle_ctx* c) {
    delete c;
    return 0;
}

int64_t oracle_idim3d(const oracle_ctx* c) { return c->idim3d; }

int oracle_set_field(oracle_ctx* c, const char* name, const double* host, int64_t n) {
    auto it = c->f3.find(name);
    if (it == c->f3.end()) return fail(MGLET_ERR_NAME, std::string("unknown field ") + name);
    if (n != c->idim3d) return fail(MGLET_ERR_SIZE, "size mismatch");
    std::copy(host, host + n, it->second.begin());
    if (std::strcmp(name, "G") == 0) c->g_user = true;
    return 0;
}

int oracle_get_field(oracle_ctx* c, const char* name, double* host, int64_t n) {
    auto it = c->f3.find(name);
    if (it == c->f3.end()) {
        auto i1 = c->f1.find(name);
        if (i1 == c->f1.end()) return fail(MGLET_ERR_NAME, std::string("unknown field ") + name);
        if (n != (int64_t)i1->second.size()) return fail(MGLET_ERR_SIZE, "size mismatch");
        std::copy(i1->second.begin(), i1->second.end(), host);
        return 0;
    }
    if (n != c->idim3d) return fail(MGLET_ERR_SIZE, "size mismatch");
    std::copy(it->second.begin(), it->second.end(), host);
    return 0;
}

// SIP_MIP_HP / SIP_IDX_HP (1-based values as the reference stores them)
int oracle_get_sip_index(oracle_ctx* c, int64_t* mip, int64_t* idx, int64_t n) {
    if (n != c->idim3d) return fail(MGLET_ERR_SIZE, "size mismatch");
    std::copy(c->mip.begin(), c->mip.end(), mip);
    std::copy(c->idxsip.begin(), c->idxsip.end(), idx);
    return 0;
}

// Number of connections (rows of sendconns) and their content.
int oracle_get_conns(oracle_ctx* c, int32_t* rows, int64_t maxrows, int64_t* nrows) {
    *nrows = (int64_t)c->conns.size();
    for (int64_t q = 0; q < *nrows && q < maxrows; ++q) {
        rows[4 * q + 0] = c->conns[q].recvgrid;
        rows[4 * q + 1] = c->conns[q].sendgrid;
        rows[4 * q + 2] = c->conns[q].recvface;
        rows[4 * q + 3] = c->conns[q].sendface;
    }
    return 0;
}

int oracle_tstle4(oracle_ctx* c) {
    tstle4(*c);
    return 0;
}

int oracle_rkstep(oracle_ctx* c, const char* p, const char* dp, const char* rhsp, double frhs,
                  double dtfu) {
    if (!c->f3.count(p) || !c->f3.count(dp) || !c->f3.count(rhsp))
        return fail(MGLET_ERR_NAME, "rkstep: unknown field");
    rkstep(c->F(p), c->F(dp), c->F(rhsp), c->idim3d, frhs, dtfu);
    return 0;
}

// Returns the number of copied points in *ncopied (the message-length check
// of connect2_mod.F90:879-885 is applied per connection).
int oracle_connect(oracle_ctx* c, int ilevel, int layers, const char* v1, const char* v2,
                   const char* v3, const char* s1, const char* s2, const char* s3, int corners,
                   int normal, int forward, int64_t* ncopied) {
    auto get = [&](const char* n) -> double* { return n ? c->F(n) : nullptr; };
    if (layers < 1 || layers > 2) return fail(MGLET_ERR_ARG, "connect: layers must be 1 or 2");
    if ((forward != 0 || normal) && corners) return fail(MGLET_ERR_ARG, "connect: bad flags");
    int64_t n;
    try {
        n = connect(*c, ilevel, layers, get(v1), get(v2), get(v3), get(s1), get(s2), get(s3),
                    corners != 0, normal != 0, forward);
    } catch (...) {
        return fail(MGLET_ERR_NAME, "connect: unknown field");
    }
    if (n < 0) return MGLET_ERR_ARG;
    if (ncopied) *ncopied = n;
    return 0;
}

int oracle_divcal(oracle_ctx* c, const char* div, double fak) {
    divcal(*c, c->F(div), c->F("U"), c->F("V"), c->F("W"), fak);
    return 0;
}

int oracle_laplacephi(oracle_ctx* c, const char* res, const char* phi) {
    laplacephi_level(*c, 0, c->F(res), c->F(phi));
    return 0;
}

int oracle_mgpoisl(oracle_ctx* c, double dt, int ittot, int irk, mglet_stage_stats* st) {
    (void)ittot; (void)irk;
    if (int rc = hierarchy_ready(*c)) return rc;
    mgpoisl(*c, dt, st);
    return 0;
}

// timeintegration_mod.F90:22-142 (noib, no LES, no Boussinesq/Coriolis)
int oracle_timeintegrate_flow(oracle_ctx* c, int itstep, int ittot, double timeph, double dt,
                              int irk, const mglet_rk_scheme* rk, mglet_stage_stats* st) {
    (void)itstep; (void)timeph;
    if (int rc = hierarchy_ready(*c)) return rc;
    double frhs, fu, dtrk, dtrki;
    int rc = oracle_rk_get_coeffs(rk, irk, &frhs, &fu, &dtrk, &dtrki);
    if (rc) return rc;
    const bool gc = c->ibtype == 1;
    // timeintegration_mod.F90:96-99: the ghost-cell fluxes of the step
    if (irk == 1 && gc)
        if (int rc2 = setibvalues(*c)) return rc2;
    tstle4(*c);
    boussinesqterm(*c);                                       // :102
    coriolisterm(*c);                                         // :103
    rkstep(c->F("U"), c->F("DU"), c->F("UO"), c->idim3d, frhs, dt * fu);
    rkstep(c->F("V"), c->F("DV"), c->F("VO"), c->idim3d, frhs, dt * fu);
    rkstep(c->F("W"), c->F("DW"), c->F("WO"), c->idim3d, frhs, dt * fu);
    if (gc) {   // :110-116
        maskbp(*c, c->F("U"), c->F("V"), c->F("W"), c->F("P"));
        if (int rc2 = gc_level(*c, 'R', c->F("U"), c->F("V"), c->F("W"))) return rc2;
    }
    // timeintegration_mod.F90:117-122: per level connect (normal, forward),
    // parent (u, v, w, p into the PAR buffers) and bound_flow
    const char* vn[3] = {"U", "V", "W"};
    const char* sn[3] = {"P", nullptr, nullptr};
    for (int l = c->minlevel; l <= c->maxlevel; ++l) {
        connect(*c, l, 1, c->F("U"), c->F("V"), c->F("W"), nullptr, nullptr, nullptr, false, true, 1);
        parent(*c, l, vn, sn, false);
        bound_flow(*c, c->F("U"), c->F("V"), c->F("W"), c->F("P"), l);
    }
    mgpoisl(*c, dtrk * dt, st);
    lesmodel(*c);                                             // :125
    (void)ittot;
    if (gc) return setpointvalues(*c, irk == rk->nrk);   // :131-134
    return 0;
}

int oracle_set_buffer(oracle_ctx* c, const char* name, int igrid, int iface, const double* data,
                      int64_t n) {
    if (!c || !name || !data || igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6)
        return fail(MGLET_ERR_ARG, "set_buffer: bad arguments");
    const Grid& G = c->g[igrid];
    const int64_t sz[3] = {(int64_t)G.kk * G.jj, (int64_t)G.kk * G.ii, (int64_t)G.jj * G.ii};
    if (n != sz[(iface - 1) / 2]) return fail(MGLET_ERR_SIZE, "set_buffer: wrong plane size");
    if (!c->f3.count(name)) return fail(MGLET_ERR_NAME, "set_buffer: unknown field");
    std::vector<double>& b = buffer_of(*c, name);
    std::copy(data, data + n, b.begin() + c->bufoff[6 * (igrid - 1) + iface - 1]);
    return 0;
}

int oracle_set_bc_real(oracle_ctx* c, int igrid, int iface, double value) {
    if (!c || igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6)
        return fail(MGLET_ERR_ARG, "set_bc_real: bad arguments");
    c->pinf[6 * (igrid - 1) + iface - 1] = value;
    c->npinf[6 * (igrid - 1) + iface - 1] = 1;
    return 0;
}

int oracle_set_stencils(oracle_ctx* c, int igrid, int comp, int ncells, const int64_t* xpoli,
                        int64_t nxi, const double* xpolr, int64_t nxr, const double* xpolrvel,
                        int64_t nxrv) {
    if (!c || igrid < 1 || igrid > c->ngrid || comp < 1 || comp > 4 || ncells < 0 ||
        (ncells > 0 && (!xpoli || !xpolr)))
        return fail(MGLET_ERR_ARG, "set_stencils: bad arguments");
    if (comp == 4) {
        GcFlux& F = c->gcf[igrid];
        if (nxi != 2LL * ncells || nxr != 7LL * ncells)
            return fail(MGLET_ERR_SIZE, "set_stencils: flux list sizes");
        F.fxpoli.assign(xpoli, xpoli + nxi);
        F.fxpolr.assign(xpolr, xpolr + nxr);
        F.ncells = ncells;
        return 0;
    }
    GcList& L = c->gcl[igrid][comp - 1];
    if (nxrv != nxr || (nxrv > 0 && !xpolrvel)) return fail(MGLET_ERR_SIZE, "set_stencils: xpolrvel");
    L.xpoli.assign(xpoli, xpoli + nxi);
    L.xpolr.assign(xpolr, xpolr + nxr);
    L.xpolrvel.assign(xpolrvel, xpolrvel + nxrv);
    L.ncells = ncells;
    L.oldsol.clear(); L.poldsol.clear(); L.oldsolvel.clear(); L.poldsolvel.clear();
    return 0;
}

int oracle_set_ghostcell(oracle_ctx* c) {
    if (!c) return fail(MGLET_ERR_ARG, "set_ghostcell: null context");
    if (c->minlevel != c->maxlevel)   // setsdivfield restricts SDIV level by level
        if (int rc = hierarchy_ready(*c)) return rc;
    c->ibtype = 1;
    giteig(*c);                       // Poisson coefficients with the blocked cells
    if (int rc = init_pressuresolver(*c)) return rc;
    setsdivfield(*c);
    if (c->f3.count("BT")) return blockbt(*c);   // scalars set before the blocking
    return 0;
}

int oracle_setpointvalues(oracle_ctx* c, int comp_new) {
    if (!c || c->ibtype != 1) return fail(MGLET_ERR_ARG, "setpointvalues: not a ghost-cell case");
    return setpointvalues(*c, comp_new != 0);
}

int oracle_gc_mode(oracle_ctx* c, const char* mode) {
    if (!c || !mode) return fail(MGLET_ERR_ARG, "gc_mode: bad arguments");
    if (mode[0] == 'M') {
        maskbp(*c, c->F("U"), c->F("V"), c->F("W"), c->F("P"));
        return 0;
    }
    if (mode[0] == 'I') return setibvalues(*c);
    return gc_level(*c, mode[0], c->F("U"), c->F("V"), c->F("W"));
}

int oracle_bound_flow(oracle_ctx* c, int ilevel) {
    bound_flow(*c, c->F("U"), c->F("V"), c->F("W"), c->F("P"), ilevel);
    return 0;
}

int oracle_set_hierarchy(oracle_ctx* c, const int32_t* iparent, const int32_t* pos) {
    if (!c || !iparent || !pos) return fail(MGLET_ERR_ARG, "set_hierarchy: bad arguments");
    for (int g = 1; g <= c->ngrid; ++g) {
        const int par = iparent[g - 1];
        if (par < 0 || par > c->ngrid || par == g) return fail(MGLET_ERR_ARG, "set_hierarchy: bad parent");
        if (par && c->g[par].level != c->g[g].level - 1)
            return fail(MGLET_ERR_ARG, "set_hierarchy: parent not one level coarser");
        c->iparent[g] = par;
        c->pos[g] = {pos[3 * (g - 1)], pos[3 * (g - 1) + 1], pos[3 * (g - 1) + 2]};
    }
    // the finer levels' G takes its PAR values now that the parents are known
    if (!c->g_user) init_viscosity(*c);
    return 0;
}

int oracle_get_buffer(oracle_ctx* c, const char* name, int igrid, int iface, double* data, int64_t n) {
    if (!c || !name || !data || igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6)
        return fail(MGLET_ERR_ARG, "get_buffer: bad arguments");
    const Grid& G = c->g[igrid];
    const int64_t sz[3] = {(int64_t)G.kk * G.jj, (int64_t)G.kk * G.ii, (int64_t)G.jj * G.ii};
    if (n != sz[(iface - 1) / 2]) return fail(MGLET_ERR_SIZE, "get_buffer: wrong plane size");
    const std::string nm(name);
    const std::vector<double>& b = buffer_of(*c, nm);
    const int64_t o = c->bufoff[6 * (igrid - 1) + iface - 1];
    std::copy(b.begin() + o, b.begin() + o + n, data);
    return 0;
}

int oracle_parent(oracle_ctx* c, int ilevel, const char* v1, const char* v2, const char* v3,
                  const char* s1, const char* s2, const char* s3, int normal) {
    if ((v1 != nullptr) != (v2 != nullptr) || (v1 != nullptr) != (v3 != nullptr))
        return fail(MGLET_ERR_ARG, "parent: give all three vector components or none");
    const char* v[3] = {v1, v2, v3};
    const char* sc[3] = {s1, s2, s3};
    for (const char* n : {v1, v2, v3, s1, s2, s3})
        if (n && !c->f3.count(n)) return fail(MGLET_ERR_NAME, "parent: unknown field");
    parent(*c, ilevel, v, sc, normal != 0);
    return 0;
}

int oracle_ftoc(oracle_ctx* c, int ilevel, const char* ff, const char* fc, char flag) {
    if (!c->f3.count(ff) || !c->f3.count(fc)) return fail(MGLET_ERR_NAME, "ftoc: unknown field");
    if (!std::strchr("UVWPRST", flag)) return fail(MGLET_ERR_ARG, "ftoc: flag is one of U V W P R S T");
    if (c->ibtype == 1 && flag == 'T' && !c->f3.count("BT"))
        return fail(MGLET_ERR_UNSUPPORTED, "ftoc: the ghost-cell T restriction weighs by BT (set_scalars first)");
    ftoc_one(*c, ilevel, ff, fc, flag);
    return 0;
}

int oracle_set_lesmodel(oracle_ctx* c, int model, double cm) {
    if (!c || (model != 0 && model != 1 && model != 2 && model != 5))
        return fail(MGLET_ERR_ARG, "set_lesmodel: model 0 (none), 1 (smagorinsky), 2 (wale) or 5 (sigma)");
    c->ilesmodel = model;
    c->cm = cm < 0.0 ? les_default_cm(model) : cm;
    // init_lesmodel (lesmodel_mod.F90:63-80): G of the current field
    if (model == 0) init_viscosity(*c);
    else lesmodel(*c);
    return 0;
}

int oracle_set_scalars(oracle_ctx* c, int nsca, const double* prmol, const int32_t* kayscrawford,
                       const double* source, double prturb) {
    if (!c || nsca < 0 || nsca > 9 || (nsca && (!prmol || !kayscrawford)))
        return fail(MGLET_ERR_ARG, "set_scalars: 0..9 scalars with prmol and kayscrawford");
    c->sca.clear();
    for (int l = 0; l < nsca; ++l) {
        Ctx::ScalarDef sd;
        sd.name = "T" + std::to_string(l + 1);
        sd.prmol = prmol[l];
        sd.kayscrawford = kayscrawford[l];
        if (source && source[l] != 0.0) sd.sources.push_back({"", source[l]});
        c->sca.push_back(sd);
        c->f3[sd.name].assign(c->idim3d, 0.0);
        c->f3["D" + sd.name].assign(c->idim3d, 0.0);
        c->f3[sd.name + "_OLD"].assign(c->idim3d, 0.0);
    }
    c->prturb = prturb;
    for (const char* n : {"QTU", "QTV", "QTW", "QTT", "BT"}) c->f3[n].assign(c->idim3d, 0.0);
    std::fill(c->f3["BT"].begin(), c->f3["BT"].end(), 1.0);   // blockbt: open everywhere (noib)
    if (c->ibtype == 1) return blockbt(*c);
    return 0;
}

int oracle_set_scastencils(oracle_ctx* c, int igrid, int ncells, const int64_t* xpoli, const double* xpolr,
                           const double* xpolrvel) {
    if (!c || igrid < 1 || igrid > c->ngrid || ncells < 0 || (ncells && (!xpoli || !xpolr || !xpolrvel)))
        return fail(MGLET_ERR_ARG, "set_scastencils: bad grid or lists");
    const Grid& G = c->g[igrid];
    const int64_t npts = (int64_t)G.kk * G.jj * G.ii;
    for (int cell = 0; cell < ncells; ++cell) {
        const int64_t* xi = xpoli + (size_t)cell * kScaIsize;
        if (xi[0] < 1 || xi[0] > npts || xi[2] < 0 || xi[2] > kScaNperi)
            return fail(MGLET_ERR_ARG, "set_scastencils: cell or stencil count out of range");
        for (int64_t n = 1; n <= xi[2]; ++n)
            if (xi[2 + n] < 1 || xi[2 + n] > npts) return fail(MGLET_ERR_ARG, "set_scastencils: stencil cell out of range");
    }
    if ((int)c->scal.size() < c->ngrid + 1) c->scal.resize(c->ngrid + 1);
    Ctx::ScaList& L = c->scal[igrid];
    L.ncells = ncells;
    L.xpoli.assign(xpoli, xpoli + (size_t)ncells * kScaIsize);
    L.xpolr.assign(xpolr, xpolr + (size_t)ncells * kScaRsize);
    L.xpolrvel.assign(xpolrvel, xpolrvel + (size_t)ncells * kScaRsize);
    return 0;
}

int oracle_set_scalar_geometry(oracle_ctx* c, int isca, int nbody, const int32_t* flag, const double* value) {
    if (!c || isca < 1 || isca > (int)c->sca.size() || nbody < 0 || (nbody && (!flag || !value)))
        return fail(MGLET_ERR_ARG, "set_scalar_geometry: bad scalar or bodies");
    for (int b = 0; b < nbody; ++b)
        if (flag[b] != 0 && flag[b] != 1) return fail(MGLET_ERR_ARG, "set_scalar_geometry: flag 0 or 1");
    c->sca[isca - 1].geo_flag.assign(flag, flag + nbody);
    c->sca[isca - 1].geo_value.assign(value, value + nbody);
    return 0;
}

int oracle_add_scalar_source(oracle_ctx* c, int isca, const char* field, double value) {
    if (!c || isca < 1 || isca > (int)c->sca.size())
        return fail(MGLET_ERR_ARG, "add_scalar_source: no such scalar");
    const std::string f = field ? field : "";
    if (!f.empty() && !c->f3.count(f)) return fail(MGLET_ERR_NAME, "add_scalar_source: unknown field");
    if (c->sca[isca - 1].sources.size() >= 8) return fail(MGLET_ERR_ARG, "add_scalar_source: at most 8 sources");
    c->sca[isca - 1].sources.push_back({f, value});
    return 0;
}

int oracle_set_scalar_bc(oracle_ctx* c, int igrid, int iface, int kind, const int32_t* types) {
    if (!c || igrid < 1 || igrid > c->ngrid || iface < 1 || iface > 6 || kind < 0 || kind > 2 ||
        (kind && !types))
        return fail(MGLET_ERR_ARG, "set_scalar_bc: bad arguments");
    const int t = c->g[igrid].bc[iface];
    if (kind && (t == MGLET_BC_CON || t == MGLET_BC_CO1 || t == MGLET_BC_PAR))
        return fail(MGLET_ERR_ARG, "set_scalar_bc: SWA and SIO sit on boundary faces");
    if (c->scabc_kind.empty()) {
        c->scabc_kind.assign(6 * (size_t)c->ngrid, 0);
        c->scabc_type.assign(6 * (size_t)c->ngrid * 9, 0);
    }
    const size_t x = 6 * (size_t)(igrid - 1) + iface - 1;
    c->scabc_kind[x] = kind;
    for (size_t l = 0; l < c->sca.size() && kind; ++l) {
        if (types[l] != 0 && types[l] != 1) return fail(MGLET_ERR_ARG, "set_scalar_bc: type 0 or 1");
        c->scabc_type[x * 9 + l] = types[l];
    }
    return 0;
}

int oracle_timeintegrate_scalar(oracle_ctx* c, double dt, int irk, const mglet_rk_scheme* rk) {
    if (!c || !rk) return fail(MGLET_ERR_ARG, "timeintegrate_scalar: null argument");
    if (int rc = hierarchy_ready(*c)) return rc;
    return timeintegrate_scalar(*c, dt, irk, rk);
}

int oracle_set_buoyancy(oracle_ctx* c, const double* gravity, double beta, int iscalar) {
    if (!c || !gravity || iscalar < 1 || iscalar > (int)c->sca.size())
        return fail(MGLET_ERR_ARG, "set_buoyancy: gravity and a scalar 1..nsca");
    for (int q = 0; q < 3; ++q) c->gravity[q] = gravity[q];
    c->beta = beta;
    c->buoyancy_scalar = iscalar;
    c->buoyancy = true;
    return 0;
}

int oracle_set_coriolis(oracle_ctx* c, const double* omega) {
    if (!c || !omega) return fail(MGLET_ERR_ARG, "set_coriolis: null argument");
    for (int q = 0; q < 3; ++q) c->omega[q] = omega[q];
    c->coriolis = true;
    return 0;
}

int oracle_set_body_force(oracle_ctx* c, const double* fx, const double* fy, const double* fz,
                          int64_t n) {
    if (!c || !fx || !fy || !fz) return fail(MGLET_ERR_ARG, "set_body_force: bad arguments");
    if (n != c->idim3d) return fail(MGLET_ERR_SIZE, "set_body_force: n must equal idim3d");
    c->f3["FBX"].assign(fx, fx + n);
    c->f3["FBY"].assign(fy, fy + n);
    c->f3["FBZ"].assign(fz, fz + n);
    c->bodyforce = true;
    return 0;
}

int oracle_par_ftoc_norm(oracle_ctx* c, int ilevel, const char* v1, const char* v2, const char* v3,
                         int sum) {
    if (!c || !v1 || !v2 || !v3) return fail(MGLET_ERR_ARG, "par_ftoc_norm: bad arguments");
    for (const char* n : {v1, v2, v3})
        if (!c->f3.count(n)) return fail(MGLET_ERR_NAME, "par_ftoc_norm: unknown field");
    par_ftoc_norm(*c, ilevel, c->F(v1), c->F(v2), c->F(v3), sum != 0);
    return 0;
}

int oracle_ftoc_multiple(oracle_ctx* c, int ilevel, const char* v1, const char* v2, const char* v3,
                         const char* s1, const char* s2, const char* s3) {
    const char* n[6] = {v1, v2, v3, s1, s2, s3};
    const char fl[6] = {'U', 'V', 'W', 'P', 'P', 'P'};
    for (int q = 0; q < 6; ++q)
        if (n[q] && !c->f3.count(n[q])) return fail(MGLET_ERR_NAME, "ftoc: unknown field");
    for (int q = 0; q < 6; ++q)
        if (n[q]) ftoc_one(*c, ilevel, n[q], n[q], fl[q]);
    return 0;
}

int oracle_ctof(oracle_ctx* c, int ilevel, const char* ff, const char* fc) {
    if (!c->f3.count(ff) || !c->f3.count(fc)) return fail(MGLET_ERR_NAME, "ctof: unknown field");
    ctof(*c, ilevel, ff, fc);
    return 0;
}

int oracle_bound_pressure(oracle_ctx* c, int ilevel, const char* name, int withbp) {
    if (!c->f3.count(name)) return fail(MGLET_ERR_NAME, "bound_pressure: unknown field");
    bound_pressure(*c, ilevel, name, withbp != 0);
    return 0;
}

int oracle_set_partition(oracle_ctx* c, const int32_t* halo, int32_t nsend, const int32_t* send,
                         int32_t nrecv, const int32_t* recv, mglet_exchange_fn fn, void* user) {
    if (!halo || !fn || c->minlevel != c->maxlevel)
        return fail(MGLET_ERR_ARG, "set_partition: one level, halo flags and a function");
    for (int g = 1; g <= c->ngrid; ++g) c->g[g].halo = halo[g - 1] != 0;
    c->xfn = fn;
    c->xuser = user;
    c->peers.clear();
    for (int r = 0; r < nsend; ++r) c->peers.push_back(send[8 * r]);
    for (int r = 0; r < nrecv; ++r) c->peers.push_back(recv[8 * r]);
    std::sort(c->peers.begin(), c->peers.end());
    c->peers.erase(std::unique(c->peers.begin(), c->peers.end()), c->peers.end());
    c->xsend.assign(c->peers.size(), {});
    c->xrecv.assign(c->peers.size(), {});
    auto add = [&](const int32_t* rows, int n, std::vector<std::vector<std::array<int, 7>>>& out) {
        for (int r = 0; r < n; ++r) {
            const int32_t* w = rows + 8 * r;
            const int q = (int)(std::lower_bound(c->peers.begin(), c->peers.end(), w[0]) - c->peers.begin());
            out[q].push_back({w[1], w[2], w[3], w[4], w[5], w[6], w[7]});
        }
    };
    add(send, nsend, c->xsend);
    add(recv, nrecv, c->xrecv);
    return 0;
}

int oracle_itinfo(oracle_ctx* c, double dt, mglet_itinfo* out) {
    itinfo(*c, dt, out);
    return 0;
}

}  // extern "C"
