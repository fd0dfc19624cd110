// internal.h -- shared declarations of the GB300 stage library.
//
// Device data layout: every 3-D field is one flat FP64 (or FP32 for the
// mixed-form inner solver) array over all grids, grid g starting at ip3(g),
// Fortran order (k fastest) inside a grid -- the reference's field_t%arr
// layout (src/core/pointers_mod.F90:23-75), so host<->device copies are
// single memcpys.  Each 24^3 grid slab (28^3 points incl. ghosts) is
// 175,616 bytes, a multiple of 256, so every grid starts 256-byte aligned.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/mglet_gpu.h"

namespace mg {

// Per-grid record visible to kernels.
struct DevGrid {
    int kk, jj, ii;
    int level;
    int bc[6];          // faces 1..6 -> bc[0..5]
    int gradpflag;
    int cls;            // index of the SIP index table of this grid's dims
    long long ip3;      // 0-based element offset of the 3-D slab
    int ipx, ipy, ipz;  // 0-based offsets into the concatenated 1-D arrays
    int halo;           // 1: read-only copy of a grid another rank owns
};

// Boundary data of one face of one grid.
struct BFace {
    long long off;      // offset of the face plane in the buffer arrays
    double pinf;        // OP1 far-field pressure (0 unless set)
};

// Ghost-cell lists of one grid as the caller set them
struct GcHostList {
    int n[4] = {0, 0, 0, 0};
    std::vector<long long> xi[4];
    std::vector<double> xr[4], xv[3];
};

// Device copies: per grid and component the offsets of its lists in the
// concatenated arrays (components 0..2: xpoli / xpolr / xpolrvel / save
// buffers; 3: flux-correction lists)
struct GcSeg {
    long long xi, xr, sv;   // offsets into xpoli, xpolr (= xpolrvel), save buffers
    int n;
    // the list's cells in dependency levels: cells cell0 + lvstart[lv0 + L]
    // .. cell0 + lvstart[lv0 + L + 1] of the cell table form level L (nlv
    // levels); within a level no cell writes what another reads or writes
    int cell0, lv0, nlv;
};
struct GcDev {
    GcSeg* seg = nullptr;           // [ngrid][4]
    long long* xpoli = nullptr;
    double *xpolr = nullptr, *xpolrvel = nullptr;
    double *oldsol = nullptr, *oldsolvel = nullptr;
    long long *poldsol = nullptr, *poldsolvel = nullptr;
    // per cell {offset of its record in the segment's xpoli, in its xpolr,
    // its position in the list, 0}, ordered by segment and level
    int4* cell = nullptr;
    int* lvstart = nullptr;
};

// One box copy of connect_self_single (connect2_mod.F90:947-995): the
// destination box starts at dst (flat element offset), the source box at
// src; extents nk*nj*ni with per-grid strides.
// One message of par_ftoc_norm (par_ftoc_mod.F90:513-779): the PAR face
// iface of fine grid gf into grid gc, whose plane of coarse faces starts at
// (i0, j0, k0) and runs na x nb along the two in-plane directions.
struct PfTask {
    int gf, gc, iface;
    int i0, j0, k0;
    int na, nb;
};

struct BoxCopy {
    long long dst, src;
    int nk, nj, ni;
    int dkk, djj;       // destination grid kk, kk*jj would overflow int? (no: <= 2^31)
    int skk, sjj;
    int slot;           // which field slot (0..5: v1 v2 v3 s1 s2 s3)
    int npts;
};

struct ConnectPlan {
    BoxCopy* d_tasks = nullptr;
    int ntasks = 0;
    long long npts = 0;
    // the same tasks grouped by the grid they read (the adjoint's transposed
    // copies add into the sources: one group per CTA, in a fixed order),
    // built on first use; group s is d_bysrc[d_srcstart[s] .. d_srcstart[s+1])
    BoxCopy* d_bysrc = nullptr;
    int* d_srcstart = nullptr;
    int nsrc = 0;
};

// Hyperplane traversal table of one grid shape (sip_hyperplane_mod.F90:269-334):
// plane start offsets mip[m] (0-based, m = 9..n3dmax+1) and the 0-based
// local linear index of every interior point in plane order.
struct HpTable {
    int kk, jj, ii;
    int n3dmin, n3dmax;
    int* d_mip = nullptr;   // [kk+jj+ii+2]
    int* d_idx = nullptr;   // [(kk-4)(jj-4)(ii-4)]
    int maxplane = 0;
    int npts = 0;
};

struct ProfEntry {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    double total_ms = 0.0;
    long long launches = 0;
};

struct MixedState;   // mixed.cu
struct Part;         // dist.cu

struct Ctx {
    MixedState* mx = nullptr;
    Part* part = nullptr;      // grid partition over ranks (null: one rank)
    int device = 0;
    cudaStream_t stream = nullptr;
    int ngrid = 0;
    int minlevel = 0, maxlevel = 0;
    long long idim3d = 0;
    int idimx = 0, idimy = 0, idimz = 0;
    bool uniform = true;      // all grids share kk, jj, ii
    mglet_flow_params prm{};
    std::vector<DevGrid> grids;            // host copy
    std::vector<std::vector<int>> nbr;     // [ngrid][27] 1-based neighbour ids
    std::vector<int> levelgrids_count;
    DevGrid* d_grids = nullptr;
    std::map<std::string, double*> f3;     // 3-D FP64 fields
    std::map<std::string, double*> f1;     // 1-D FP64 spacing / coefficient arrays
    std::vector<HpTable> hp;               // one per distinct grid shape
    std::vector<int> d_cls_host;
    // connection table rows (recvgrid, sendgrid, recvface, sendface), 1-based
    std::vector<int> conns;
    std::map<std::string, ConnectPlan> plans;
    // reductions
    double* d_gridred = nullptr;   // [4*ngrid]
    int* d_bpone = nullptr;
    double* d_guni = nullptr;      // [2*ngrid] tstle4's uniform-G flag and face mean        // [ngrid] 1 where BP is 1.0 at every point laplacephi reads
    double* d_scalar = nullptr;    // [8]
    double* h_scalar = nullptr;    // pinned [8]
    // boundary buffers of U, V, W (field_t%get_buffer): one plane per grid and
    // face, (kk,jj) / (kk,ii) / (jj,ii) column-major, at bface[6*g+f].off;
    // bface also holds the OP1 far-field pressure of the face
    double* d_buf[3] = {nullptr, nullptr, nullptr};
    std::vector<BFace> bface;
    BFace* d_bface = nullptr;
    long long nbuf = 0;
    // grids (0-based) with a FIX/OP1/NOS/SLI face, per face
    std::vector<int> bgrids[6];
    int* d_bgrids[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // ghost-cell IB: 0 NONE, 1 GHOSTCELL; host lists per grid (1..3 u, v, w;
    // 4 flux correction) until gc_upload, then their device copies
    int ibtype = 0;
    // the ghost-cell saves of setibvalues ('S') and setpointvalues ('Z')
    // have run since the lists were set: their restores may follow
    bool gc_saved[2] = {false, false};
    bool bodyforce = false;      // FBX, FBY, FBZ added in tstle4 (plain form)
    bool g_user = false;         // G set by the caller: set_hierarchy keeps it
    // passive scalars T1..Tn (scacore_mod.F90): molecular Prandtl number,
    // Kays/Crawford switch, constant source
    struct ScalarDef {
        std::string name;
        double prmol = 1.0;
        int kayscrawford = 0;
        // sources in order: empty field name = constant (sourceterm_const),
        // else value * field (sourceterm_field)
        std::vector<std::pair<std::string, double>> sources;
        // per body of the ghost-cell IB (sca%geometries): flag 0 fixed
        // value, 1 fixed flux, and the value
        std::vector<int> geo_flag;
        std::vector<double> geo_value;
    };
    std::vector<ScalarDef> sca;
    double prturb = 1.0;
    // scalar conditions beside a face's flow condition: kind 1 SWA (wall),
    // 2 SIO (in/outflow); per scalar 0 fixed value, 1 fixed flux
    std::vector<int> scabc_kind, scabc_type;
    int *d_scabc_kind = nullptr, *d_scabc_type = nullptr;
    // boussinesqterm_mod.F90 / coriolisterm_mod.F90 parameters
    bool buoyancy = false, coriolis = false;
    double gravity[3] = {0.0, 0.0, 0.0}, beta = 0.0, omega[3] = {0.0, 0.0, 0.0};
    int buoyancy_scalar = 1;
    int ilesmodel = 0;           // 0 none, 1 smagorinsky, 2 wale, 5 sigma
    bool fma = false;            // MGLET_FORM_PLAIN_FMA: the plain kernels' contracted build
    double cm = 0.0;             // the LES model constant
    void* d_sptab = nullptr;     // device table of the 12 spacing arrays (adjoint)
    std::vector<GcHostList> gch;
    GcDev gcd;
    // scalar ghost-cell lists (gc_scastencils_mod.F90:10-16) per grid: per
    // cell 9 integers {intcell, body, nstencils, six stencil cells} and 8
    // reals {areabyvol, six coefficients, acoeffvel}; on the device all
    // grids' records back to back with the first cell of each grid
    struct ScaList {
        int ncells = 0;
        std::vector<int64_t> xpoli;
        std::vector<double> xpolr, xpolrvel;
    };
    std::vector<ScaList> scal;
    long long* d_sxi = nullptr;
    double *d_sxr = nullptr, *d_sxrv = nullptr;
    long long* d_scell0 = nullptr;   // [ngrid + 1]
    int scal_maxbody = 0;            // the largest body number in the lists
    // grid hierarchy (gridinfo%iparent, i/j/kposition): per grid {parent
    // 0-based or -1, iposition, jposition, kposition}; per level the grids
    // with a parent (ftoc / ctof) and per level and face the grids with a
    // PAR face there (parent, bound_flow, bound_pressure); boundary buffers
    // of fields other than U, V, W, allocated on first use
    std::vector<int4> hier;
    int4* d_hier = nullptr;
    int* d_ftoc_skip = nullptr;     // [ngrid] sibling faces a grid does not restrict
    std::map<int, std::vector<int>> children;
    std::map<int, int*> d_children;
    std::vector<int> pgrids[6];
    int* d_pgrids[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int* d_pargrids = nullptr;                  // grids with any PAR face (tstle4_par)
    std::map<int, std::vector<PfTask>> pftasks; // per level: par_ftoc_norm messages
    std::map<int, PfTask*> d_pftasks;
    int npargrids = 0;
    std::map<int, std::vector<int>> plist[6];   // per level: grids with a parent and PAR on the face
    std::map<int, int*> d_plist[6];
    std::map<std::string, double*> fbuf;
    long long launches = 0;
    bool prof = false;
    std::map<std::string, ProfEntry> profd;

    double* F(const char* n) { return f3.at(n); }
    double* L(const char* n) { return f1.at(n); }
};

// ---- error reporting -------------------------------------------------------
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define MG_CUDA(call)                                            \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return ::mg::cuda_fail(e_, #call); \
    } while (0)

// Host <-> device copies and fills ordered on a stream.  The context's stream
// is non-blocking, so the legacy-stream cudaMemcpy / cudaMemset are not
// ordered with its kernels; copies also wait for completion, so the host
// buffer may be released right after.
inline cudaError_t copy_on(cudaStream_t s, void* dst, const void* src, size_t n,
                           cudaMemcpyKind kind) {
    cudaError_t e = cudaMemcpyAsync(dst, src, n, kind, s);
    return e != cudaSuccess ? e : cudaStreamSynchronize(s);
}
inline cudaError_t zero_on(cudaStream_t s, void* p, size_t n) { return cudaMemsetAsync(p, 0, n, s); }

#define MG_LAUNCHED(ctx)                                              \
    do {                                                              \
        (ctx)->launches++;                                            \
        cudaError_t e_ = cudaGetLastError();                          \
        if (e_ != cudaSuccess) return ::mg::cuda_fail(e_, "launch");  \
    } while (0)

// Brackets the kernels launched in its scope with CUDA events on the
// context's stream while profiling is enabled.
struct ProfScope {
    Ctx* c;
    ProfEntry* e = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(Ctx* ctx, const char* name) : c(ctx) {
        if (!c->prof) return;
        e = &c->profd[name];
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, c->stream);
    }
    ~ProfScope() {
        if (!e) return;
        cudaEventRecord(b, c->stream);
        e->pending.emplace_back(a, b);
    }
};

// ---- kernels: FP64 parity form (plain_*.cu, compiled with -fmad=false) ---
// The flux and Poisson kernels (plain_flux.cu, plain_poisson.cu) are also
// compiled a second time with multiply-add contraction, into mg::contract: the
// plain form's performance build (MGLET_FORM_PLAIN_FMA).  MG_PLAIN_FN picks
// the build the context runs.
#include "plain_decl.h"
namespace contract {
#include "plain_decl.h"
}
#define MG_PLAIN_FN(c, fn) ((c)->fma ? ::mg::contract::fn : ::mg::fn)
#ifdef MG_FMA_BUILD
#define MG_PLAIN_BEGIN namespace contract {
#define MG_PLAIN_END }
#else
#define MG_PLAIN_BEGIN
#define MG_PLAIN_END
#endif
int launch_itinfo(Ctx* c, double dt);
// bound_flow%bound on U, V, W and (unless null) P: faces 1..6 in order, the
// grids of ilevel (0: all levels)
int launch_bound_flow(Ctx* c, double* u, double* v, double* w, double* p, int ilevel = 0);
// multi-level operators (plain_level.cu)
int level_init(Ctx* c);                      // PAR face lists (create)
int init_viscosity(Ctx* c);                  // G of init_lesmodel, model "none"
int launch_bound_g(Ctx* c, int ilevel);      // the bound of G (lesmodel_mod.F90:573-764)
int lesmodel(Ctx* c);                        // G from the LES model (les.cu)
int set_lesmodel(Ctx* c, int model, double cm);
// scalar ghost-cell IB (scalar.cu): BT from BP, the lists, the conditions
int scalar_blockbt(Ctx* c);
int set_scastencils(Ctx* c, int igrid, int ncells, const int64_t* xpoli, const double* xpolr,
                    const double* xpolrvel);
int set_scalar_geometry(Ctx* c, int isca, int nbody, const int32_t* flag, const double* value);
int fill_field(Ctx* c, double* a, double v);   // a[0..idim3d) = v (api.cu)
// scalar transport (scalar.cu)
int set_scalars(Ctx* c, int nsca, const double* prmol, const int32_t* kayscrawford, const double* source,
                double prturb);
int timeintegrate_scalar(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk);
// boussinesqterm and coriolisterm on UO, VO, WO after tstle4 (scalar.cu)
int launch_momentum_sources(Ctx* c);
int set_scalar_bc(Ctx* c, int igrid, int iface, int kind, const int32_t* types);
int add_scalar_source(Ctx* c, int isca, const char* field, double value);
int set_hierarchy(Ctx* c, const int32_t* iparent, const int32_t* pos);
double* field_buffer(Ctx* c, const std::string& name);   // boundary buffers of a field
int launch_bound_par(Ctx* c, int iface, int ilevel, double* u, double* v, double* w);
// tstle4_par on every grid with a PAR face, after kon, diff and gradp
int launch_tstle4_par(Ctx* c, double* uo, double* vo, double* wo, const double* u, const double* v,
                      const double* w, const double* ut, const double* vt, const double* wt);
int launch_parent(Ctx* c, int ilevel, const char* const v[3], const char* const s[3], bool normal);
int launch_ftoc(Ctx* c, int ilevel, const double* ff, double* fc, char flag);
int launch_ctof(Ctx* c, int ilevel, double* ff, const double* fc);
int launch_bound_pressure(Ctx* c, int ilevel, double* p, const double* buf, bool withbp);
// boundary buffers and face table (create)
int bound_init(Ctx* c);
// 3-D FP64 field of idim3d points, zeroed (api.cu)
int alloc_field3(Ctx* c, const char* name);
// ghost-cell IB (plain_gc.cu)
int gc_upload(Ctx* c);                       // lists to the device, PWU/PWV/PWW, SDIV
// the outer loop of mgpoisl on RHS into DP (api.cu)
int solve_pressure_system(Ctx* c, double prefak, mglet_stage_stats* st, bool zero_work = true);
int rk_coeffs(const mglet_rk_scheme* rk, int irk, double* frhs, double* fu, double* dtrk,
              double* dtrki);
int timeintegrate(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk, mglet_stage_stats* st);
// the discrete adjoint (adjoint.cu)
int adjoint_ready(Ctx* c);
int adjoint_stage(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk);
int energy_gradient_init(Ctx* c, double* J);
int adjoint_fold_initial(Ctx* c);
int energy_gradient(Ctx* c, int nsteps, int ncheck, double dt, const mglet_rk_scheme* rk, double* J);
// F C S R X Y Z on the grids of ilevel (0: every grid)
int launch_gc_mode(Ctx* c, char mode, double* u, double* v, double* w, int ilevel = 0);
// par_ftoc_norm (par_ftoc_mod.F90:36-64) of the grids of ilevel
int launch_par_ftoc_norm(Ctx* c, int ilevel, double* u, double* v, double* w, bool sum);
int launch_maskbp(Ctx* c, double* u, double* v, double* w, double* p);
int gc_setibvalues(Ctx* c, double* u, double* v, double* w);
int gc_setpointvalues(Ctx* c, bool comp_new);
int launch_connect(Ctx* c, const ConnectPlan& plan, double* const fields[6]);
// connect(ilevel, layers, v1..s3, corners, normal, forward) (api.cu)
int connect(Ctx* c, int ilevel, int layers, double* v1, double* v2, double* v3, double* s1,
            double* s2, double* s3, bool corners, bool normal, int forward);
// FP32 copy of the same task list; returns early when *skip != 0 (device
// flag of the mixed form's converged outer loop), skip may be null.
int launch_connect32(Ctx* c, const ConnectPlan& plan, float* const fields[6], const int* skip);
int get_plan(Ctx* c, int ilevel, int layers, int slots, bool corners, bool normal, int fwd,
             const ConnectPlan** out);
// grid-partitioned runs (dist.cu): halo copies refreshed before a connect,
// reductions completed across ranks (op 1 max, 2 sum), release
int part_exchange(Ctx* c, double* const fields[6]);
int part_allreduce(Ctx* c, double* v, int n, int op);
int set_partition(Ctx* c, const int32_t* halo, int nsend, const int32_t* send, int nrecv,
                  const int32_t* recv, mglet_exchange_fn fn, void* user);
void part_release(Ctx* c);

}  // namespace mg
