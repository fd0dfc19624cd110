/*
 * mglet_gpu.h -- C ABI of the GB300 implementation of MGLET-base's
 * Runge-Kutta stage (momentum fluxes, RK update, pressure-Poisson solve with
 * divergence and projection, intra-level halo copies).
 *
 * Conventions (mirroring the reference's own C interop, e.g.
 * src/core/exprtk_wrapper.h:18-24, src/core/jsoncpp_wrapper.h:11-30):
 *   - every entry point returns an int status: 0 = ok, > 0 = error
 *     (MGLET_ERR_*); the Fortran side turns a nonzero status into
 *     errr(__FILE__, __LINE__) exactly as it does for its other C helpers;
 *   - scalars by value, arrays as plain pointers plus element counts;
 *   - the library never takes ownership of caller memory.
 *
 * Storage contract (src/core/pointers_mod.F90:23-75, field_t%arr):
 *   a 3-D field is one flat array over all grids, grid g (1-based, in grid
 *   order) starting at element ip3(g) = sum of kk*jj*ii of grids 1..g-1;
 *   inside a grid the layout is Fortran column-major (k fastest), with two
 *   ghost layers on each side (interior k = 3..kk-2 etc.).  1-D spacing
 *   arrays are concatenated per grid the same way (ip1x/ip1y/ip1z).
 *   Real type is FP64 (the reference's -DMGLET_REAL64=ON build).
 */
#ifndef MGLET_GPU_H
#define MGLET_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGLET_GPU_ABI_VERSION 1

/* Status codes */
enum {
    MGLET_OK = 0,
    MGLET_ERR_ARG = 1,          /* invalid argument / inconsistent description */
    MGLET_ERR_UNSUPPORTED = 2,  /* feature of the reference not built (e.g. PAR faces) */
    MGLET_ERR_CUDA = 3,         /* CUDA runtime error; see mglet_gpu_last_error() */
    MGLET_ERR_NAME = 4,         /* unknown field name */
    MGLET_ERR_SIZE = 5,         /* element count does not match the field */
    MGLET_ERR_EXPLODED = 6,     /* NaN/Inf detected (itinfo "exploded") */
    MGLET_ERR_NOMEM = 7         /* device allocation failed */
};

/* Boundary-condition type codes of itypboconds(1, iface, igrid),
 * src/core/grids_mod.F90:252-289 (setcobone). */
enum {
    MGLET_BC_FIX = 2,
    MGLET_BC_OP1 = 3,
    MGLET_BC_NOS = 5,
    MGLET_BC_SLI = 6,
    MGLET_BC_CON = 7,
    MGLET_BC_PAR = 8,
    MGLET_BC_CO1 = 19
};

/* Pressure solver types, src/flow/pressuresolver_mod.F90:17-21,96-107. */
enum {
    MGLET_PSOLVER_SIP = 0,      /* hyperplane SIP (default "sip") */
    MGLET_PSOLVER_SOR = 1,      /* SIP on minlevel, red-black SOR above ("sor") */
    MGLET_PSOLVER_CLASSIC = 2   /* lexicographic SIP ("classic") */
};

/* Execution forms of the stage. */
enum {
    /* FP64 throughout, reference operation order, no FMA contraction:
     * the parity form (relative L2 <= 1e-12 against the FP64 oracle). */
    MGLET_FORM_PLAIN = 0,
    /* Batched mixed precision: FP64 velocity/pressure storage, FP64
     * projection and reductions, float-float outer defect-correction
     * residual, FP32 fluxes and inner SIP sweeps; stage captured in one
     * CUDA graph with a device-side convergence flag.  Runs grids of equal
     * dimensions with CON, CO1, FIX, NOS, SLI, PAR (hierarchies, SIP on
     * every level) and OP1 faces (OP1 on the high faces 2, 4, 6), with or
     * without the ghost-cell IB (BP of 0 or 1), and with an LES model or a
     * caller-set viscosity field G (the fluxes then read G at every point;
     * the LES model itself runs in FP64). */
    MGLET_FORM_MIXED = 1,
    /* The plain FP64 form with multiply-add contraction in its flux and
     * Poisson kernels (the performance build the parity bar allows): the
     * same operations in the same order, each a*b+c rounded once, so the
     * fields stay within a relative 1e-12 of the reference instead of
     * matching it bit for bit. */
    MGLET_FORM_PLAIN_FMA = 2
};

/* Grid hierarchy description: what grids.h5 (GRIDINFO + BC tables,
 * src/core/gridio_mod.F90:12-46) and the spacing arrays of
 * src/core/corefields_mod.F90:98-151 hold for a single-rank run. */
typedef struct mglet_grid_desc {
    int32_t ngrid;
    const int32_t* mgdims;    /* [ngrid][3]: kk, jj, ii (incl. ghosts)   */
    const int32_t* level;     /* [ngrid]                                   */
    const int32_t* bctype;    /* [ngrid][6]: faces F,B,R,L,Bo,T (1..6)     */
    const int32_t* nbrgrid;   /* [ngrid][26]: neighbour grid ids (1-based,
                                 0 = none), NBRGRID of grids.h5          */
    const int32_t* gradpflag; /* [ngrid] or NULL (= all 1)                 */
    /* concatenated 1-D arrays; x/dx/ddx have sum(ii) entries etc. */
    const double* x;   const double* y;   const double* z;
    const double* dx;  const double* dy;  const double* dz;
    const double* ddx; const double* ddy; const double* ddz;
} mglet_grid_desc;

/* Flow and pressure-solver parameters (src/flow/flowcore_mod.F90:30-148,
 * src/flow/pressuresolver_mod.F90:47-145). */
typedef struct mglet_flow_params {
    double gmol;
    double rho;
    double gradp[3];
    int32_t psolver;      /* MGLET_PSOLVER_* */
    int32_t ninner;
    int32_t nouter;
    int32_t nouter_min;
    double epcorr;
    double omega;         /* SOR relaxation factor */
    int32_t form;         /* MGLET_FORM_* */
    int32_t reserved;
} mglet_flow_params;

/* Low-storage (2N) Runge-Kutta scheme, rk_2n_t of
 * src/core/rungekutta_mod.F90:29-44. */
typedef struct mglet_rk_scheme {
    int32_t nrk;
    int32_t reserved;
    double cflmax;
    double a[6];
    double b[6];
    double c[6];
} mglet_rk_scheme;

/* Per-stage statistics (the reference samples ipc into itinfo,
 * src/flow/pressuresolver_mod.F90:306-308). */
typedef struct mglet_stage_stats {
    int32_t ipc;          /* inner iterations performed (nouter_done*ninner) */
    int32_t nouter_done;  /* outer defect-correction iterations performed   */
    double maxrhs;        /* last max|rhs| (level scaled), before /prefak   */
    double prefak;        /* rho/dt of the solve                            */
} mglet_stage_stats;

/* itinfo diagnostics (src/flow/timeintegration_mod.F90:145-252,306-452). */
typedef struct mglet_itinfo {
    double cflmax;
    double divmax;
    double energy;        /* enerfg: volume-weighted mean 0.5|u|^2 */
    int32_t exploded;     /* 1 if any of the above is NaN/Inf       */
    int32_t reserved;
} mglet_itinfo;

typedef struct mglet_ctx mglet_ctx;

/* ---- Runge-Kutta coefficients (host only) -------------------------------
 * Replaces rk_2n_t%init (src/core/rungekutta_mod.F90:49-67): name is one of
 * "williamson", "berland", "carpenter", "bernardini". */
int mglet_rk_init(const char* name, mglet_rk_scheme* out);
/* Replaces rk_2n_t%get_coeffs (src/core/rungekutta_mod.F90:240-256). */
int mglet_rk_get_coeffs(const mglet_rk_scheme* rk, int32_t irk, double* frhs,
                        double* fu, double* dtrk, double* dtrki);

/* ---- Context lifetime ---------------------------------------------------
 * Replaces the device-side part of init_core/init_ib/init_flow:
 * init_connect_core (src/core/connect/connect_core_mod.F90:167-370),
 * giteig (src/ib/noib_mod.F90:81-250), init_pressuresolver
 * (src/flow/pressuresolver_mod.F90:47-145: SIP hyperplane/classic LU,
 * SOR_RAP).  Allocates every device field (U,V,W,P,G,DU,DV,DW, BP, SDIV,
 * the pooled scratch UO..RES and the solver coefficients); G is set to
 * gmol and BP to 1 as the reference does for ib type "noib". */
int mglet_gpu_create(const mglet_grid_desc* desc, const mglet_flow_params* prm,
                     int32_t device, mglet_ctx** out);
int mglet_gpu_destroy(mglet_ctx* ctx);

/* Number of elements of a 3-D field (idim3d, pointers_mod.F90:11). */
int64_t mglet_gpu_idim3d(const mglet_ctx* ctx);

/* ---- Host <-> device field transfer --------------------------------------
 * Equivalent of map_arr_to_device / map_arr_from_device
 * (src/core/fieldhelper_mod.F90:97-143).  name is a field name of the
 * reference (U, V, W, P, G, DU, DV, DW, BP, SDIV, UO, VO, WO, DP, HILF,
 * RHS, RES, GSAP, SIPLW, SIPLS, SIPLB, SIPLPR, SIPUE, SIPUN, SIPUT); n must
 * equal idim3d.  Host memory may be pageable or pinned. */
int mglet_gpu_set_field(mglet_ctx* ctx, const char* name, const double* host, int64_t n);
int mglet_gpu_get_field(mglet_ctx* ctx, const char* name, double* host, int64_t n);

/* ---- The RK stage ---------------------------------------------------------
 * Replaces timeintegrate_flow (src/flow/timeintegration_mod.F90:22-142) for
 * ib types "noib" and "ghostcell": tstle4 -> rkstep(u,v,w) -> per level
 * connect(1, normal, forward=1), parent(u,v,w,p), bound_flow -> mgpoisl.
 * stats may be NULL. */
int mglet_gpu_timeintegrate_flow(mglet_ctx* ctx, int32_t itstep, int32_t ittot,
                                 double timeph, double dt, int32_t irk,
                                 const mglet_rk_scheme* rk, mglet_stage_stats* stats);

/* ---- Module-level drop-ins ------------------------------------------------
 * tstle4(uo,vo,wo,u,v,w,u,v,w,p,g) (src/flow/tstle4_mod.F90:13-120):
 * kon, diff, gradp and, on grids with PAR faces, tstle4_par; writes the
 * device fields UO, VO, WO. */
int mglet_gpu_tstle4(mglet_ctx* ctx);
/* rkstep(p, dp, rhsp, frhs, dtfu) over the whole flat arrays
 * (src/core/rungekutta_mod.F90:315-333); arguments are field names. */
int mglet_gpu_rkstep(mglet_ctx* ctx, const char* p, const char* dp, const char* rhsp,
                     double frhs, double dtfu);
/* connect(ilevel, layers, v1..s3, corners, normal, forward)
 * (src/core/connect/connect2_mod.F90:75-139); ilevel <= 0 means all levels;
 * unused field slots are NULL. */
int mglet_gpu_connect(mglet_ctx* ctx, int32_t ilevel, int32_t layers,
                      const char* v1, const char* v2, const char* v3,
                      const char* s1, const char* s2, const char* s3,
                      int32_t corners, int32_t normal, int32_t forward);
/* ib%divcal(div, u, v, w, fak) for noib (src/ib/noib_mod.F90:253-354). */
int mglet_gpu_divcal(mglet_ctx* ctx, const char* div, double fak);
/* laplacephi(res, phi) over all grids (src/flow/laplacephi_mod.F90:14-70). */
int mglet_gpu_laplacephi(mglet_ctx* ctx, const char* res, const char* phi);
/* mgpoisl(u, v, w, p, dt, ittot, irk) (src/flow/pressuresolver_mod.F90:160-357):
 * divergence, outer defect-correction loop, projection (mgpcorr) and the
 * closing connect(2 layers, corners). */
int mglet_gpu_mgpoisl(mglet_ctx* ctx, double dt, int32_t ittot, int32_t irk,
                      mglet_stage_stats* stats);
/* bound_flow%bound(ilevel, u, v, w, p) (src/core/bound_mod.F90:36-76 over
 * src/flow/bound_flow_mod.F90:23-730): FIX, OP1, NOS, SLI and PAR faces of the
 * grids of level ilevel (<= 0: every level), faces 1..6 in order, on the
 * device fields U, V, W, P.  CON/CO1 faces are left to connect; PAR faces
 * take their values from the U, V, W buffers that mglet_gpu_parent fills. */
int mglet_gpu_bound_flow(mglet_ctx* ctx, int32_t ilevel);
/* Boundary buffer of a field on face iface (1..6) of grid igrid (1-based),
 * the plane field_t%get_buffer(buf, igrid, iface) returns
 * (src/core/field_t/realfield_mod.F90:430-503): (kk,jj) for faces 1-2,
 * (kk,ii) for 3-4, (jj,ii) for 5-6, first index fastest; n its size.  FIX
 * faces take their prescribed velocities from it (setboundarybuffers fills
 * it in the reference), OP1 faces their inflow tangential velocities. */
int mglet_gpu_set_buffer(mglet_ctx* ctx, const char* name, int32_t igrid, int32_t iface,
                         const double* host, int64_t n);
/* The real parameter of an OP1 face, the far-field pressure pinf
 * (get_bcprms with nreal = 1, src/flow/bound_flow_mod.F90:226-236); faces
 * without one use pinf = 0. */
int mglet_gpu_set_bc_real(mglet_ctx* ctx, int32_t igrid, int32_t iface, double value);
/* Reads a boundary buffer back (same plane layout as mglet_gpu_set_buffer). */
int mglet_gpu_get_buffer(mglet_ctx* ctx, const char* name, int32_t igrid, int32_t iface,
                         double* host, int64_t n);

/* ---- Grid hierarchies (more than one level, PAR faces) -------------------
 * A context may hold several levels with PAR (code 8) faces (both forms;
 * the mixed form's inner solver is SIP on every level).  These module-level
 * drop-ins then
 * run on it, level by level as the reference calls them; mglet_gpu_tstle4
 * adds tstle4_par on PAR faces (src/flow/tstle4_mod.F90:532-1753), and
 * mglet_gpu_mgpoisl and mglet_gpu_timeintegrate_flow run the multi-level
 * schedule (per level connect, parent and bound_flow before the pressure
 * solve, timeintegration_mod.F90:117-122).  Both need the hierarchy set.
 * With the ghost-cell IB the multi-level schedule of setibvalues (level
 * sweeps, ftoc and par_ftoc_norm between them), setpointvalues and
 * setsdivfield runs too; call mglet_gpu_set_hierarchy before
 * mglet_gpu_set_ghostcell.
 *
 * gridinfo%iparent and i/j/kposition (src/core/grids_mod.F90:768-781):
 * iparent[g] the 1-based parent of grid g+1 (0 = none, one level coarser),
 * position[3g..3g+2] = iposition, jposition, kposition, the parent's
 * 1-based cell index where the fine grid starts.  Required before parent,
 * ftoc and ctof. */
int mglet_gpu_set_hierarchy(mglet_ctx* ctx, const int32_t* iparent, const int32_t* position);
/* parent(ilevel, v1, v2, v3, s1, s2, s3, normal) (src/ib/parent/parent_mod.F90:16,
 * parent1_mod.F90:24-584): for every PAR face of the grids of level ilevel the
 * parent's boundary slab, prolonged onto the fine face (piecewise constant;
 * along a staggered direction the first fine point averages two coarse
 * ones), into the field's boundary buffer.  v1..v3 (all or none) are the
 * velocity components staggered along x, y, z; with normal only the
 * face-normal one; s1..s3 scalars; NULL for absent. */
int mglet_gpu_parent(mglet_ctx* ctx, int32_t ilevel, const char* v1, const char* v2,
                     const char* v3, const char* s1, const char* s2, const char* s3,
                     int32_t normal);
/* ftoc(ilevel, ff, fc, flag) (src/ib/ftoc_mod.F90:39-60,581-626 with the no-IB
 * restriction src/ib/noib_restrict_mod.F90:126-298): the grids of level
 * ilevel restricted into their parents -- face-area means for U, V, W,
 * volume means for P, R, S, T.  With the ghost-cell IB P and R take the
 * BP-weighted forms of src/ib/gc_restrict_mod.F90:59-259 and T is refused
 * (it weighs by the temperature blocking BT, which is not kept).  ff and fc
 * may be the same field. */
int mglet_gpu_ftoc(mglet_ctx* ctx, int32_t ilevel, const char* ff, const char* fc, char flag);
/* ftoc(ilevel, v1, v2, v3, s1, s2, s3) (src/ib/ftoc_mod.F90:64-85): flags U, V,
 * W for v1..v3 and P for the scalars, each field into itself. */
int mglet_gpu_ftoc_multiple(mglet_ctx* ctx, int32_t ilevel, const char* v1, const char* v2,
                            const char* v3, const char* s1, const char* s2, const char* s3);
/* par_ftoc_norm(ilevel, v1, v2, v3, sum) (src/ib/par_ftoc_mod.F90:36-810):
 * on every PAR face of the grids of level ilevel the face-normal component
 * (v1 on x faces, v2 on y, v3 on z), the area mean of 2x2 fine faces (the
 * plain sum when sum is nonzero), is written into the parent -- inside it,
 * or onto its own face when the PAR lies on a coarse face, and then also
 * onto the opposite face of the parent's neighbour across it. */
int mglet_gpu_par_ftoc_norm(mglet_ctx* ctx, int32_t ilevel, const char* v1, const char* v2,
                            const char* v3, int32_t sum);
/* ctof(ilevel, ff, fc) (src/ib/ctof/ctof_mod.F90:16-56, ctof1_mod.F90:167-331):
 * every point of the grids of level ilevel, ghosts included, takes the
 * value of the parent cell it lies in; nothing on the coarsest level. */
int mglet_gpu_ctof(mglet_ctx* ctx, int32_t ilevel, const char* ff, const char* fc);
/* bound_pressure(ilevel, dp, bp) (src/flow/bound_pressure_mod.F90:106-609):
 * the ghost plane of dp on every PAR face of the grids of level ilevel from
 * the field's boundary buffer (mglet_gpu_parent with s1 = dp) corrected by
 * the fine mean next to the face; with_bp selects the BP-weighted form
 * (the reference passes bp for the ghost-cell IB only). */
int mglet_gpu_bound_pressure(mglet_ctx* ctx, int32_t ilevel, const char* dp, int32_t with_bp);
/* The LES model of the stage (lesmodel_mod.F90:34-84, both forms): 0 none,
 * 1 smagorinsky, 2 wale, 5 sigma; cm < 0 takes the model's default
 * constant.  Computes G of the current velocity at once, as
 * init_lesmodel does; the stage then updates G after the pressure solve and
 * tstle4_diff adds its LES cross term.  Model 0 restores G = gmol with the
 * ghost layers of init_lesmodel. */
int mglet_gpu_set_lesmodel(mglet_ctx* ctx, int32_t model, double cm);
/* Passive scalars (src/scalar, plain form, no ghost-cell IB): nsca (0..9)
 * scalars as the device fields T1..Tn with their RK increments DT1..DTn;
 * prmol the molecular Prandtl numbers, kayscrawford the switch of the
 * turbulent Prandtl number fit (scacore_mod.F90:232-262, else prturb),
 * source (may be NULL) a constant source per scalar.  A boundary face
 * without a scalar condition (mglet_gpu_set_scalar_bc) carries no scalar
 * flux. */
int mglet_gpu_set_scalars(mglet_ctx* ctx, int32_t nsca, const double* prmol,
                          const int32_t* kayscrawford, const double* source, double prturb);
/* A scalar boundary condition beside the flow condition of boundary face
 * iface of grid igrid (bound_scalar_mod.F90:124-210 and twins): kind 1 SWA
 * (wall), 2 SIO (inflow/outflow), 0 none; types[l] per scalar: 0 fixed
 * value, 1 fixed flux, the value or flux taken from the scalar's boundary
 * buffer (mglet_gpu_set_buffer with the scalar's name). */
int mglet_gpu_set_scalar_bc(mglet_ctx* ctx, int32_t igrid, int32_t iface, int32_t kind,
                            const int32_t* types);
/* Appends a source to scalar isca (1-based), as an entry of sca%sources
 * (timeintegrate_scalar_mod.F90:549-634): field NULL or "" adds value to
 * the scalar's balance on every interior cell (sourceterm_const), else
 * value times the named cell-centred field (sourceterm_field).  Sources
 * apply in the order added, after a constant source from
 * mglet_gpu_set_scalars; at most 8 per scalar. */
int mglet_gpu_add_scalar_source(mglet_ctx* ctx, int32_t isca, const char* field, double value);
/* Ghost-cell IB of the scalars (plain form).  With the ghost-cell IB
 * (mglet_gpu_set_ghostcell) the scalars' blocking BT comes from BP as
 * blockbt does (blockbt_mod.F90:11-208, also opening the cells behind PAR
 * faces from the coarse BT), and each stage applies maskbt and
 * set_scastencils("P") to QTT (the fixed-flux bodies) and to T (the
 * fixed-value bodies), timeintegrate_scalar_mod.F90:71-90; the ftoc of T
 * weighs by BT.  mglet_gpu_set_scastencils uploads grid igrid's list
 * (gc_scastencils_mod.F90:10-16): per cell 9 integers {intcell, body,
 * nstencils <= 6, six stencil cells; 1-based positions in the grid's flat
 * array} and 8 reals {areabyvol, six coefficients, acoeffvel}, for the 'C'
 * (xpolr) and 'P' (xpolrvel) forms.  mglet_gpu_set_scalar_geometry sets a
 * scalar's condition per body (sca%geometries): flag 0 fixed value, 1 fixed
 * flux, and the value; at most 16 bodies.  A cell without a body counts as
 * fixed flux 0, as in the reference. */
int mglet_gpu_set_scastencils(mglet_ctx* ctx, int32_t igrid, int32_t ncells, const int64_t* xpoli,
                              const double* xpolr, const double* xpolrvel);
int mglet_gpu_set_scalar_geometry(mglet_ctx* ctx, int32_t isca, int32_t nbody, const int32_t* flag,
                                  const double* value);
/* timeintegrate_scalar (src/scalar/timeintegrate_scalar_mod.F90:17-108): one
 * RK stage of every scalar on the current velocity; the reference calls it
 * before timeintegrate_flow in each stage (timeloop_mod.F90:233-235). */
int mglet_gpu_timeintegrate_scalar(mglet_ctx* ctx, double dt, int32_t irk,
                                   const mglet_rk_scheme* rk);
/* The Boussinesq buoyancy term (boussinesqterm_mod.F90): -gravity beta T_old
 * of scalar iscalar (1-based) added to uo, vo, wo after tstle4; T_old is
 * the scalar before its latest mglet_gpu_timeintegrate_scalar. */
int mglet_gpu_set_buoyancy(mglet_ctx* ctx, const double* gravity, double beta, int32_t iscalar);
/* The Coriolis term (coriolisterm_mod.F90): -2 omega x u added to uo, vo, wo
 * after tstle4 (and the buoyancy term). */
int mglet_gpu_set_coriolis(mglet_ctx* ctx, const double* omega);
/* ---- Body force and the discrete adjoint (no counterpart in the reference) --
 * A steady body force per unit mass, added to uo, vo, wo in tstle4 after
 * gradp over the same points (plain form); n must equal idim3d. */
int mglet_gpu_set_body_force(mglet_ctx* ctx, const double* fx, const double* fy, const double* fz,
                             int64_t n);
/* The adjoint of one RK stage of mglet_gpu_timeintegrate_flow (plain form,
 * one level, no IB, every face CON, uniform spacing): the device fields U, V,
 * W hold the stage's input velocity, LU, LV, LW, LP, LDU, LDV, LDW the
 * adjoint of its output state; on return they hold the adjoint of its input
 * state and GFX, GFY, GFZ have gained the stage's dJ/d(body force).  The
 * pressure solve is transposed with the prm's SIP outer loop. */
int mglet_gpu_adjoint_rk_stage(mglet_ctx* ctx, int32_t irk, double dt, const mglet_rk_scheme* rk);
/* The gradient of the kinetic energy (the itinfo energy) after nsteps time
 * steps with respect to the body force: a forward run from the current state
 * keeping a checkpoint every ncheck steps, then each segment recomputed from
 * its checkpoint and run backwards stage by stage.  energy receives J;
 * GFX, GFY, GFZ dJ/df; LU, LV, LW, LP dJ/d of the initial state.  The
 * context ends in the final forward state. */
int mglet_gpu_energy_gradient(mglet_ctx* ctx, int32_t nsteps, int32_t ncheck, double dt,
                              const mglet_rk_scheme* rk, double* energy);
/* ---- Ghost-cell immersed boundary (ib%type = "GHOSTCELL") -------------------
 * Stencil lists of grid igrid (1-based) in the formats of
 * gc_flowstencils_mod.F90:37-100 (what the reference reads from
 * ib_stencils.h5 and create_flowstencils builds): comp 1..3 for u, v, w with
 * xpoli = [intcell, n, stcell x n] per ghost cell (1-based positions in the
 * grid's flat array), xpolr and xpolrvel = [coeff x n, const] per ghost cell
 * (nxrv == nxr); comp 4 for the flux correction with xpoli = [foundnr,
 * intcell] and xpolr = [ax1, ax2, ay1, ay2, az1, az2, acoeff] per cell. */
int mglet_gpu_set_stencils(mglet_ctx* ctx, int32_t igrid, int32_t comp, int32_t ncells,
                           const int64_t* xpoli, int64_t nxi, const double* xpolr, int64_t nxr,
                           const double* xpolrvel, int64_t nxrv);
/* Switch the context to the ghost-cell IB after BP (mglet_gpu_set_field)
 * and every grid's lists are set: Poisson coefficients and SIP factors are
 * rebuilt with the blocked cells (giteig, src/ib/noib_mod.F90:81-250), the
 * lists go to the device and SDIV is built (setsdivfield,
 * gc_flowstencils_mod.F90:1488-1535).  In the mixed form the flux kernel
 * transports the point values PWU, PWV, PWW on the grids where they differ
 * from U, V, W (found at every stage), and grids with blocked cells get
 * SIP classes of their own with the blocked couplings masked; BP must be 0
 * or 1 there (else MGLET_ERR_UNSUPPORTED). */
int mglet_gpu_set_ghostcell(mglet_ctx* ctx);
/* ---- Ghost-cell stencil construction (host only, no device needed) -------
 * Replaces create_flowstencils (src/flow/gc_flowstencils_mod.F90:37-100):
 * from the blocking of every grid it builds the lists mglet_gpu_set_stencils
 * takes -- fluxcorrection (:199-553) for component 4 and fluxstencil /
 * calcflux (:556-752,838-920) for u, v, w.  The geometry arrays are what the
 * reference's blocking leaves in its fields (gc_blockbp_mod.F90:41-271):
 * all idim3d-sized arrays in field_t layout, BP/BU/BV/BW 1 open, 0 blocked,
 * AREAU/AREAV/AREAW the open area of the face at i+1/2 (j+1/2, k+1/2);
 * BZELLTYP negative, -(n), at the n-th intersected cell of its grid (1-based),
 * non-negative elsewhere; icells[g] the intersected cells of grid g+1; per
 * intersected cell, grid after grid, nvecs = the plane a x + b y + c z = dpl
 * of the body surface (unit normal pointing into the fluid) and ucell = the
 * body velocity.  Spacing comes from desc (x, dx give xstag = x + dx/2). */
/* Bodies given as triangles (the reference reads STL, readstl.cxx): a closed,
 * outward-oriented mesh of ntri triangles (9 doubles each) prepared for
 * signed-distance queries (host only): phi[q] of point q, negative inside,
 * and, unless normal is NULL, the unit direction from the closest surface
 * point to the point, pointing out of the body.  The distances feed the
 * blocking from which mglet_create_flowstencils builds the lists. */
int mglet_mesh_create(const double* tri, int64_t ntri, void** mesh);
int mglet_mesh_distance(const void* mesh, const double* pts, int64_t npts, double* phi,
                        double* normal);
int mglet_mesh_free(void* mesh);

typedef struct mglet_ib_geometry {
    const double *bp, *bu, *bv, *bw;
    const double *areau, *areav, *areaw;
    const int32_t* bzelltyp;
    const int32_t* icells;    /* [ngrid] */
    const double* nvecs;      /* [sum icells][4]: a, b, c, dpl */
    const double* ucell;      /* [sum icells][3] */
} mglet_ib_geometry;
typedef struct mglet_flowstencils mglet_flowstencils;
int mglet_create_flowstencils(const mglet_grid_desc* desc, const mglet_ib_geometry* geo,
                              mglet_flowstencils** out);
/* Sizes of the lists of grid igrid (1-based), component comp (1..4): the
 * entry count and the lengths of xpoli and of xpolr (= xpolrvel for 1..3). */
int mglet_flowstencils_size(const mglet_flowstencils* s, int32_t igrid, int32_t comp,
                            int32_t* ncells, int64_t* nxi, int64_t* nxr);
/* Copies them out (xpolrvel NULL for component 4). */
int mglet_flowstencils_copy(const mglet_flowstencils* s, int32_t igrid, int32_t comp,
                            int64_t* xpoli, double* xpolr, double* xpolrvel);
int mglet_flowstencils_free(mglet_flowstencils* s);
/* The scalar ghost-cell lists, create_scastencils (src/scalar/
 * gc_scastencils_mod.F90:21-946), host code: from BP, BZELLTYP and per cut
 * cell (gc_t) its plane, interface area and body id; per grid the records
 * mglet_gpu_set_scastencils takes (9 integers, 8 reals per cell; unused
 * stencil slots -1 and -HUGE as in the reference). */
typedef struct mglet_sca_geometry {
    const double* bp;
    const int32_t* bzelltyp;  /* negative: 1-based index into the grid's cut cells */
    const int32_t* icells;    /* [ngrid] */
    const double* nvecs;      /* [sum icells][4]: a, b, c, dpl */
    const double* arealist;   /* [sum icells] */
    const int32_t* bodyid;    /* [sum icells] */
} mglet_sca_geometry;
typedef struct mglet_scastencils mglet_scastencils;
int mglet_create_scastencils(const mglet_grid_desc* desc, const mglet_sca_geometry* geo,
                             mglet_scastencils** out);
int mglet_scastencils_size(const mglet_scastencils* s, int32_t igrid, int32_t* ncells);
int mglet_scastencils_copy(const mglet_scastencils* s, int32_t igrid, int64_t* xpoli, double* xpolr,
                           double* xpolrvel);
int mglet_scastencils_free(mglet_scastencils* s);
/* setibvalues(u, v, w), getibvalues(u, v, w) and setpointvalues(pwu, pwv,
 * pww, u, v, w, comp_new) (gc_flowstencils_mod.F90:1323-1453), maskbp(u, v,
 * w, p) (src/flow/timeintegration_mod.F90:255-303) on the device fields. */
int mglet_gpu_setibvalues(mglet_ctx* ctx);
int mglet_gpu_getibvalues(mglet_ctx* ctx);
int mglet_gpu_setpointvalues(mglet_ctx* ctx, int32_t comp_new);
int mglet_gpu_maskbp(mglet_ctx* ctx);
/* compcflmax / compdivmax / enerfg of itinfo_flow
 * (src/flow/timeintegration_mod.F90:202-240); out->exploded mirrors the NaN
 * check of itinfo_print (src/flow/itinfo_mod.F90:296-320). */
int mglet_gpu_itinfo(mglet_ctx* ctx, double dt, mglet_itinfo* out);

/* ---- Allocation-free diagnostic ---------------------------------------------
 * No counterpart in the reference: an addition for callers that must not let
 * this library allocate device memory -- builds whose fields already live on
 * the GPU under another runtime (an OpenMP-offload build maps field_t%arr
 * itself and passes device addresses via use_device_ptr), and per-step
 * diagnostics inside the time loop, where cudaMalloc/cudaFree would
 * synchronise the device.
 *
 * max |div u| over the interior of ngrid grids of identical dimensions
 * (kk, jj, ii) in field_t layout, ib type noib -- the divmax of
 * mglet_gpu_itinfo.  u, v, w, the concatenated rddx/rddy/rddz arrays
 * (ngrid*ii, ngrid*jj, ngrid*kk values) and the one-double result divmax
 * are DEVICE pointers; work is queued on stream (a cudaStream_t, NULL for
 * the default stream) and the call returns without synchronising.
 * It allocates nothing: its scratch, one double per grid, is a static
 * __device__ array of MGLET_NOALLOC_MAX_GRIDS doubles (512 KiB) held by every
 * GPU that loads the library.  ngrid > MGLET_NOALLOC_MAX_GRIDS returns
 * MGLET_ERR_SIZE.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  All calls share the one array, so calls
 * that overlap on the GPU (different streams, no ordering) race.
 * Unlike the reference's compdivmax (ABS(div) > divmax skips a NaN) and
 * unlike mglet_gpu_itinfo (which reports MGLET_ERR_EXPLODED), a NaN in the
 * interior divergence propagates: *divmax becomes NaN and the call still
 * returns 0, so a caller detects an exploded field by testing the result
 * for NaN. */
#define MGLET_NOALLOC_MAX_GRIDS 65536
int mglet_gpu_divmax_noalloc(const double* u, const double* v, const double* w, int32_t ngrid,
                             int32_t kk, int32_t jj, int32_t ii, const double* rddx,
                             const double* rddy, const double* rddz, double* divmax,
                             void* stream);

/* ---- Device roofs (no counterpart in the reference) ------------------------
 * The measured FP64 issue rate of device: out[0] DFMA, out[1] DADD, out[2]
 * DMUL thread instructions per second over the whole GPU (one DFMA = two
 * flops), each from independent dependent chains on every SM, timed with
 * CUDA events (best of five).  The second roof of the FP64 parity form. */
int mglet_gpu_fp64_roof(int32_t device, double* out);

/* ---- Grid-partitioned runs (several ranks) ---------------------------------
 * The reference distributes whole grids over MPI ranks (dist_grids,
 * src/core/grids_mod.F90:344-394) and exchanges halos between ranks inside
 * connect (send/recv of connect2_mod.F90:406-548) and the maximum residual
 * with MPI_Allreduce (pressuresolver_mod.F90:295).  Here a rank's context
 * holds the grids it owns plus read-only copies of the remote grids next to
 * them ("halo grids", halo[g] = 1); before every connect the library packs
 * the boxes of its owned grids that other ranks' copies need, hands them to
 * the caller's exchange function, and unpacks what it receives into its own
 * copies, so every owned grid sees the same neighbour values as in a
 * single-rank run.  Maximum reductions (pressure residual, CFL, divergence)
 * skip the copies and are completed across ranks through the same function;
 * the kinetic energy is summed across ranks.  Plain form, one level.
 *
 * send/recv rows are [peer, grid (1-based, of this context), k0, k1, j0, j1,
 * i0, i1] (inclusive 1-based boxes); for every peer both sides list the same
 * boxes in the same order.  The exchange function gets host buffers:
 * op 0 exchanges -- send sendbuf[q] (sendn[q] doubles) to peers[q] and
 * receive recvbuf[q] (recvn[q] doubles) from it, for all q at once; op 1
 * replaces sendbuf[0][0..sendn[0]) by its maximum over all ranks, op 2 by its
 * sum.  It returns 0, or nonzero to fail the calling entry point
 * (MGLET_ERR_CUDA is not used for it: MGLET_ERR_ARG with its message). */
typedef int (*mglet_exchange_fn)(void* user, int32_t op, int32_t npeers, const int32_t* peers,
                                 double* const* sendbuf, const int64_t* sendn,
                                 double* const* recvbuf, const int64_t* recvn);
int mglet_gpu_set_partition(mglet_ctx* ctx, const int32_t* halo, int32_t nsend,
                            const int32_t* send, int32_t nrecv, const int32_t* recv,
                            mglet_exchange_fn fn, void* user);

/* ---- Launch tuning of the mixed form (no counterpart in the reference) -----
 * mglet_gpu_create times the launch variants of the mixed form's pre-pass
 * (points loaded ahead, CTAs per SM, and the uniform-coefficient variant
 * where every coefficient class allows it) on the case itself and keeps the
 * fastest, cached per grid shape for the process; the environment variable
 * MGLET_TUNE=0 keeps the defaults.  The same holds for the packed sweeps
 * (ranks per thread, CTAs per SM), the flux kernel (plane loads or TMA) and
 * the persistent solve of single-level cases (the whole outer loop of
 * mgpoisl as one cooperative launch with grid-wide barriers; timed and
 * reported, run only when forced: the per-phase kernels are faster in the
 * stage graph).  mglet_gpu_tuning describes the
 * choices ("" for the plain form); mglet_gpu_force_variant overrides one
 * (kernel "mx_sip_pre" 0..9, "mx_sip_sweep" 0..4, "mx_flux" 0..1,
 * "mx_sip_solve" 0..5, "mx_outer_pre" 0..1 -- 1: on one level the outer step
 * writes the next hilf-zero pre-pass itself; -1 = default, for
 * "mx_sip_solve" the per-phase kernels).  All variants compute the same
 * bits. */
int mglet_gpu_tuning(mglet_ctx* ctx, char* buf, int64_t buflen);
int mglet_gpu_force_variant(mglet_ctx* ctx, const char* kernel, int32_t variant);
/* Test switch for the failure path of the bounded waits: the next mixed
 * stage's flux kernel (TMA variant) leaves one plane's bulk copy out, so
 * its mbarrier wait gives up after about a second, the kernel raises the
 * control block's error flag and that stage returns MGLET_ERR_CUDA ("timed
 * out waiting for its bulk copies"); the context stays usable and the next
 * stage runs normally.  No fault, trap or hang is involved. */
int mglet_gpu_test_wait_timeout(mglet_ctx* ctx);
/* Test switch for the grid-wide barriers of the persistent solve: in the next
 * mixed stage (issued without its graph) one CTA of the persistent solve
 * leaves before its first arrival, so the other CTAs' barrier wait gives up
 * after about a second; they raise the error flag and return, and the stage
 * returns MGLET_ERR_CUDA ("timed out").  Needs the persistent solve in use
 * (mglet_gpu_force_variant "mx_sip_solve").  The context stays usable. */
int mglet_gpu_test_barrier_timeout(mglet_ctx* ctx);

/* ---- Misc ----------------------------------------------------------------- */
int mglet_gpu_synchronize(mglet_ctx* ctx);
/* The cudaStream_t all of this context's work is issued on (for callers that
 * time or order their own work against it). */
void* mglet_gpu_stream(const mglet_ctx* ctx);
/* Per-kernel device timing: while enabled, every launch is bracketed by CUDA
 * events on the context's stream.  mglet_gpu_profile_get returns the
 * accumulated milliseconds and launch count of one kernel family (name as
 * listed by mglet_gpu_profile_names, comma separated) and resets it. */
int mglet_gpu_profile(mglet_ctx* ctx, int32_t enable);
int mglet_gpu_profile_get(mglet_ctx* ctx, const char* kernel, double* total_ms, int64_t* launches);
int mglet_gpu_profile_names(mglet_ctx* ctx, char* buf, int64_t buflen);
/* Number of kernels this context has launched so far (graph launches count
 * the kernels inside the graph). */
int64_t mglet_gpu_kernel_launches(const mglet_ctx* ctx);
/* Message of the last error in this thread ("" if none). */
const char* mglet_gpu_last_error(void);
int32_t mglet_gpu_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MGLET_GPU_H */
