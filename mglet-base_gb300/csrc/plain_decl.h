// plain_decl.h -- the kernels of plain_flux.cu and plain_poisson.cu, declared
// once in namespace mg (the parity build, no multiply-add contraction) and
// once in mg::contract (the performance build); included by internal.h inside
// each namespace, so it has no include guard.
//
// u, v, w: the transported velocities (point values PWU.. with the ghost-cell
// IB), ut, vt, wt: the transporting ones (tstle4_mod.F90:13, 139)
int launch_tstle4(Ctx* c, double* uo, double* vo, double* wo, const double* u, const double* v,
                  const double* w, const double* ut, const double* vt, const double* wt,
                  const double* p, const double* g);
int launch_rkstep(Ctx* c, double* p, double* dp, const double* rhs, double frhs, double dtfu);
int launch_g_uniform(Ctx* c);   // d_guni: per grid, is G one value on the box 2..n-1
int launch_divcal(Ctx* c, double* div, const double* u, const double* v, const double* w,
                  double fak);
int launch_bp_ones(Ctx* c);
int launch_laplacephi(Ctx* c, int ilevel, double* res, const double* phi);
int launch_sip_lu_hp(Ctx* c);
int launch_sip_lu_classic(Ctx* c);
int launch_sipiter1(Ctx* c, int ilevel, const double* rhs, double* res);
int launch_sipiter2(Ctx* c, int ilevel, double* phi, double* res);
int launch_sor(Ctx* c, int ilevel, double* dp, const double* rhs);
int launch_giteig(Ctx* c);
int launch_rescal_maxabs(Ctx* c, double* rhs, const double* res);
int launch_accumulate(Ctx* c, double* dp, double* hilf);
int launch_mgpcorr(Ctx* c, double* u, double* v, double* w, double* p, const double* dp,
                   double rfak);
void release_tables(Ctx* c);
