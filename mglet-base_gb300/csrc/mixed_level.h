// mixed_level.h -- grid hierarchies in the batched mixed form (mixed_level.cu).
#pragma once

#include <vector>

#include "mixed_sip.h"

namespace mg {

// Per level (index ilevel - minlevel): its grids and those with a PAR face,
// host and device lists; every grid with a PAR face.  With the ghost-cell IB
// (ibflag set before the set-up) d_skip holds per grid, at every stage,
// whether its transported point values PWU, PWV, PWW differ from U, V, W:
// the flux kernel then transports those point values.
struct LevelState {
    bool ready = false;
    std::vector<std::vector<int>> grids, pars;
    std::vector<int*> d_grids, d_pars;
    std::vector<int> parall;
    int* d_parall = nullptr;
    std::vector<unsigned char> ibflag;
    unsigned char* d_skip = nullptr;
};

// Lists, the PAR ghost planes of hilf and the level operators' buffers; once,
// after the hierarchy is known and before the stage is captured.
int mx_level_prepare(Ctx* c, SipState& st, LevelState& lv);
void mx_level_release(LevelState& lv);
// ctof of hilf into the grids of ilevel (nothing on the coarsest level)
int mx_ctof(Ctx* c, SipState& st, const LevelState& lv, int ilevel, const int* ctl);
// parent + bound_pressure of hilf: the PAR ghost planes of the grids of ilevel
int mx_bound_pressure(Ctx* c, SipState& st, const LevelState& lv, int ilevel, const int* ctl);
// ftoc from the grids of ilevel into their parents: hilf ('P') or the
// float-float residual ('R')
int mx_ftoc(Ctx* c, SipState& st, const LevelState& lv, int ilevel, bool rhs, const int* ctl);
// per-grid max |rhs| into the context's grid reduction array
int mx_gridmax(Ctx* c, SipState& st, const int* ctl);
// the RK update from UO, VO, WO of the grids with a PAR face
int mx_rk_par(Ctx* c, const LevelState& lv, float* du, float* dv, float* dw, const double* sprm);
// ghost-cell IB: d_skip = the grids whose PWU, PWV, PWW differ from U, V, W
int mx_pw_flags(Ctx* c, const LevelState& lv);

}  // namespace mg
