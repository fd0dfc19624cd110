// mixed.h -- batched mixed-precision form of the stage (MGLET_FORM_MIXED).
#pragma once

#include <string>

#include "internal.h"

namespace mg {

int mixed_init(Ctx* c);
void mixed_release(Ctx* c);
void mixed_field_changed(Ctx* c, const char* name);
void mixed_field_sync_out(Ctx* c, const char* name);
int mixed_stage(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk, mglet_stage_stats* st);
int mixed_mgpoisl(Ctx* c, double dt, mglet_stage_stats* st);
std::string mixed_tuning(Ctx* c);
int mixed_force_variant(Ctx* c, const char* kernel, int v);
int mixed_test_wait_timeout(Ctx* c);
int mixed_test_barrier_timeout(Ctx* c);
// G is a field from now on (LES model or a caller-set G)
void mixed_g_field(Ctx* c);
// the ghost-cell IB (after mglet_gpu_set_ghostcell's plain set-up)
int mixed_ghostcell(Ctx* c);

// shared with api.cu
int connect(Ctx* c, int ilevel, int layers, double* v1, double* v2, double* v3, double* s1,
            double* s2, double* s3, bool corners, bool normal, int forward);
int rk_coeffs(const mglet_rk_scheme* rk, int irk, double* frhs, double* fu, double* dtrk,
              double* dtrki);

}  // namespace mg
