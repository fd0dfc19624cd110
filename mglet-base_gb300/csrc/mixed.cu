// mixed.cu -- placeholder until the mixed form lands.
#include "mixed.h"

namespace mg {

int mixed_init(Ctx* c) { (void)c; set_error("mixed form not built yet"); return MGLET_ERR_UNSUPPORTED; }
void mixed_release(Ctx* c) { (void)c; }
void mixed_field_changed(Ctx* c, const char* name) { (void)c; (void)name; }
int mixed_stage(Ctx* c, double dt, int irk, const mglet_rk_scheme* rk, mglet_stage_stats* st) {
    (void)c; (void)dt; (void)irk; (void)rk; (void)st;
    return MGLET_ERR_UNSUPPORTED;
}
int mixed_mgpoisl(Ctx* c, double dt, mglet_stage_stats* st) {
    (void)c; (void)dt; (void)st;
    return MGLET_ERR_UNSUPPORTED;
}

}  // namespace mg
