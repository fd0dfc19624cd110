// mixed_sip.h -- hyperplane-layout inner solver of the mixed form.
#pragma once

#include "internal.h"

namespace mg {

struct SipState {
    int kk = 0, jj = 0, ii = 0, ni = 0, nj = 0, nk = 0, npts = 0, fs = 0;
    int nm = 0;                 // hyperplanes per grid
    int npp = 0;                // points per grid with every plane padded to 4 floats
    int maxlp = 0;              // longest padded plane
    int* d_tpos = nullptr;      // [nm][ni] padded plane positions
    int* d_pst = nullptr;       // [nm+1] padded plane starts
    int* d_idxp = nullptr;      // [npp] natural local index, -1 for padding
    int* d_qmap = nullptr;      // [npp] unpadded plane position (iacc-1), -1 for padding
    int* d_pq = nullptr;        // [npp] io | jo << 10 | ko << 20 of each padded position, -1 for padding
    short* d_rowoff = nullptr;  // [nm][ni] rank of (io, jo = 0) in plane m
    int* d_fnbr = nullptr;      // [ngrid][6] face neighbours (0-based)
    float* h32 = nullptr;                                     // [ngrid][npp]
    // res in three rotating slots (inner iteration G writes G % 3): the
    // forward sweep reads its low ghosts from the neighbours' res of the last
    // fully exchanged iteration, the backward sweep its high ghosts from this
    // iteration's
    float* rs[3] = {nullptr, nullptr, nullptr};
    // outer residual and accumulated correction as float-float pairs; the
    // leading float of the residual is the sweeps' FP32 rhs
    float *rhs32 = nullptr, *rhsl = nullptr, *dph = nullptr, *dpl = nullptr;
    int* d_facepos = nullptr;   // [6][fs] padded position of each face point
    int* d_dscf = nullptr;      // [npp][2] forward / backward sweep neighbour positions
    int* d_dscb = nullptr;
    // packed sweeps (shapes whose neighbour positions fit one word): the
    // words, and per class the records {word, three coefficients}
    bool packed = false;
    int* d_wf = nullptr;
    int* d_wb = nullptr;
    float4* swf = nullptr;      // [ncls][npp]
    float4* swb = nullptr;
    // packed pre-pass (npp + 6 fs < 32768): neighbour codes [npp][3] and per
    // class the records [ncls][3][npp]
    bool prepk = false;
    int* d_pcode = nullptr;
    float4* spr = nullptr;
    int order = 0;              // direction of the next per-grid kernel (next_order)
    // every class has constant Laplacian coefficients: [ncls][8] aw, ae, as,
    // an, ab, at, ap for the uniform pre-pass
    bool unicls = false;
    float* uni = nullptr;
    // launch variant of the pre-pass (index into the variant table), picked by
    // the tuner or forced by the caller; -1 = default
    int pre_variant = -1;
    double pre_ms = 0.0;        // its measured time per launch (tuner)
    // launch variant of the packed sweeps (points per thread, CTAs per SM),
    // -1 = default; the tuner's time of one forward + backward pair
    int sweep_variant = -1;
    double sweep_ms = 0.0;
    // hierarchies: the hilf ghost planes of PAR faces [ngrid][6][fs], set by
    // the mixed bound_pressure before every inner iteration of a level
    float* pg = nullptr;
    // ghost-cell IB: per grid and padded position the open couplings (bit f
    // for faces i-1, i+1, j-1, j+1, k-1, k+1), null without the IB
    unsigned char* bm = nullptr;
    // persistent solve (one cooperative launch per mgpoisl): its variant
    // (-1: the per-phase kernels), the tuner's times of one outer iteration
    // in it and in the per-phase kernels, the barrier words [arrivals,
    // abort], and the test switch that makes its first barrier wait run out
    int solve_variant = -1;
    int solve_best = -1;        // the fastest persistent variant the tuner timed
    double solve_ms = 0.0, phases_ms = 0.0;
    double solve_var_ms[6] = {0, 0, 0, 0, 0, 0};   // each variant's time (0: not run)
    unsigned* d_bar = nullptr;
    bool solve_skip = false;
    // one level: the outer step writes the next iteration's pre-pass (its
    // hilf is zero), which then is not launched.  Off by default: on 4096
    // grids of 24^3 it saves 3.2 ms of pre-pass per step and costs the outer
    // step 3.5 ms (the records' lpr and one more array written)
    bool fuse_pre = false;
    // divcal and the scatter of dp in natural order (coalesced FP64 side);
    // false: in plane order
    bool natural = true;
    // outer-step variant (0 staged, 1 / 2 direct at 3 / 4 CTAs per SM; -1
    // default 0) and the tuner's times per launch
    int outer_variant = -1;
    double outer_ms[3] = {0, 0, 0};
    float* a1[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // FP32 GSAW..GSAT
    float* a1lo[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr}; // FP32 of the remainders
};

int sip_init(Ctx* c, SipState& st);
// Class coefficients: FP32 blocks [lw|ls|lb|lpr|ap] and [ue|un|ut] per padded
// plane, and ap split in two floats [hi npp | lo npp], from the representative
// grid of each class.
int sip_extract(Ctx* c, SipState& st, int nclass, const int* d_reps, const int* d_idx,
                bool planeorder, float** cf, float** cb, float** apx);
void sip_release(SipState& st);
// fak (the solve's prefak) is read from device memory
int sip_divcal(Ctx* c, SipState& st, const double* fak);
// glist / nlist: the grids of one level (null: every grid)
// skip_pre: the pre-pass values are in slot rwrite already (the outer step
// wrote them, pre_next of sip_outer)
int sip_forward(Ctx* c, SipState& st, const float* cf, const int* gcls, int* ctl, int rlow,
                int rwrite, bool hzero, const int* glist = nullptr, int nlist = 0,
                bool skip_pre = false);
int sip_backward(Ctx* c, SipState& st, const float* cb, const int* gcls, int* ctl, int rhi,
                 bool hzero, const int* glist = nullptr, int nlist = 0);
// pre_next: where the next inner iteration's pre-pass goes when it starts from
// hilf = 0 on a single level (null: the pre-pass kernel computes it)
int sip_outer(Ctx* c, SipState& st, const float* apx, const int* gcls, const int* ctl,
              float* pre_next = nullptr);
int sip_scatter_dp(Ctx* c, SipState& st);
// The open-coupling masks of every grid from BP (ghost-cell IB)
int sip_bpmask(Ctx* c, SipState& st);
// Times every valid pre-pass variant on the current buffers and keeps the
// fastest (cached per grid shape and class layout for the process).
int sip_tune(Ctx* c, SipState& st, const float* cf, const int* gcls, int* ctl);
// The pre-pass variants: count, and a description of variant v.
int sip_pre_variants();
const char* sip_pre_variant_name(int v);
bool sip_pre_variant_uniform(int v);
int sip_sweep_variants();
const char* sip_sweep_variant_name(int v);
int sip_outer_variants();
const char* sip_outer_variant_name(int v);
// maxabscal over the grids and the outer-loop stopping test (one CTA)
int sip_conv(Ctx* c, int* ctl, double* maxrhs, const double* sprm);
// The persistent solve: every inner iteration, outer step and stopping test
// of one single-level mgpoisl in one cooperative launch, the same bits as the
// per-phase kernels.  fits: variant v can run on this case (one level, the
// packed pre-pass and sweeps, planes of at most 512 points).
int sip_solve_variants();
const char* sip_solve_variant_name(int v);
bool sip_solve_fits(Ctx* c, const SipState& st, int v);
int sip_solve_alloc(SipState& st);
int sip_solve(Ctx* c, SipState& st, const float* cf, const float* apx, const int* gcls, int* ctl,
              double* maxrhs, const double* sprm);
// Times the outer-step variants on the case and keeps the fastest.
int sip_tune_outer(Ctx* c, SipState& st, const float* apx, const int* gcls, int* ctl);
// Times the persistent variants against the per-phase kernels (which the
// tuner must have picked already) and records the times; the persistent
// solve runs only when forced.
int sip_tune_solve(Ctx* c, SipState& st, const float* cf, const float* apx, const int* gcls,
                   int* ctl, double* maxrhs, const double* sprm);

}  // namespace mg
