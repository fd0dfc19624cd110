// mixed_sip.h -- hyperplane-layout inner solver of the mixed form.
#pragma once

#include "internal.h"

namespace mg {

struct SipCoef {   // FP32 class coefficients, plane order [nclass][npts]
    const float *lw, *ls, *lb, *lpr, *ue, *un, *ut, *ap;
};

struct SipState {
    int kk = 0, jj = 0, ii = 0, ni = 0, nj = 0, nk = 0, npts = 0, fs = 0;
    int* d_tpos = nullptr;      // plane position table
    int* d_fnbr = nullptr;      // [ngrid][6] face neighbours (0-based)
    float *h32 = nullptr, *r32 = nullptr, *rhs32 = nullptr;   // plane order
    double *rhs64 = nullptr, *dp64 = nullptr;                 // plane order
    float* hout = nullptr;      // [ngrid][6][fs] hilf boundary planes
    float* rout[3] = {nullptr, nullptr, nullptr};   // rotating res boundary planes
    float* a1[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // FP32 GSAW..GSAT
};

int sip_init(Ctx* c, SipState& st);
void sip_release(SipState& st);
int sip_divcal(Ctx* c, SipState& st, const int* idx, double fak);
int sip_forward(Ctx* c, SipState& st, const SipCoef& cf, const int* gcls, const int* conv,
                int rlow, int rwrite, bool hzero);
int sip_backward(Ctx* c, SipState& st, const SipCoef& cf, const int* gcls, const int* conv,
                 int rhi, bool hzero);
int sip_outer(Ctx* c, SipState& st, const int* idx, const double* ap64, const int* gcls,
              const int* conv);
int sip_scatter_dp(Ctx* c, SipState& st, const int* idx);

}  // namespace mg
