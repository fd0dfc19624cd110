// plain_bound.cu -- bound_flow for FIX, OP1, NOS and SLI faces, FP64 (PAR
// faces: plain_level.cu).
//
// bound_flow_mod.F90 bfront (:23-256), bright (:259-494) and bbottom
// (:497-730), dispatched as bound_t%bound does (src/core/bound_mod.F90:36-76):
// grid by grid, faces 1..6 in order.  Faces of one grid overlap on their
// edges and corners, so the faces run as separate launches in that order
// over all grids that have a boundary there; within a face every position is
// independent.  The pressure of a face depends on the tangential velocities
// the same face has just written, so it is a second launch.  Compiled
// without FMA contraction: every value matches the CPU restatement bit for
// bit.
#include <algorithm>
#include <vector>

#include "internal.h"

namespace mg {
namespace {

__device__ __forceinline__ double fsign(double a, double b) { return copysign(fabs(a), b); }

// Face geometry: normal axis, ghost/interior planes, staggered planes and
// the tangential extents; a runs fastest in the reference's loops.
struct Face {
    int axis, n2, n3, st1, st2, na, nb, kk, jj;
    double dir;
    __device__ long long at(int a, int b, int n) const {
        int k, j, i;
        if (axis == 0) { k = a; j = b; i = n; }
        else if (axis == 1) { k = a; j = n; i = b; }
        else { k = n; j = a; i = b; }
        return (long long)(i - 1) * kk * jj + (long long)(j - 1) * kk + (k - 1);
    }
};

__device__ Face make_face(const DevGrid& G, int iface) {
    Face f;
    f.axis = (iface - 1) / 2;
    const bool lo = (iface % 2) == 1;
    const int nn = f.axis == 0 ? G.ii : (f.axis == 1 ? G.jj : G.kk);
    f.n2 = lo ? 2 : nn - 1;
    f.n3 = lo ? 3 : nn - 2;
    f.st1 = lo ? 1 : nn - 1;
    f.st2 = lo ? 2 : nn - 2;
    f.dir = lo ? -1.0 : 1.0;
    f.na = f.axis == 2 ? G.jj : G.kk;
    f.nb = f.axis == 0 ? G.jj : G.ii;
    f.kk = G.kk;
    f.jj = G.jj;
    return f;
}

struct BoundArgs {
    const DevGrid* grids;
    const int* list;            // grids with a FIX/OP1/NOS/SLI face iface
    const BFace* bface;
    const double *ub, *vb, *wb;
    double *u, *v, *w, *p;
    int iface;
    int ilevel;                 // 0: all levels
    double rho;
};

// Velocities of one face.  Normal component vn, tangential t1 (staggered
// along b) and t2 (staggered along a): x faces (u | v, w), y faces
// (v | u, w), z faces (w | u, v).  Writes follow the reference's order.
__global__ void k_bound_vel(BoundArgs a) {
    const int g = a.list[blockIdx.y];
    const DevGrid G = a.grids[g];
    if (a.ilevel && G.level != a.ilevel) return;
    const int typ = G.bc[a.iface - 1];
    const Face f = make_face(G, a.iface);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= f.na * f.nb) return;
    const int ia = q % f.na + 1, ib = q / f.na + 1;
    const BFace bf = a.bface[6 * g + a.iface - 1];
    const long long o = G.ip3;
    double* vn = (f.axis == 0 ? a.u : (f.axis == 1 ? a.v : a.w)) + o;
    double* t1 = (f.axis == 0 ? a.v : a.u) + o;
    double* t2 = (f.axis == 2 ? a.v : a.w) + o;
    const double* bn = (f.axis == 0 ? a.ub : (f.axis == 1 ? a.vb : a.wb)) + bf.off;
    const double* b1 = (f.axis == 0 ? a.vb : a.ub) + bf.off;
    const double* b2 = (f.axis == 2 ? a.vb : a.wb) + bf.off;
    const long long bi = (long long)(ia - 1) + (long long)(ib - 1) * f.na;
    if (typ == MGLET_BC_FIX) {
        const double vnb = bn[bi];
        const double n1v = 2.0 * b1[bi] - t1[f.at(ia, ib, f.n3)];
        const double n2v = 2.0 * b2[bi] - t2[f.at(ia, ib, f.n3)];
        vn[f.at(ia, ib, f.st2)] = vnb;
        t1[f.at(ia, ib, f.n2)] = n1v;
        t2[f.at(ia, ib, f.n2)] = n2v;
    } else if (typ == MGLET_BC_OP1) {
        if (ia > f.na - 1 || ib > f.nb - 1) return;
        const double c0 = vn[f.at(ia, ib, f.st2)];
        double f1 = fsign(1.0, f.dir * (c0 + vn[f.at(ia, ib + 1, f.st2)]));
        double f2 = fsign(1.0, f.dir * (c0 + vn[f.at(ia + 1, ib, f.st2)]));
        f1 = 0.5 * (f1 + 1.0);
        f2 = 0.5 * (f2 + 1.0);
        const double t1i = t1[f.at(ia, ib, f.n3)], t2i = t2[f.at(ia, ib, f.n3)];
        const double n1v = f1 * t1i + (1.0 - f1) * (2.0 * b1[bi] - t1i);
        const double n2v = f2 * t2i + (1.0 - f2) * (2.0 * b2[bi] - t2i);
        vn[f.at(ia, ib, f.st1)] = c0;
        t1[f.at(ia, ib, f.n2)] = n1v;
        t2[f.at(ia, ib, f.n2)] = n2v;
    } else if (typ == MGLET_BC_NOS) {
        vn[f.at(ia, ib, f.st2)] = 0.0;
        t1[f.at(ia, ib, f.n2)] = 0.0;
        t2[f.at(ia, ib, f.n2)] = 0.0;
    } else if (typ == MGLET_BC_SLI) {
        vn[f.at(ia, ib, f.st2)] = 0.0;
        t1[f.at(ia, ib, f.n2)] = t1[f.at(ia, ib, f.n3)];
        t2[f.at(ia, ib, f.n2)] = t2[f.at(ia, ib, f.n3)];
    }
}

// Pressure of one face: OP1 far-field pressure minus the dynamic pressure of
// inflow, zero gradient on FIX, NOS and SLI.
__global__ void k_bound_p(BoundArgs a) {
    const int g = a.list[blockIdx.y];
    const DevGrid G = a.grids[g];
    if (a.ilevel && G.level != a.ilevel) return;
    const int typ = G.bc[a.iface - 1];
    const Face f = make_face(G, a.iface);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= f.na * f.nb) return;
    const int ia = q % f.na + 1, ib = q / f.na + 1;
    const long long o = G.ip3;
    double* p = a.p + o;
    if (typ == MGLET_BC_OP1) {
        if (ia < 2 || ib < 2) return;
        const double* vn = (f.axis == 0 ? a.u : (f.axis == 1 ? a.v : a.w)) + o;
        const double* t1 = (f.axis == 0 ? a.v : a.u) + o;
        const double* t2 = (f.axis == 2 ? a.v : a.w) + o;
        const double c1 = 0.25 * (t1[f.at(ia, ib - 1, f.n2)] + t1[f.at(ia, ib, f.n2)] +
                                  t1[f.at(ia, ib - 1, f.n3)] + t1[f.at(ia, ib, f.n3)]);
        const double c2 = 0.25 * (t2[f.at(ia - 1, ib, f.n2)] + t2[f.at(ia, ib, f.n2)] +
                                  t2[f.at(ia - 1, ib, f.n3)] + t2[f.at(ia, ib, f.n3)]);
        const double un = vn[f.at(ia, ib, f.st2)];
        double umagsqr;
        if (f.axis == 0) umagsqr = un * un + c1 * c1 + c2 * c2;
        else if (f.axis == 1) umagsqr = c1 * c1 + un * un + c2 * c2;
        else umagsqr = c1 * c1 + c2 * c2 + un * un;
        const double pin = a.bface[6 * g + a.iface - 1].pinf;
        p[f.at(ia, ib, f.n2)] = pin + fmin(0.0, 0.5 * a.rho * fsign(umagsqr, f.dir * un));
    } else {
        p[f.at(ia, ib, f.n2)] = p[f.at(ia, ib, f.n3)];
    }
}

}  // namespace

int bound_init(Ctx* c) {
    c->bface.assign(6 * (size_t)c->ngrid, BFace{0, 0.0});
    long long nb = 0;
    for (int g = 0; g < c->ngrid; ++g) {
        const DevGrid& G = c->grids[g];
        const long long sz[3] = {(long long)G.kk * G.jj, (long long)G.kk * G.ii,
                                 (long long)G.jj * G.ii};
        for (int f = 0; f < 6; ++f) {
            c->bface[6 * g + f].off = nb;
            nb += sz[f / 2];
            const int t = G.bc[f];
            if (t == MGLET_BC_FIX || t == MGLET_BC_OP1 || t == MGLET_BC_NOS || t == MGLET_BC_SLI)
                c->bgrids[f].push_back(g);
        }
    }
    c->nbuf = nb;
    for (int q = 0; q < 3; ++q) {
        MG_CUDA(cudaMalloc(&c->d_buf[q], (size_t)nb * sizeof(double)));
        MG_CUDA(zero_on(c->stream, c->d_buf[q], (size_t)nb * sizeof(double)));
    }
    MG_CUDA(cudaMalloc(&c->d_bface, c->bface.size() * sizeof(BFace)));
    MG_CUDA(copy_on(c->stream, c->d_bface, c->bface.data(), c->bface.size() * sizeof(BFace),
                    cudaMemcpyHostToDevice));
    for (int f = 0; f < 6; ++f) {
        if (c->bgrids[f].empty()) continue;
        MG_CUDA(cudaMalloc(&c->d_bgrids[f], c->bgrids[f].size() * sizeof(int)));
        MG_CUDA(copy_on(c->stream, c->d_bgrids[f], c->bgrids[f].data(),
                        c->bgrids[f].size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    return 0;
}

int launch_bound_flow(Ctx* c, double* u, double* v, double* w, double* p, int ilevel) {
    ProfScope ps_(c, "bound_flow");
    for (int f = 0; f < 6; ++f) {
        // PAR faces (plain_level.cu): no pressure, other grids than this
        // face's FIX/OP1/NOS/SLI ones, so the order within a face is free
        if (int rc = launch_bound_par(c, f + 1, ilevel, u, v, w)) return rc;
        if (c->bgrids[f].empty()) continue;
        int maxq = 0;
        for (int g : c->bgrids[f]) {
            const DevGrid& G = c->grids[g];
            const int na = f / 2 == 2 ? G.jj : G.kk, nb = f / 2 == 0 ? G.jj : G.ii;
            maxq = std::max(maxq, na * nb);
        }
        BoundArgs a{};
        a.grids = c->d_grids;
        a.list = c->d_bgrids[f];
        a.bface = c->d_bface;
        a.ub = c->d_buf[0]; a.vb = c->d_buf[1]; a.wb = c->d_buf[2];
        a.u = u; a.v = v; a.w = w; a.p = p;
        a.iface = f + 1;
        a.ilevel = ilevel;
        a.rho = c->prm.rho;
        const dim3 grid((maxq + 127) / 128, (unsigned)c->bgrids[f].size());
        k_bound_vel<<<grid, 128, 0, c->stream>>>(a);
        MG_LAUNCHED(c);
        if (p) {
            k_bound_p<<<grid, 128, 0, c->stream>>>(a);
            MG_LAUNCHED(c);
        }
    }
    return 0;
}

}  // namespace mg
