// mesh_sdf.cu -- signed distance to a closed triangle mesh (host code).
//
// The reference blocks bodies given as STL triangles (readstl.cxx,
// gc_blockbp_mod.F90:41-271: cut edges, node filling, cut cells and their
// normals).  Here a mesh is turned into a signed-distance function, the input
// of the library's blocking and stencil construction: for every query point
// the closest point on the mesh (closest point on a triangle by Voronoi
// regions, Ericson, "Real-Time Collision Detection", 5.1.5), found through a
// uniform grid of bins searched in growing shells, and the sign from the
// angle-weighted pseudo-normal of the closest feature -- face, edge or
// vertex (Baerentzen and Aanaes, IEEE TVCG 11(3), 2005), which is exact for
// closed, consistently oriented meshes.  Outward normals: negative inside.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

#include "internal.h"

namespace mg {
namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 unit(V3 a) {
    const double n = norm(a);
    return n > 0 ? (1.0 / n) * a : V3{0, 0, 0};
}

// closest point on triangle abc to p; region: 0 face, 1..3 vertex a/b/c,
// 4 edge ab, 5 edge bc, 6 edge ca
V3 closest_on_triangle(V3 p, V3 a, V3 b, V3 c, int& region) {
    const V3 ab = b - a, ac = c - a, ap = p - a;
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) { region = 1; return a; }
    const V3 bp = p - b;
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { region = 2; return b; }
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) {
        region = 4;
        return a + (d1 / (d1 - d3)) * ab;
    }
    const V3 cp = p - c;
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) { region = 3; return c; }
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) {
        region = 6;
        return a + (d2 / (d2 - d6)) * ac;
    }
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        region = 5;
        return b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
    }
    region = 0;
    const double den = 1.0 / (va + vb + vc);
    return a + (vb * den) * ab + (vc * den) * ac;
}

struct Mesh {
    std::vector<V3> vtx;                    // welded vertices
    std::vector<std::array<int, 3>> tri;    // vertex ids
    std::vector<V3> fn;                     // face normals (unit)
    std::vector<V3> vn;                     // angle-weighted vertex pseudo-normals
    std::map<std::pair<int, int>, V3> en;   // edge pseudo-normals (sum of the two face normals)
    V3 lo, hi;
    int nb[3];
    double bs[3];
    std::vector<std::vector<int>> bins;
};

void build(Mesh& M, const double* tri, long long ntri) {
    std::map<std::array<double, 3>, int> weld;
    auto vid = [&](const double* p) {
        const std::array<double, 3> key = {p[0], p[1], p[2]};
        auto it = weld.find(key);
        if (it != weld.end()) return it->second;
        const int id = (int)M.vtx.size();
        weld.emplace(key, id);
        M.vtx.push_back({p[0], p[1], p[2]});
        return id;
    };
    for (long long t = 0; t < ntri; ++t)
        M.tri.push_back({vid(tri + 9 * t), vid(tri + 9 * t + 3), vid(tri + 9 * t + 6)});
    M.vn.assign(M.vtx.size(), {0, 0, 0});
    for (const auto& T : M.tri) {
        const V3 a = M.vtx[T[0]], b = M.vtx[T[1]], c = M.vtx[T[2]];
        const V3 n = unit(cross(b - a, c - a));
        M.fn.push_back(n);
        const V3 p[3] = {a, b, c};
        for (int q = 0; q < 3; ++q) {
            const V3 e1 = unit(p[(q + 1) % 3] - p[q]), e2 = unit(p[(q + 2) % 3] - p[q]);
            const double ang = std::acos(std::max(-1.0, std::min(1.0, dot(e1, e2))));
            M.vn[T[q]] = M.vn[T[q]] + ang * n;
            const int u = T[q], v = T[(q + 1) % 3];
            auto key = std::make_pair(std::min(u, v), std::max(u, v));
            M.en[key] = M.en[key] + n;
        }
    }
    M.lo = M.hi = M.vtx[0];
    for (const V3& v : M.vtx) {
        M.lo = {std::min(M.lo.x, v.x), std::min(M.lo.y, v.y), std::min(M.lo.z, v.z)};
        M.hi = {std::max(M.hi.x, v.x), std::max(M.hi.y, v.y), std::max(M.hi.z, v.z)};
    }
    // about two triangles per bin along the longest extent
    const double ext[3] = {M.hi.x - M.lo.x, M.hi.y - M.lo.y, M.hi.z - M.lo.z};
    const double emax = std::max(ext[0], std::max(ext[1], ext[2]));
    const int nmax = std::max(1, std::min(256, (int)std::cbrt((double)M.tri.size() / 2.0) + 1));
    for (int d = 0; d < 3; ++d) {
        M.nb[d] = std::max(1, (int)std::ceil(nmax * ext[d] / emax));
        M.bs[d] = std::max(ext[d] / M.nb[d], emax * 1e-9);
    }
    M.bins.assign((size_t)M.nb[0] * M.nb[1] * M.nb[2], {});
    auto cell = [&](double v, int d, double o) {
        return std::max(0, std::min(M.nb[d] - 1, (int)std::floor((v - o) / M.bs[d])));
    };
    for (int t = 0; t < (int)M.tri.size(); ++t) {
        const V3 a = M.vtx[M.tri[t][0]], b = M.vtx[M.tri[t][1]], c = M.vtx[M.tri[t][2]];
        const int i0 = cell(std::min(a.x, std::min(b.x, c.x)), 0, M.lo.x);
        const int i1 = cell(std::max(a.x, std::max(b.x, c.x)), 0, M.lo.x);
        const int j0 = cell(std::min(a.y, std::min(b.y, c.y)), 1, M.lo.y);
        const int j1 = cell(std::max(a.y, std::max(b.y, c.y)), 1, M.lo.y);
        const int k0 = cell(std::min(a.z, std::min(b.z, c.z)), 2, M.lo.z);
        const int k1 = cell(std::max(a.z, std::max(b.z, c.z)), 2, M.lo.z);
        for (int i = i0; i <= i1; ++i)
            for (int j = j0; j <= j1; ++j)
                for (int k = k0; k <= k1; ++k)
                    M.bins[((size_t)i * M.nb[1] + j) * M.nb[2] + k].push_back(t);
    }
}

// signed distance of p and the pseudo-normal of its closest feature
double query(const Mesh& M, V3 p, V3& nrm) {
    // bin of p, clamped into the grid; shells of bins around it until the
    // best distance is below the distance to the next shell
    int c[3];
    const double pv[3] = {p.x, p.y, p.z}, lv[3] = {M.lo.x, M.lo.y, M.lo.z};
    double outside = 0.0;   // distance from p to the bin grid's box
    for (int d = 0; d < 3; ++d) {
        const double f = (pv[d] - lv[d]) / M.bs[d];
        c[d] = std::max(0, std::min(M.nb[d] - 1, (int)std::floor(f)));
        const double lo = lv[d], hi = lv[d] + M.nb[d] * M.bs[d];
        const double o = std::max(0.0, std::max(lo - pv[d], pv[d] - hi));
        outside += o * o;
    }
    outside = std::sqrt(outside);
    const double bmin = std::min(M.bs[0], std::min(M.bs[1], M.bs[2]));
    const int rmax = std::max(M.nb[0], std::max(M.nb[1], M.nb[2]));
    double best = 1e300;
    int bt = -1, breg = 0;
    V3 bq{0, 0, 0};
    auto visit = [&](int i, int j, int k) {
        for (int t : M.bins[((size_t)i * M.nb[1] + j) * M.nb[2] + k]) {
            int reg;
            const V3 q = closest_on_triangle(p, M.vtx[M.tri[t][0]], M.vtx[M.tri[t][1]],
                                             M.vtx[M.tri[t][2]], reg);
            const double d2 = dot(p - q, p - q);
            if (d2 < best) { best = d2; bt = t; breg = reg; bq = q; }
        }
    };
    for (int r = 0; r <= rmax; ++r) {
        // the bins of the shell at Chebyshev distance r, clamped to the grid
        const int i0 = std::max(0, c[0] - r), i1 = std::min(M.nb[0] - 1, c[0] + r);
        const int j0 = std::max(0, c[1] - r), j1 = std::min(M.nb[1] - 1, c[1] + r);
        for (int i = i0; i <= i1; ++i)
            for (int j = j0; j <= j1; ++j) {
                if (std::abs(i - c[0]) == r || std::abs(j - c[1]) == r) {
                    const int k0 = std::max(0, c[2] - r), k1 = std::min(M.nb[2] - 1, c[2] + r);
                    for (int k = k0; k <= k1; ++k) visit(i, j, k);
                } else {
                    if (c[2] - r >= 0) visit(i, j, c[2] - r);
                    if (r > 0 && c[2] + r < M.nb[2]) visit(i, j, c[2] + r);
                }
            }
        // every unvisited bin is at least r bin sizes, and at least the
        // distance to the bin grid's box, away from p
        if (bt >= 0 && std::sqrt(best) <= std::max(outside, r * bmin)) break;
    }
    const auto& T = M.tri[bt];
    V3 n;
    if (breg == 0) n = M.fn[bt];
    else if (breg <= 3) n = M.vn[T[breg - 1]];
    else {
        const int u = breg == 4 ? T[0] : (breg == 5 ? T[1] : T[2]);
        const int v = breg == 4 ? T[1] : (breg == 5 ? T[2] : T[0]);
        n = M.en.at(std::make_pair(std::min(u, v), std::max(u, v)));
    }
    const V3 dv = p - bq;
    const double dist = std::sqrt(best);
    nrm = dist > 0 ? (1.0 / dist) * dv : unit(n);
    const double s = dot(dv, n) < 0 ? -1.0 : 1.0;
    if (s < 0) nrm = -1.0 * nrm;
    return s * dist;
}

}  // namespace
}  // namespace mg

// A mesh of ntri triangles (9 doubles each, outward orientation) prepared
// for distance queries.
extern "C" int mglet_mesh_create(const double* tri, int64_t ntri, void** out) {
    using namespace mg;
    if (!tri || ntri <= 0 || !out) {
        set_error("mesh_create: needs triangles and an output handle");
        return MGLET_ERR_ARG;
    }
    Mesh* M = new Mesh();
    build(*M, tri, ntri);
    *out = M;
    return 0;
}

// phi[q] the signed distance of point q (negative inside); normal[3q..] the
// unit direction from the closest surface point towards the point, flipped
// inside so that it points out of the body (NULL: not wanted).
extern "C" int mglet_mesh_distance(const void* mesh, const double* pts, int64_t npts, double* phi,
                                   double* normal) {
    using namespace mg;
    if (!mesh || (npts > 0 && (!pts || !phi))) {
        set_error("mesh_distance: needs a mesh, points and an output");
        return MGLET_ERR_ARG;
    }
    const Mesh& M = *static_cast<const Mesh*>(mesh);
    const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int w = 0; w < nth; ++w)
        pool.emplace_back([&, w]() {
            for (int64_t q = w; q < npts; q += nth) {
                V3 n;
                phi[q] = query(M, {pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]}, n);
                if (normal) {
                    normal[3 * q] = n.x;
                    normal[3 * q + 1] = n.y;
                    normal[3 * q + 2] = n.z;
                }
            }
        });
    for (auto& t : pool) t.join();
    return 0;
}

extern "C" int mglet_mesh_free(void* mesh) {
    delete static_cast<mg::Mesh*>(mesh);
    return 0;
}
