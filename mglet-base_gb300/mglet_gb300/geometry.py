"""Blocking of a body given by its signed-distance function.

The reference blocks bodies given as STL triangles (gc_blockbp_mod.F90:41-271:
cut corners, node filling, face blocking, open face areas, intersected
cells with their normals) and writes the result with the stencils to
ib_stencils.h5.  Here a body is a signed-distance function phi (negative
inside), and the same fields are derived from it per grid, ghost layers
included:

  BP      1 where the cell centre lies in the fluid (phi > 0), else 0, on
          cells no finer grid covers; a cell under a finer grid is open if
          any of its 2x2x2 children is (the restriction ftoc(.., 'E') of
          gc_blockbp_mod.F90:283-301, gc_restrict_mod.F90:290-324); a ghost
          cell that no grid of its level owns (a PAR ghost) takes the value
          of the coarser cell it lies in, as parent(bp) gives it;
  BU      BP(i) * BP(i+1) -- a velocity point is open between two open
          cells (BV, BW alike along j and k);
  AREAU   the open area of the face at xstag(i) (spanning ddy(j) x ddz(k)),
          from s x s midpoint samples of phi where the surface comes within
          half a face diagonal of the face centre, else the whole face or 0;
  BZELLTYP -(n) for the n-th cell (in field order) that the surface passes
          through (phi changes sign over the cell box), 1 elsewhere;
  nvecs   per intersected cell the tangent plane of the body at the surface
          point nearest the cell centre, a x + b y + c z = dpl, with the unit
          normal pointing into the fluid;
  ucell   the body velocity there (a stationary body: 0);
  arealist per intersected cell the area of its tangent plane inside the
          cell box (the interface area the scalar flux condition weighs);
  bodyid  per intersected cell the body's id (`body.body_id`, 1 by default).

These are the inputs of the stencil construction (create_flowstencils,
gc_flowstencils_mod.F90:37-100, and create_scastencils,
gc_scastencils_mod.F90:21-946), built by the library's
mglet_create_flowstencils and mglet_create_scastencils.
"""
import numpy as np


class Sphere:
    """Signed distance to a sphere: |x - c| - r."""

    def __init__(self, center, radius):
        self.c = np.asarray(center, dtype=np.float64)
        self.r = float(radius)

    def phi(self, X, Y, Z):
        return np.sqrt((X - self.c[0]) ** 2 + (Y - self.c[1]) ** 2 + (Z - self.c[2]) ** 2) - self.r

    def plane(self, X, Y, Z):
        """Tangent plane (a, b, c, dpl) at the surface point nearest each
        point, normal pointing out of the sphere (into the fluid)."""
        d = np.stack([X - self.c[0], Y - self.c[1], Z - self.c[2]], axis=-1)
        nrm = np.linalg.norm(d, axis=-1, keepdims=True)
        safe = np.where(nrm > 0, nrm, 1.0)
        nv = np.where(nrm > 0, d / safe, np.array([1.0, 0.0, 0.0]))
        dpl = nv @ self.c + self.r
        return np.concatenate([nv, dpl[..., None]], axis=-1)

    def box_cut(self, lo, hi):
        """True where the surface passes through the box [lo, hi] (arrays
        [..., 3]): nearest distance <= r <= farthest distance."""
        near = np.maximum(np.maximum(lo - self.c, self.c - hi), 0.0)
        far = np.maximum(np.abs(lo - self.c), np.abs(hi - self.c))
        return (np.sqrt((near ** 2).sum(-1)) <= self.r) & (np.sqrt((far ** 2).sum(-1)) >= self.r)

    def reach(self, lo, hi):
        """Distance from the box [lo, hi] (3-vectors) to the surface, 0 if
        the surface passes through it."""
        near = np.sqrt((np.maximum(np.maximum(lo - self.c, self.c - hi), 0.0) ** 2).sum())
        far = np.sqrt((np.maximum(np.abs(lo - self.c), np.abs(hi - self.c)) ** 2).sum())
        if near > self.r:
            return near - self.r
        if far < self.r:
            return self.r - far
        return 0.0


def _open_area(body, xf, yc, zc, hy, hz, axis, samples):
    """Open area of faces normal to `axis` at position xf (along axis),
    centred at (yc, zc) in the two other directions with widths hy, hz; all
    arrays of one shape.  Faces far from the surface are all open or all
    shut; the others are sampled at samples x samples midpoints."""
    def pts(a, b, c):
        # (a along axis, b, c in-plane) -> X, Y, Z
        if axis == 0:
            return a, b, c
        if axis == 1:
            return b, a, c
        return b, c, a

    X, Y, Z = pts(xf, yc, zc)
    ph = body.phi(X, Y, Z)
    full = hy * hz
    area = np.where(ph > 0, full, 0.0)
    near = np.abs(ph) < 0.5 * np.sqrt(hy * hy + hz * hz)
    if np.any(near):
        s = (np.arange(samples) + 0.5) / samples - 0.5
        a0, b0, c0 = xf[near], yc[near], zc[near]
        wy, wz = hy[near], hz[near]
        B = b0[:, None, None] + wy[:, None, None] * s[None, :, None]
        C = c0[:, None, None] + wz[:, None, None] * s[None, None, :]
        A = np.broadcast_to(a0[:, None, None], B.shape + ())
        A = np.broadcast_to(A, np.broadcast_shapes(A.shape, C.shape))
        B = np.broadcast_to(B, A.shape)
        C = np.broadcast_to(C, A.shape)
        Xs, Ys, Zs = pts(A, B, C)
        frac = (body.phi(Xs, Ys, Zs) > 0).mean(axis=(1, 2))
        area[near] = full[near] * frac
    return area


class _Levels:
    """Which grid of a level owns a point: level-L grids tile a lattice of
    boxes of size n * h_L, periodic along the axes without wall faces."""

    def __init__(self, case):
        self.nint = np.array([case.ii - 4, case.jj - 4, case.kk - 4])
        hx = case.dx.reshape(case.ngrid, case.ii)[:, 0]
        hy = case.dy.reshape(case.ngrid, case.jj)[:, 0]
        hz = case.dz.reshape(case.ngrid, case.kk)[:, 0]
        self.levels = sorted(set(int(v) for v in case.level))
        self.h, self.have, self.ntile = {}, {}, {}
        for L in self.levels:
            sel = np.where(case.level == L)[0]
            self.h[L] = np.array([hx[sel[0]], hy[sel[0]], hz[sel[0]]])
            self.have[L] = case.gridpos[sel].astype(np.int64)
        l1 = case.level == self.levels[0]
        self.ntile[self.levels[0]] = case.gridpos[l1].max(axis=0).astype(np.int64) + 1
        for L in self.levels[1:]:
            self.ntile[L] = self.ntile[L - 1] * 2
        bc = case.bctype[l1]
        from .abi import BC_CON
        self.periodic = [bool(np.all(bc[:, 2 * d] == BC_CON) and np.all(bc[:, 2 * d + 1] == BC_CON))
                         for d in range(3)]
        self.keys = {L: np.sort(self._key(self.have[L], L)) for L in self.levels}

    def _key(self, idx, L):
        nt = self.ntile[L]
        return (idx[:, 0] * nt[1] + idx[:, 1]) * nt[2] + idx[:, 2]

    def owned(self, P, L):
        """Points (N, 3) inside the interior of some level-L grid."""
        size = self.h[L] * self.nint
        idx = np.floor(P / size).astype(np.int64)
        nt = self.ntile[L]
        ok = np.ones(len(idx), dtype=bool)
        for d in range(3):
            if self.periodic[d]:
                idx[:, d] %= nt[d]
            else:
                ok &= (idx[:, d] >= 0) & (idx[:, d] < nt[d])
        keys = self.keys[L]
        k = self._key(np.where(ok[:, None], idx, 0), L)
        pos = np.minimum(np.searchsorted(keys, k), len(keys) - 1)
        return ok & (keys[pos] == k)


def _open(levels, body, P, L):
    """BP of the level-L cells centred at P (N, 3): see the module text."""
    out = np.empty(len(P), dtype=bool)
    if len(P) == 0:
        return out
    own = levels.owned(P, L)
    top = levels.levels[0]
    if not own.all():
        q = ~own
        if L > top:
            hc = levels.h[L - 1]
            out[q] = _open(levels, body, (np.floor(P[q] / hc) + 0.5) * hc, L - 1)
        else:
            out[q] = body.phi(P[q, 0], P[q, 1], P[q, 2]) > 0
    if own.any():
        Po = P[own]
        res = np.empty(len(Po), dtype=bool)
        cov = levels.owned(Po, L + 1) if (L + 1) in levels.h else np.zeros(len(Po), dtype=bool)
        if cov.any():
            hf = levels.h[L + 1]
            kids = [Po[cov] + np.array([a, b, c]) * 0.5 * hf
                    for a in (-1, 1) for b in (-1, 1) for c in (-1, 1)]
            res[cov] = np.any([_open(levels, body, kq, L + 1) for kq in kids], axis=0)
        nc = ~cov
        res[nc] = body.phi(Po[nc, 0], Po[nc, 1], Po[nc, 2]) > 0
        out[own] = res
    return out


# the 12 edges of a box as pairs of corner numbers (bit 0: x, 1: y, 2: z)
_EDGES = [(q, q | b) for b in (1, 2, 4) for q in range(8) if not q & b]


def plane_box_area(nv, lo, hi):
    """Area of the plane a x + b y + c z = dpl (rows of nv, unit normal)
    inside each box [lo, hi] (rows of 3): the polygon through the points
    where the plane crosses the box edges, ordered by angle about their
    mean in the plane, summed as triangles (0 where fewer than three)."""
    nv, lo, hi = (np.atleast_2d(np.asarray(a, dtype=np.float64)) for a in (nv, lo, hi))
    nrm, dpl = nv[:, :3], nv[:, 3]
    m = len(nv)
    corners = np.empty((m, 8, 3))
    for q in range(8):
        for ax in range(3):
            corners[:, q, ax] = np.where((q >> ax) & 1, hi[:, ax], lo[:, ax])
    f = np.einsum("nqa,na->nq", corners, nrm) - dpl[:, None]
    pts = np.zeros((m, 12, 3))
    ok = np.zeros((m, 12), dtype=bool)
    for e, (q0, q1) in enumerate(_EDGES):
        f0, f1 = f[:, q0], f[:, q1]
        hit = ((f0 <= 0) & (f1 > 0)) | ((f1 <= 0) & (f0 > 0))
        t = np.where(hit, f0 / np.where(hit, f0 - f1, 1.0), 0.0)
        pts[:, e] = corners[:, q0] + t[:, None] * (corners[:, q1] - corners[:, q0])
        ok[:, e] = hit
    cnt = ok.sum(1)
    cen = (pts * ok[..., None]).sum(1) / np.maximum(cnt, 1)[:, None]
    # an in-plane basis: u orthogonal to the normal, w = n x u
    ref = np.eye(3)[np.argmin(np.abs(nrm), axis=1)]
    u = np.cross(nrm, ref)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = np.cross(nrm, u)
    rel = pts - cen[:, None, :]
    ang = np.arctan2(np.einsum("nea,na->ne", rel, w), np.einsum("nea,na->ne", rel, u))
    order = np.argsort(np.where(ok, ang, np.inf), axis=1)
    rel = np.take_along_axis(rel, order[..., None], axis=1)
    nxt = (np.arange(12)[None, :] + 1) % np.maximum(cnt, 1)[:, None]
    rel2 = np.take_along_axis(rel, nxt[..., None], axis=1)
    tri = np.einsum("nea,na->ne", np.cross(rel, rel2), nrm)
    use = np.arange(12)[None, :] < cnt[:, None]
    area = 0.5 * np.abs((tri * use).sum(1))
    return np.where(cnt >= 3, area, 0.0)


def block(case, body, samples=8):
    """Blocking fields of every grid of `case` for `body`.  Returns a dict
    with flat field_t-layout arrays bp, bu, bv, bw, areau, areav, areaw
    (float64) and bzelltyp (int32), plus icells (int32 [ngrid]), nvecs
    (float64 [sum icells, 4]), ucell (float64 [sum icells, 3]), arealist
    (float64 [sum icells]) and bodyid (int32 [sum icells])."""
    ng, ii, jj, kk = case.ngrid, case.ii, case.jj, case.kk
    npg = ii * jj * kk
    out = {n: np.ones(case.idim3d) for n in ("bp", "bu", "bv", "bw")}
    for n in ("areau", "areav", "areaw"):
        out[n] = np.empty(case.idim3d)
    out["bzelltyp"] = np.ones(case.idim3d, dtype=np.int32)
    icells = np.zeros(ng, dtype=np.int32)
    nvecs, ucell, areas = [], [], []
    levels = _Levels(case)
    X, Y, Z = case.coords()
    DX, DY, DZ = (a.reshape(ng, -1) for a in (case.dx, case.dy, case.dz))
    DDX, DDY, DDZ = (a.reshape(ng, -1) for a in (case.ddx, case.ddy, case.ddz))
    for g in range(ng):
        sl = slice(g * npg, (g + 1) * npg)
        x, y, z = X[g], Y[g], Z[g]
        hx, hy, hz = DDX[g], DDY[g], DDZ[g]
        # (i, j, k) meshes of the grid, C order [i, j, k] = field order
        HX, HY, HZ = np.meshgrid(hx, hy, hz, indexing="ij")
        lo = np.array([x[0] - hx[0], y[0] - hy[0], z[0] - hz[0]])
        hi = np.array([x[-1] + hx[-1], y[-1] + hy[-1], z[-1] + hz[-1]])
        if body.reach(lo, hi) > 0 and body.phi(*[np.array([v]) for v in 0.5 * (lo + hi)])[0] > 0:
            # nowhere near the body and outside it: all open, whole faces
            out["areau"][sl] = (HY * HZ).ravel()
            out["areav"][sl] = (HX * HZ).ravel()
            out["areaw"][sl] = (HX * HY).ravel()
            continue
        # cell centres, one layer beyond the last point for the +1 neighbours
        xe = np.append(x, x[-1] + DX[g][-1])
        ye = np.append(y, y[-1] + DY[g][-1])
        ze = np.append(z, z[-1] + DZ[g][-1])
        XE, YE, ZE = np.meshgrid(xe, ye, ze, indexing="ij")
        pts = np.stack([XE.ravel(), YE.ravel(), ZE.ravel()], axis=1)
        bpe = _open(levels, body, pts, int(case.level[g])).reshape(XE.shape).astype(np.float64)
        bp = bpe[:ii, :jj, :kk]
        out["bp"][sl] = bp.ravel()
        out["bu"][sl] = (bp * bpe[1:, :jj, :kk]).ravel()
        out["bv"][sl] = (bp * bpe[:ii, 1:, :kk]).ravel()
        out["bw"][sl] = (bp * bpe[:ii, :jj, 1:]).ravel()
        XC, YC, ZC = XE[:ii, :jj, :kk], YE[:ii, :jj, :kk], ZE[:ii, :jj, :kk]
        xs = x + 0.5 * DX[g]
        ys = y + 0.5 * DY[g]
        zs = z + 0.5 * DZ[g]
        XS = np.broadcast_to(xs[:, None, None], XC.shape)
        YS = np.broadcast_to(ys[None, :, None], XC.shape)
        ZS = np.broadcast_to(zs[None, None, :], XC.shape)
        out["areau"][sl] = _open_area(body, XS, YC, ZC, HY, HZ, 0, samples).ravel()
        out["areav"][sl] = _open_area(body, YS, XC, ZC, HX, HZ, 1, samples).ravel()
        out["areaw"][sl] = _open_area(body, ZS, XC, YC, HX, HY, 2, samples).ravel()
        lo3 = np.stack([XC - 0.5 * HX, YC - 0.5 * HY, ZC - 0.5 * HZ], axis=-1)
        hi3 = np.stack([XC + 0.5 * HX, YC + 0.5 * HY, ZC + 0.5 * HZ], axis=-1)
        cut = body.box_cut(lo3, hi3).ravel()
        n = int(cut.sum())
        icells[g] = n
        if n:
            bz = np.ones(npg, dtype=np.int32)
            bz[cut] = -np.arange(1, n + 1, dtype=np.int32)
            out["bzelltyp"][sl] = bz
            pl = body.plane(XC.ravel()[cut], YC.ravel()[cut], ZC.ravel()[cut])
            nvecs.append(pl)
            ucell.append(np.zeros((n, 3)))
            areas.append(plane_box_area(pl, lo3.reshape(-1, 3)[cut], hi3.reshape(-1, 3)[cut]))
    out["icells"] = icells
    out["nvecs"] = np.concatenate(nvecs) if nvecs else np.zeros((0, 4))
    out["ucell"] = np.concatenate(ucell) if ucell else np.zeros((0, 3))
    out["arealist"] = np.concatenate(areas) if areas else np.zeros(0)
    out["bodyid"] = np.full(int(icells.sum()), int(getattr(body, "body_id", 1)), dtype=np.int32)
    return out


# ---------------------------------------------------------------------------
# Bodies given as triangles (STL), the reference's geometry input
# (src/core/readstl.cxx): the library turns the mesh into signed distances
# (mglet_mesh_create / mglet_mesh_distance), and the blocking above runs on
# them unchanged.

def read_stl(path):
    """Triangles (ntri, 3, 3) of an ASCII or binary STL file."""
    raw = open(path, "rb").read()
    if len(raw) >= 84:
        n = int(np.frombuffer(raw[80:84], dtype="<u4")[0])
        if len(raw) == 84 + 50 * n:
            rec = np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")])
            return np.frombuffer(raw[84:], dtype=rec, count=n)["v"].astype(np.float64)
    verts = []
    for line in raw.decode("ascii", errors="replace").splitlines():
        parts = line.split()
        if parts and parts[0] == "vertex":
            verts.append([float(v) for v in parts[1:4]])
    a = np.array(verts, dtype=np.float64)
    if len(a) % 3:
        raise ValueError(f"{path}: vertex count {len(a)} is not a multiple of three")
    return a.reshape(-1, 3, 3)


def write_stl(path, tris, binary=True):
    """Writes triangles (ntri, 3, 3) as STL (facet normals from the vertex order)."""
    tris = np.asarray(tris, dtype=np.float64)
    nrm = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-300)
    if binary:
        rec = np.zeros(len(tris), dtype=[("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")])
        rec["n"] = nrm
        rec["v"] = tris
        with open(path, "wb") as f:
            f.write(b"binary STL".ljust(80, b" "))
            f.write(np.array([len(tris)], dtype="<u4").tobytes())
            f.write(rec.tobytes())
        return
    with open(path, "w") as f:
        f.write("solid body\n")
        for t, n in zip(tris, nrm):
            f.write(f" facet normal {n[0]:.17g} {n[1]:.17g} {n[2]:.17g}\n  outer loop\n")
            for v in t:
                f.write(f"   vertex {v[0]:.17g} {v[1]:.17g} {v[2]:.17g}\n")
            f.write("  endloop\n endfacet\n")
        f.write("endsolid body\n")


def icosphere(center, radius, level=3):
    """A closed, outward-oriented triangle mesh of a sphere: the icosahedron
    subdivided `level` times, vertices pushed onto the sphere."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    for _ in range(level):
        mid = {}

        def m(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                p = verts[a] + verts[b]
                verts.append(p / np.linalg.norm(p))
                mid[key] = len(verts) - 1
            return mid[key]

        f = [tri for (a, b, c) in f
             for tri in ((a, m(a, b), m(c, a)), (b, m(b, c), m(a, b)), (c, m(c, a), m(b, c)),
                         (m(a, b), m(b, c), m(c, a)))]
    V = np.array(verts) * radius + np.asarray(center, dtype=np.float64)
    return V[np.array(f)]


class Mesh:
    """A body given by a closed, outward-oriented triangle mesh, with the
    interface of Sphere (phi, plane, box_cut, reach) for block()."""

    def __init__(self, tris):
        import ctypes as C
        from . import gpu
        self._lib = gpu.load()
        self.tris = np.ascontiguousarray(np.asarray(tris, dtype=np.float64).reshape(-1, 9))
        self._h = C.c_void_p()
        gpu._check(self._lib.mglet_mesh_create(self.tris.ctypes.data, len(self.tris),
                                                C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.mglet_mesh_free(self._h)
            self._h = None

    def _query(self, X, Y, Z, want_normal):
        from . import gpu
        X, Y, Z = np.broadcast_arrays(X, Y, Z)
        pts = np.ascontiguousarray(np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1))
        phi = np.empty(len(pts))
        nrm = np.empty((len(pts), 3)) if want_normal else None
        gpu._check(self._lib.mglet_mesh_distance(self._h, pts.ctypes.data, len(pts),
                                                 phi.ctypes.data,
                                                 nrm.ctypes.data if want_normal else None))
        return phi.reshape(X.shape), (nrm.reshape(X.shape + (3,)) if want_normal else None)

    def phi(self, X, Y, Z):
        return self._query(X, Y, Z, False)[0]

    def plane(self, X, Y, Z):
        phi, n = self._query(X, Y, Z, True)
        P = np.stack(np.broadcast_arrays(X, Y, Z), axis=-1)
        q = P - phi[..., None] * n
        return np.concatenate([n, np.sum(n * q, axis=-1, keepdims=True)], axis=-1)

    def box_cut(self, lo, hi):
        c = 0.5 * (lo + hi)
        half = 0.5 * np.linalg.norm(hi - lo, axis=-1)
        return np.abs(self.phi(c[..., 0], c[..., 1], c[..., 2])) <= half

    def reach(self, lo, hi):
        c = 0.5 * (lo + hi)
        half = 0.5 * float(np.linalg.norm(hi - lo))
        d = abs(float(self.phi(np.array([c[0]]), np.array([c[1]]), np.array([c[2]]))[0]))
        return max(0.0, d - half)
