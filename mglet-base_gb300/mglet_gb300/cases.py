"""Host-side case generation: grid tables, spacing arrays, initial fields.

This plays the role of the reference's grid preprocessor (grids.h5 with
GRIDINFO, NBRGRID and the BC tables, src/core/gridio_mod.F90:12-46) for the
uniform periodic tilings the hot path is measured on, and of init_uvwp
(src/flow/flow_mod.F90:123-172) for the closed-form initial fields.

Conventions: faces 1..6 = front(-x), back(+x), right(-y), left(+y),
bottom(-z), top(+z); neighbour slots 7..26 follow facelist of
src/core/connect/connect_core_mod.F90:38-64.  Field arrays are flat FP64,
grid after grid, each grid Fortran-ordered (k fastest) with two ghost
layers (src/core/pointers_mod.F90:23-75).
"""
import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from .abi import BC_CON, GridDesc

# Elementary directions of the 26 neighbour slots (facelist of
# connect_core_mod.F90:38-64): each slot is a combination of faces.
_FACE_DIR = {1: (-1, 0, 0), 2: (1, 0, 0), 3: (0, -1, 0), 4: (0, 1, 0), 5: (0, 0, -1), 6: (0, 0, 1)}
FACELIST = [
    (1,), (2,), (3,), (4,), (5,), (6,),
    (1, 3), (1, 4), (1, 5), (1, 6), (2, 3), (2, 4), (2, 5), (2, 6), (3, 5), (3, 6), (4, 5), (4, 6),
    (1, 3, 5), (1, 3, 6), (1, 4, 5), (1, 4, 6), (2, 3, 5), (2, 3, 6), (2, 4, 5), (2, 4, 6),
]


def slot_offset(slot):
    """(di, dj, dk) of neighbour slot 1..26."""
    d = [0, 0, 0]
    for f in FACELIST[slot - 1]:
        for q in range(3):
            d[q] += _FACE_DIR[f][q]
    return tuple(d)


@dataclass
class Case:
    """A single-level grid hierarchy plus its flat-array geometry."""
    ngrid: int
    kk: int
    jj: int
    ii: int
    mgdims: np.ndarray        # int32 [ngrid, 3] (kk, jj, ii)
    level: np.ndarray         # int32 [ngrid]
    bctype: np.ndarray        # int32 [ngrid, 6]
    nbrgrid: np.ndarray       # int32 [ngrid, 26]
    gridpos: np.ndarray       # int32 [ngrid, 3] (gx, gy, gz)
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    dx: np.ndarray
    dy: np.ndarray
    dz: np.ndarray
    ddx: np.ndarray
    ddy: np.ndarray
    ddz: np.ndarray
    # grid hierarchy: 1-based parent per grid (0 = none) and the parent cell
    # (iposition, jposition, kposition) where a fine grid starts
    iparent: np.ndarray = None
    position: np.ndarray = None
    _keep: list = field(default_factory=list, repr=False)

    @property
    def idim3d(self):
        return self.ngrid * self.kk * self.jj * self.ii

    @property
    def n_interior(self):
        """Interior cells per grid along i (the grids of a case share it)."""
        return self.ii - 4

    @property
    def ncells(self):
        """Interior cells (the TPC denominator of timeloop_mod.F90:149)."""
        return self.ngrid * (self.kk - 4) * (self.jj - 4) * (self.ii - 4)

    def desc(self):
        """A GridDesc whose pointers stay valid as long as this Case lives."""
        d = GridDesc()
        d.ngrid = self.ngrid
        arrs = {}
        for name in ("mgdims", "level", "bctype", "nbrgrid"):
            a = np.ascontiguousarray(getattr(self, name), dtype=np.int32)
            arrs[name] = a
            setattr(d, name, a.ctypes.data_as(C.POINTER(C.c_int32)))
        d.gradpflag = C.POINTER(C.c_int32)()
        for name in ("x", "y", "z", "dx", "dy", "dz", "ddx", "ddy", "ddz"):
            a = np.ascontiguousarray(getattr(self, name), dtype=np.float64)
            arrs[name] = a
            setattr(d, name, a.ctypes.data_as(C.POINTER(C.c_double)))
        self._keep.append(arrs)
        return d

    # -- field helpers ------------------------------------------------------
    def zeros(self):
        return np.zeros(self.idim3d, dtype=np.float64)

    def view(self, flat):
        """[ngrid, ii, jj, kk] view of a flat field (C order of the Fortran slab)."""
        return flat.reshape(self.ngrid, self.ii, self.jj, self.kk)

    def interior(self, flat):
        v = self.view(flat)
        return v[:, 2:self.ii - 2, 2:self.jj - 2, 2:self.kk - 2]

    def coords(self):
        """Per-grid 1-D coordinate arrays as [ngrid, n] views."""
        return (self.x.reshape(self.ngrid, self.ii), self.y.reshape(self.ngrid, self.jj),
                self.z.reshape(self.ngrid, self.kk))


def periodic_box(nx, ny, nz, n=24, length=(2 * np.pi, 2 * np.pi, 2 * np.pi), nk=None, nj=None,
                 walls=None):
    """nx*ny*nz grids of n^3 interior cells tiling a box, periodic unless
    told otherwise.

    Every face is CON (code 7) and every one of the 26 neighbour slots
    points at the periodic image grid, as a grids.h5 for a fully periodic
    one-level domain holds.  `walls` maps box faces 1..6 to a boundary
    code (FIX, OP1, NOS, SLI): the grids on that side of the box get it on
    that face, and a direction with a boundary face is not periodic, so
    neighbour slots that would cross it are 0.  Grid ids run x fastest.
    """
    walls = dict(walls or {})
    ni = n
    nj = n if nj is None else nj
    nk = n if nk is None else nk
    ii, jj, kk = ni + 4, nj + 4, nk + 4
    ngrid = nx * ny * nz
    gx, gy, gz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    gx = gx.transpose(2, 1, 0).ravel()
    gy = gy.transpose(2, 1, 0).ravel()
    gz = gz.transpose(2, 1, 0).ravel()
    gid = lambda a, b, c: 1 + (a % nx) + nx * ((b % ny) + ny * (c % nz))
    periodic = [not (2 * d + 1 in walls or 2 * d + 2 in walls) for d in range(3)]
    nbr = np.zeros((ngrid, 26), dtype=np.int32)
    for s in range(1, 27):
        di, dj, dk = slot_offset(s)
        ok = np.ones(ngrid, dtype=bool)
        for d, (g, dd, nn) in enumerate(((gx, di, nx), (gy, dj, ny), (gz, dk, nz))):
            if not periodic[d]:
                ok &= (g + dd >= 0) & (g + dd < nn)
        nbr[:, s - 1] = np.where(ok, gid(gx + di, gy + dj, gz + dk), 0)
    bctype = np.full((ngrid, 6), BC_CON, dtype=np.int32)
    for f, code in walls.items():
        d, hi = (f - 1) // 2, (f - 1) % 2
        g, nn = ((gx, nx), (gy, ny), (gz, nz))[d]
        bctype[g == (nn - 1 if hi else 0), f - 1] = code
    hx, hy, hz = length[0] / (nx * ni), length[1] / (ny * nj), length[2] / (nz * nk)

    def axis(g0, h, npts):
        # cell i (1-based) spans [g0 + (i-3) h, g0 + (i-2) h]; x(i) its centre
        i = np.arange(1, npts + 1, dtype=np.float64)
        return g0[:, None] + (i[None, :] - 2.5) * h

    x = axis(gx * ni * hx, hx, ii).ravel()
    y = axis(gy * nj * hy, hy, jj).ravel()
    z = axis(gz * nk * hz, hz, kk).ravel()
    return Case(
        ngrid=ngrid, kk=kk, jj=jj, ii=ii,
        mgdims=np.tile(np.array([kk, jj, ii], dtype=np.int32), (ngrid, 1)),
        level=np.ones(ngrid, dtype=np.int32),
        bctype=bctype,
        nbrgrid=nbr,
        gridpos=np.stack([gx, gy, gz], axis=1).astype(np.int32),
        x=x, y=y, z=z,
        dx=np.full(ngrid * ii, hx), dy=np.full(ngrid * jj, hy), dz=np.full(ngrid * kk, hz),
        ddx=np.full(ngrid * ii, hx), ddy=np.full(ngrid * jj, hy), ddz=np.full(ngrid * kk, hz),
    )


def refined_box(nx, ny, nz, n=8, refine=(1,), length=(2 * np.pi, 2 * np.pi, 2 * np.pi),
                octants=None):
    """A two-level hierarchy: the periodic tiling of periodic_box (level 1)
    with every coarse grid listed in `refine` (1-based, not adjacent to each
    other) covered by 2x2x2 grids of n^3 cells at half its spacing (level 2),
    or by the subset `octants` of them ((ox, oy, oz) in {0, 1}^3).  A fine
    face towards a sibling is CON, every other fine face PAR (code 8) with
    the coarse grid as parent, as a grids.h5 of a locally refined domain
    holds (src/core/gridio_mod.F90:61-245).  n must be even."""
    from .abi import BC_PAR
    assert n % 2 == 0
    c = periodic_box(nx, ny, nz, n=n, length=length)
    nc = c.ngrid
    ii = jj = kk = n + 4
    octs = [(ox, oy, oz) for oz in range(2) for oy in range(2) for ox in range(2)]
    if octants is not None:
        octs = [o for o in octs if tuple(o) in {tuple(x) for x in octants}]
    no = len(octs)
    nf = no * len(refine)
    ngrid = nc + nf
    hx, hy, hz = c.dx[0], c.dy[0], c.dz[0]
    bct = np.full((nf, 6), BC_PAR, dtype=np.int32)
    nbr = np.zeros((nf, 26), dtype=np.int32)
    iparent = np.zeros(ngrid, dtype=np.int32)
    position = np.zeros((ngrid, 3), dtype=np.int32)
    xs, ys, zs = [c.x], [c.y], [c.z]
    for r, gc in enumerate(refine):
        gx, gy, gz = c.gridpos[gc - 1]
        for q, (ox, oy, oz) in enumerate(octs):
            g = nc + no * r + q            # 0-based id of the fine grid
            iparent[g] = gc
            position[g] = (3 + ox * (n // 2), 3 + oy * (n // 2), 3 + oz * (n // 2))
            for s in range(1, 27):
                di, dj, dk = slot_offset(s)
                tx, ty, tz = ox + di, oy + dj, oz + dk
                if (tx, ty, tz) in octs:
                    nbr[g - nc, s - 1] = nc + no * r + octs.index((tx, ty, tz)) + 1
            for f in range(1, 7):
                d, hi = (f - 1) // 2, (f - 1) % 2
                o = list((ox, oy, oz))
                o[d] += 1 if hi else -1
                if tuple(o) in octs:
                    bct[g - nc, f - 1] = BC_CON
            i = np.arange(1, ii + 1, dtype=np.float64)
            xs.append(gx * n * hx + ox * n * hx / 2 + (i - 2.5) * hx / 2)
            ys.append(gy * n * hy + oy * n * hy / 2 + (i - 2.5) * hy / 2)
            zs.append(gz * n * hz + oz * n * hz / 2 + (i - 2.5) * hz / 2)
    full = lambda a, h: np.concatenate([a, np.full(nf * ii, h / 2)])
    return Case(
        ngrid=ngrid, kk=kk, jj=jj, ii=ii,
        mgdims=np.tile(np.array([kk, jj, ii], dtype=np.int32), (ngrid, 1)),
        level=np.concatenate([np.ones(nc, dtype=np.int32), np.full(nf, 2, dtype=np.int32)]),
        bctype=np.concatenate([c.bctype, bct]),
        nbrgrid=np.concatenate([c.nbrgrid, nbr]),
        gridpos=np.concatenate([c.gridpos, np.zeros((nf, 3), dtype=np.int32)]),
        x=np.concatenate(xs), y=np.concatenate(ys), z=np.concatenate(zs),
        dx=full(c.dx, hx), dy=full(c.dy, hy), dz=full(c.dz, hz),
        ddx=full(c.ddx, hx), ddy=full(c.ddy, hy), ddz=full(c.ddz, hz),
        iparent=iparent, position=position,
    )


def _stag(case):
    xg, yg, zg = case.coords()
    hx = case.dx.reshape(case.ngrid, case.ii)
    hy = case.dy.reshape(case.ngrid, case.jj)
    hz = case.dz.reshape(case.ngrid, case.kk)
    # calc_stag, corefields_mod.F90:176-192
    return xg, yg, zg, xg + 0.5 * hx, yg + 0.5 * hy, zg + 0.5 * hz


def _eval(case, fn, xa, ya, za):
    out = np.empty((case.ngrid, case.ii, case.jj, case.kk))
    for g in range(case.ngrid):
        X = xa[g][:, None, None]
        Y = ya[g][None, :, None]
        Z = za[g][None, None, :]
        out[g] = fn(X, Y, Z)
    return out.ravel()


def taylor_green(case):
    """3-D Taylor-Green vortex at the staggered positions (init_uvw_expr,
    src/flow/flow_mod.F90:201-248): u at (xstag, y, z), v at (x, ystag, z),
    w at (x, y, zstag), p at the cell centre."""
    xg, yg, zg, xs, ys, zs = _stag(case)
    u = _eval(case, lambda X, Y, Z: np.sin(X) * np.cos(Y) * np.cos(Z), xs, yg, zg)
    v = _eval(case, lambda X, Y, Z: -np.cos(X) * np.sin(Y) * np.cos(Z), xg, ys, zg)
    w = np.zeros(case.idim3d)
    p = _eval(case, lambda X, Y, Z: (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0,
              xg, yg, zg)
    return u, v, w, p


def splitmix64_uniform(n, seed, lo, hi):
    """n uniform doubles in [lo, hi) from a splitmix64 counter stream."""
    with np.errstate(over="ignore"):
        s = (np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
        z = s
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u01 = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u01


def add_noise(case, fields, amplitude=1e-2, seed=42):
    """Seeded uniform noise in [-a, a] on the interior of each field."""
    out = []
    for q, f in enumerate(fields):
        f = f.copy()
        it = case.interior(f)
        it += splitmix64_uniform(it.size, seed + 7919 * q, -amplitude, amplitude).reshape(it.shape)
        out.append(f)
    return out


def gaussian_force(case, rms=0.1, length=0.5, seed=2025):
    """A steady body force drawn from a seeded Gaussian random field: white
    noise on the global periodic cell lattice of the tiling, filtered in
    Fourier space by exp(-(k length)^2 / 2) (correlation length `length`),
    each component scaled to the given rms over the interior.  Returns
    (fx, fy, fz) as flat fields; the ghost layers are 0 (tstle4 reads the
    force on interior points only)."""
    rng = np.random.default_rng(seed)
    n = case.ii - 4
    gp = case.gridpos
    nx, ny, nz = (int(gp[:, q].max()) + 1 for q in range(3))
    N = (nx * n, ny * n, nz * n)
    h = (case.dx[0], case.dy[0], case.dz[0])
    ks = [2 * np.pi * np.fft.fftfreq(N[q], d=h[q]) for q in range(3)]
    k2 = ks[0][:, None, None] ** 2 + ks[1][None, :, None] ** 2 + ks[2][None, None, :] ** 2
    filt = np.exp(-0.5 * k2 * length ** 2)
    out = []
    for _ in range(3):
        g = np.real(np.fft.ifftn(np.fft.fftn(rng.standard_normal(N)) * filt))
        g *= rms / np.sqrt(np.mean(g * g))
        f = np.zeros((case.ngrid, case.ii, case.jj, case.kk))
        for q in range(case.ngrid):
            x0, y0, z0 = gp[q, 0] * n, gp[q, 1] * n, gp[q, 2] * n
            f[q, 2:-2, 2:-2, 2:-2] = g[x0:x0 + n, y0:y0 + n, z0:z0 + n]
        out.append(f.ravel())
    return tuple(out)


def divergence_free_modes(case, nmodes=24, kpeak=4.0, urms=1.0, seed=1234):
    """Solenoidal random field: a sum of Fourier modes with |k| drawn from a
    Gaussian shell around kpeak, each amplitude orthogonal to its wave
    vector (continuous divergence exactly zero), scaled to rms urms."""
    rng = np.random.default_rng(seed)
    Lx = case.dx[0] * (case.ii - 4) * (case.gridpos[:, 0].max() + 1)
    Ly = case.dy[0] * (case.jj - 4) * (case.gridpos[:, 1].max() + 1)
    Lz = case.dz[0] * (case.kk - 4) * (case.gridpos[:, 2].max() + 1)
    modes = []
    while len(modes) < nmodes:
        kmag = rng.normal(kpeak, 1.0)
        if kmag < 1.0:
            continue
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        n = np.round(d * kmag * np.array([Lx, Ly, Lz]) / (2 * np.pi))
        if not n.any():
            continue
        k = 2 * np.pi * n / np.array([Lx, Ly, Lz])
        a = np.cross(k, rng.normal(size=3))
        a /= np.linalg.norm(a)
        modes.append((k, a, rng.uniform(0, 2 * np.pi)))
    xg, yg, zg, xs, ys, zs = _stag(case)

    def comp(c, xa, ya, za):
        def fn(X, Y, Z):
            s = 0.0
            for k, a, ph in modes:
                s = s + a[c] * np.cos(k[0] * X + k[1] * Y + k[2] * Z + ph)
            return s
        return _eval(case, fn, xa, ya, za)

    u = comp(0, xs, yg, zg)
    v = comp(1, xg, ys, zg)
    w = comp(2, xg, yg, zs)
    rms = np.sqrt((np.mean(case.interior(u) ** 2) + np.mean(case.interior(v) ** 2)
                   + np.mean(case.interior(w) ** 2)) / 3.0)
    s = urms / rms
    return u * s, v * s, w * s


def stretch(case, seed=11, amount=0.3):
    """Replace the uniform spacing of a case by a smooth random stretching
    (per grid and axis): cell widths ddx vary by +-amount, cell centres x
    follow from them and dx(i) = x(i+1) - x(i), as a grid generator writes
    them.  Used to exercise non-uniform coefficients; the geometry is no
    longer periodic, which the parity tests do not need."""
    rng = np.random.default_rng(seed)

    def axis(n, ngrid):
        X, D, DD = [], [], []
        for _ in range(ngrid):
            w = 1.0 + amount * np.sin(np.linspace(0, 3, n) + rng.uniform(0, 6)) * rng.uniform(0.5, 1)
            w = w * (2 * np.pi / 24)
            edges = np.concatenate([[0.0], np.cumsum(w)])
            x = 0.5 * (edges[:-1] + edges[1:])
            dx = np.empty(n)
            dx[:-1] = x[1:] - x[:-1]
            dx[-1] = w[-1]
            X.append(x)
            D.append(dx)
            DD.append(w)
        return np.concatenate(X), np.concatenate(D), np.concatenate(DD)

    case.x, case.dx, case.ddx = axis(case.ii, case.ngrid)
    case.y, case.dy, case.ddy = axis(case.jj, case.ngrid)
    case.z, case.dz, case.ddz = axis(case.kk, case.ngrid)
    return case


def block_body(case, lo, hi, nstc=3, seed=7, grids=None):
    """A blocked box of cells in every grid of a case and ghost-cell lists
    around it, in the formats the reference reads from ib_stencils.h5
    (gc_flowstencils_mod.F90:37-100).  lo/hi are the 1-based (i, j, k) of the
    first and last blocked cell; they must stay two cells inside the
    interior.  `grids` (0-based ids) limits the body to those grids; the
    others stay open with empty lists.  The stencils are synthetic (random
    nearby fluid points with random weights): they exercise the runtime, not
    a geometry.

    Returns (bp, lists) with lists[g] = {1: (ncells, xpoli, xpolr,
    xpolrvel), 2: ..., 3: ..., 4: (ncells, fxpoli, fxpolr)}."""
    rng = np.random.default_rng(seed)
    kk, jj, ii = case.kk, case.jj, case.ii
    bp1 = np.ones((ii, jj, kk))
    bp1[lo[0] - 1:hi[0], lo[1] - 1:hi[1], lo[2] - 1:hi[2]] = 0.0
    sel = set(range(case.ngrid)) if grids is None else set(grids)
    bp = np.concatenate([bp1.ravel() if g in sel else np.ones(ii * jj * kk) for g in range(case.ngrid)])
    flat = lambda i, j, k: (k - 1) + (j - 1) * kk + (i - 1) * kk * jj + 1   # 1-based
    shift = {1: (1, 0, 0), 2: (0, 1, 0), 3: (0, 0, 1)}
    lists = []
    empty = (0, np.zeros(0, dtype=np.int64), np.zeros(0), np.zeros(0))
    for g in range(case.ngrid):
        if g not in sel:
            lists.append({1: empty, 2: empty, 3: empty, 4: (0, np.zeros(0, dtype=np.int64), np.zeros(0))})
            continue
        gl = {}
        for comp in (1, 2, 3):
            di, dj, dk = shift[comp]
            xi, xr, xv, n = [], [], [], 0
            for i in range(3, ii - 1):
                for j in range(3, jj - 1):
                    for k in range(3, kk - 1):
                        open_ = bp1[i - 1, j - 1, k - 1] * bp1[i - 1 + di, j - 1 + dj, k - 1 + dk]
                        if open_ != 0.0:
                            continue
                        near = [(i + a, j + b, k + cc) for a in (-1, 0, 1) for b in (-1, 0, 1)
                                for cc in (-1, 0, 1)
                                if bp1[i + a - 1, j + b - 1, k + cc - 1] *
                                bp1[i + a - 1 + di, j + b - 1 + dj, k + cc - 1 + dk] != 0.0]
                        if not near:
                            continue
                        pick = rng.choice(len(near), size=min(nstc, len(near)), replace=False)
                        xi += [flat(i, j, k), len(pick)] + [flat(*near[q]) for q in pick]
                        w = rng.uniform(0.1, 1.0, len(pick))
                        xr += list(-w / w.sum()) + [rng.uniform(-1e-3, 1e-3)]
                        w2 = rng.uniform(0.1, 1.0, len(pick))
                        xv += list(-w2 / w2.sum()) + [0.0]
                        n += 1
            gl[comp] = (n, np.array(xi, dtype=np.int64), np.array(xr), np.array(xv))
        fi, fr, n = [], [], 0
        for i in range(3, ii - 1):
            for j in range(3, jj - 1):
                for k in range(3, kk - 1):
                    if bp1[i - 1, j - 1, k - 1] == 0.0:
                        continue
                    cut = any(bp1[i - 1 + a, j - 1 + b, k - 1 + cc] == 0.0
                              for a, b, cc in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0),
                                               (0, 0, 1), (0, 0, -1)))
                    if not cut:
                        continue
                    fi += [n + 1, flat(i, j, k)]
                    fr += list(rng.uniform(0.2, 1.0, 6) * case.dx[0] * case.dx[0]) + \
                        [rng.uniform(-1e-4, 1e-4)]
                    n += 1
        gl[4] = (n, np.array(fi, dtype=np.int64), np.array(fr))
        lists.append(gl)
    return bp, lists


def _box_ball_distance(lo, hi, c):
    """Distance from point c to the axis-aligned box [lo, hi] (0 inside)."""
    d = np.maximum(np.maximum(lo - c, c - hi), 0.0)
    return float(np.sqrt(np.sum(d * d)))


def body_refined(nx, ny, nz, n=24, length=(8.0, 4.0, 4.0), center=(2.0, 2.0, 2.0),
                 refine_radii=(1.0, 0.7), walls=None):
    """A hierarchy refined around a body: level 1 tiles the box with nx*ny*nz
    grids of n^3 cells (periodic_box, with `walls` on box faces); level L+1
    covers every level-L grid whose box comes within refine_radii[L-1] of
    `center` by 2x2x2 grids at half its spacing, if all its 26 same-level
    neighbours exist (proper nesting), as grids.h5 of a locally refined
    domain holds (src/core/gridio_mod.F90:61-245).  A fine face with
    a same-level grid across it is CON, a fine face on a box face with a
    wall code gets that code, every other fine face is PAR (code 8) towards
    the parent.  Grid ids run level by level, x fastest within a level."""
    from .abi import BC_PAR
    assert n % 2 == 0
    walls = dict(walls or {})
    c0 = periodic_box(nx, ny, nz, n=n, length=length, walls=walls)
    c = np.asarray(center, dtype=np.float64)
    L = np.asarray(length, dtype=np.float64)
    periodic = [not (2 * d + 1 in walls or 2 * d + 2 in walls) for d in range(3)]
    ii = jj = kk = n + 4
    # per level: lattice positions (gx, gy, gz) in grids of that level
    levels = [[tuple(p) for p in c0.gridpos]]
    parents = [[None] * len(levels[0])]
    ntile = [np.array([nx, ny, nz])]
    for lv, r in enumerate(refine_radii):
        size = L / ntile[lv]
        kids, kpar = [], []
        have = set(levels[lv])

        def nested(p, nt=ntile[lv]):
            # proper nesting: all 26 same-level neighbours exist (or lie
            # across a wall), so no fine face looks two levels down
            for s in range(1, 27):
                t = [p[a] + slot_offset(s)[a] for a in range(3)]
                for a in range(3):
                    if periodic[a]:
                        t[a] %= nt[a]
                    elif not 0 <= t[a] < nt[a]:
                        t = None
                        break
                if t is not None and tuple(t) not in have:
                    return False
            return True

        for q, (gx, gy, gz) in enumerate(levels[lv]):
            lo = np.array([gx, gy, gz]) * size
            if _box_ball_distance(lo, lo + size, c) <= r and nested((gx, gy, gz)):
                for oz in range(2):
                    for oy in range(2):
                        for ox in range(2):
                            kids.append((2 * gx + ox, 2 * gy + oy, 2 * gz + oz))
                            kpar.append((q, ox, oy, oz))
        order = sorted(range(len(kids)), key=lambda t: (kids[t][2], kids[t][1], kids[t][0]))
        levels.append([kids[t] for t in order])
        parents.append([kpar[t] for t in order])
        ntile.append(ntile[lv] * 2)
    base = np.cumsum([0] + [len(lv) for lv in levels])
    ngrid = int(base[-1])
    nbr = np.zeros((ngrid, 26), dtype=np.int32)
    bct = np.zeros((ngrid, 6), dtype=np.int32)
    level = np.zeros(ngrid, dtype=np.int32)
    iparent = np.zeros(ngrid, dtype=np.int32)
    position = np.zeros((ngrid, 3), dtype=np.int32)
    gridpos = np.zeros((ngrid, 3), dtype=np.int32)
    xs, ys, zs, hs = [], [], [], []
    for lv, grids in enumerate(levels):
        index = {p: base[lv] + q for q, p in enumerate(grids)}
        nt = ntile[lv]
        size = L / nt
        h = size / n
        for q, p in enumerate(grids):
            g = base[lv] + q
            level[g] = lv + 1
            gridpos[g] = p
            if lv == 0:
                nbr[g] = c0.nbrgrid[q]
                bct[g] = c0.bctype[q]
            else:
                pq, ox, oy, oz = parents[lv][q]
                iparent[g] = base[lv - 1] + pq + 1
                position[g] = (3 + ox * (n // 2), 3 + oy * (n // 2), 3 + oz * (n // 2))

                def find(d):
                    t = [p[0] + d[0], p[1] + d[1], p[2] + d[2]]
                    for a in range(3):
                        if periodic[a]:
                            t[a] %= nt[a]
                        elif not 0 <= t[a] < nt[a]:
                            return 0
                    return index.get(tuple(t), -1) + 1

                for s in range(1, 27):
                    nbr[g, s - 1] = max(find(slot_offset(s)), 0)
                for f in range(1, 7):
                    d = (f - 1) // 2
                    step = [0, 0, 0]
                    step[d] = 1 if f % 2 == 0 else -1
                    t = p[d] + step[d]
                    if not periodic[d] and not 0 <= t < nt[d] and f in walls:
                        bct[g, f - 1] = walls[f]
                    else:
                        bct[g, f - 1] = BC_CON if find(step) > 0 else BC_PAR
            i = np.arange(1, ii + 1, dtype=np.float64)
            xs.append(p[0] * size[0] + (i - 2.5) * h[0])
            ys.append(p[1] * size[1] + (i - 2.5) * h[1])
            zs.append(p[2] * size[2] + (i - 2.5) * h[2])
            hs.append(h)
    hs = np.array(hs)
    return Case(
        ngrid=ngrid, kk=kk, jj=jj, ii=ii,
        mgdims=np.tile(np.array([kk, jj, ii], dtype=np.int32), (ngrid, 1)),
        level=level, bctype=bct, nbrgrid=nbr, gridpos=gridpos,
        x=np.concatenate(xs), y=np.concatenate(ys), z=np.concatenate(zs),
        dx=np.repeat(hs[:, 0], ii), dy=np.repeat(hs[:, 1], jj), dz=np.repeat(hs[:, 2], kk),
        ddx=np.repeat(hs[:, 0], ii), ddy=np.repeat(hs[:, 1], jj), ddz=np.repeat(hs[:, 2], kk),
        iparent=iparent, position=position,
    )
