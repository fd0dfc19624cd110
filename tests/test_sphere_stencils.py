"""The ghost-cell stencil construction (mglet_create_flowstencils) and the
sphere blocking, on the CPU.

The library's builder restates fluxcorrection / fluxstencil / calcflux of
src/flow/gc_flowstencils_mod.F90:199-920 with the helpers of
src/ib/gc_createstencils_mod.F90; here a second, loop-by-loop numpy/Python
transcription of the same Fortran (written independently of the C++) must
reproduce every list bit for bit on a small sphere case.  The blocking
checks are the hierarchy rules the reference's blocking leaves behind: the
'E' restriction (a coarse cell under fine grids is open iff one of its
children is, gc_restrict_mod.F90:290-324) and BU = BP(i) BP(i+1)."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases, channel

MACCUR = float(np.float32(1.0e-4))
F09 = float(np.float32(0.9))
F061 = float(np.float32(0.61))


def _ball():
    out = []
    for i in range(1, 8):
        for j in range(1, 8):
            for k in range(1, 8):
                a, b, c = i - 4, j - 4, k - 4
                if (a, b, c) != (0, 0, 0) and (a * a + b * b + c * c) ** 0.5 <= 3:
                    out.append((a, b, c))
    return out


BALL = _ball()


class G:
    """One grid's arrays with the reference's 1-based (k, j, i) access."""

    def __init__(self, case, geo, g):
        self.kk, self.jj, self.ii = case.kk, case.jj, case.ii
        npg = case.kk * case.jj * case.ii
        sl = slice(g * npg, (g + 1) * npg)
        shp = (case.ii, case.jj, case.kk)
        for n in ("bp", "bu", "bv", "bw", "areau", "areav", "areaw"):
            setattr(self, n, geo[n][sl].reshape(shp))
        self.bz = geo["bzelltyp"][sl].reshape(shp)
        off = int(geo["icells"][:g].sum())
        n = int(geo["icells"][g])
        self.nv = geo["nvecs"][off:off + n]
        self.uc = geo["ucell"][off:off + n]
        self.bc = list(case.bctype[g])
        x, y, z = (a[g] for a in case.coords())
        dx, dy, dz = (a.reshape(case.ngrid, -1)[g] for a in (case.dx, case.dy, case.dz))
        ddx, ddy, ddz = (a.reshape(case.ngrid, -1)[g] for a in (case.ddx, case.ddy, case.ddz))
        pad = lambda a: np.concatenate([[0.0], a])          # 1-based
        self.x, self.y, self.z = pad(x), pad(y), pad(z)
        self.xs, self.ys, self.zs = pad(x + 0.5 * dx), pad(y + 0.5 * dy), pad(z + 0.5 * dz)
        self.ddx, self.ddy, self.ddz = pad(ddx), pad(ddy), pad(ddz)

    @staticmethod
    def v(a, k, j, i):
        return float(a[i - 1, j - 1, k - 1])

    def flat(self, k, j, i):
        return 1 + (k - 1) + (j - 1) * self.kk + (i - 1) * self.jj * self.kk


def findif(gr, b, k, j, i):
    v = G.v
    f = dict(found=0, x1=0, x2=0, y1=0, y2=0, z1=0, z2=0, nr=0)
    if v(b, k, j, i) <= 0.5:
        for key, (kq, jq, iq) in (("x1", (k, j, i + 1)), ("x2", (k, j, i - 1)), ("y1", (k, j + 1, i)),
                                  ("y2", (k, j - 1, i)), ("z1", (k + 1, j, i)), ("z2", (k - 1, j, i))):
            if v(b, kq, jq, iq) >= 0.5:
                f["nr"] += 1
                f["found"] = 1
                f[key] = 1
    return f


def calcfluxu(k, j, i, x, y, z, xstag, ystag, zstag, a, b, c, dpl, avel, pts):
    velpts = len(pts)
    dpoint = a * xstag[i] + b * ystag[j] + c * zstag[k] - dpl
    dist = []
    dall = 0.0
    for (it, jt, kt) in pts:
        d = a * xstag[it] + b * ystag[jt] + c * zstag[kt] - dpl
        if d < abs(dpoint) * F09:
            d = 0.0
        dist.append(d)
        dall = dall + d * d
    if abs(dall) <= 2.2250738585072014e-308:
        return 0, None
    ce = [d / dall for d in dist]
    cesum = 0.0
    for q in ce:
        cesum = cesum + q
    dy = y[j] - y[j - 1]
    dz = z[k] - z[k - 1]
    ddy = dy / 20.0
    ddz = dz / 20.0
    ys = y[j - 1] - ddy / 2.0
    zs = z[k - 1] - ddz / 2.0
    co = [0.0] * velpts
    ac = 0.0
    carea2 = 0
    xm = xstag[i]
    dt = -dpl + a * xm
    for jt in range(1, 21):
        ym = ys + ddy * float(jt)
        for kt in range(1, 21):
            zm = zs + ddz * float(kt)
            if dt + b * ym + c * zm > 0.0:
                dp = a * xm + b * ym + c * zm - dpl
                for n in range(velpts):
                    co[n] = co[n] + dp * ce[n]
                ac = ac + 1.0 - dp * cesum
            else:
                carea2 += 1
    area = ddy * ddz
    co = [q * area / (dy * dz) for q in co]
    ac = ac * avel * area / (dy * dz)
    ac = ac + avel * (float(carea2) * area) / (dy * dz)
    dpoint = a * xstag[i] + b * ystag[j] + c * zstag[k] - dpl
    cv = [dpoint * q for q in ce]
    acv = avel * (1.0 - dpoint * cesum)
    s = 0.0
    for q in co:
        s = s + q
    return (-1 if s > F061 else 1), (co, ac, cv, acv)


def fluxstencil(gr, b, compon):
    xi, xr, xv, n = [], [], [], 0
    kb, jb, ib = (2 if compon == 3 else 3), (2 if compon == 2 else 3), (2 if compon == 1 else 3)
    di, dj, dk = int(compon == 1), int(compon == 2), int(compon == 3)
    ir = []
    for t in gr.bc:
        r = 2
        if t in (3, 4, 6):
            r = 0
        if t in (7, 8):
            r = 1
        ir.append(r)
    for i in range(ib, gr.ii - 1):
        for j in range(jb, gr.jj - 1):
            for k in range(kb, gr.kk - 1):
                if findif(gr, b, k, j, i)["found"] != 1:
                    continue
                cells = []
                if gr.v(gr.bz, k, j, i) < 0:
                    cells.append((k, j, i))
                if gr.v(gr.bz, k + dk, j + dj, i + di) < 0:
                    cells.append((k + dk, j + dj, i + di))
                if not cells:
                    xi += [gr.flat(k, j, i), 0]
                    xr += [0.0]
                    xv += [0.0]
                    n += 1
                    continue
                # wmcheckneighbor + choosestencil
                open_ = []
                for (a, bb, c) in BALL:
                    it, jt, kt = i + a, j + bb, k + c
                    if it < 3 - ir[0] or it > gr.ii - 2 + ir[1] or jt < 3 - ir[2] or \
                            jt > gr.jj - 2 + ir[3] or kt < 3 - ir[4] or kt > gr.kk - 2 + ir[5]:
                        continue
                    if int(round(gr.v(b, kt, jt, it))) == 1:
                        open_.append((it, jt, kt))
                pts = [p for p in open_ if abs(p[0] - i) + abs(p[1] - j) + abs(p[2] - k) == 1]
                if len(pts) == 1:
                    t = (2 * pts[0][0] - i, 2 * pts[0][1] - j, 2 * pts[0][2] - k)
                    pts += [p for p in open_ if p == t]
                if len(pts) == 1:
                    pts = []
                done = False
                for (kt, jt, it) in cells:
                    if len(pts) > 6 or not pts:
                        continue
                    a, bb, c, dpl = gr.nv[-int(gr.v(gr.bz, kt, jt, it)) - 1]
                    uc = gr.uc[-int(gr.v(gr.bz, kt, jt, it)) - 1]
                    if compon == 1:
                        f, res = calcfluxu(k, j, i, gr.x, gr.ys, gr.zs, gr.xs, gr.y, gr.z, a, bb, c,
                                           dpl, uc[0], [(p[0], p[1], p[2]) for p in pts])
                    elif compon == 2:
                        f, res = calcfluxu(k, i, j, gr.y, gr.xs, gr.zs, gr.ys, gr.x, gr.z, bb, a, c,
                                           dpl, uc[1], [(p[1], p[0], p[2]) for p in pts])
                    else:
                        f, res = calcfluxu(i, j, k, gr.z, gr.ys, gr.xs, gr.zs, gr.y, gr.x, c, bb, a,
                                           dpl, uc[2], [(p[2], p[1], p[0]) for p in pts])
                    if f == 1 and any(abs(q) > 12.0 for q in res[2]):
                        f = -4
                    if f != 1:
                        continue
                    co, ac, cv, acv = res
                    if not done:
                        xi += [gr.flat(k, j, i), len(pts)] + [gr.flat(p[2], p[1], p[0]) for p in pts]
                        xr += co + [ac]
                        xv += cv + [acv]
                        done = True
                    else:
                        m = len(pts) + 1
                        xr[-m:] = [0.5 * o + 0.5 * q for o, q in zip(xr[-m:], co + [ac])]
                        xv[-m:] = [0.5 * o + 0.5 * q for o, q in zip(xv[-m:], cv + [acv])]
                if not done:
                    k0, j0, i0 = cells[0]
                    av = gr.uc[-int(gr.v(gr.bz, k0, j0, i0)) - 1][compon - 1]
                    xi += [gr.flat(k, j, i), 0]
                    xr += [av]
                    xv += [av]
                n += 1
    return n, np.array(xi, dtype=np.int64), np.array(xr), np.array(xv)


def fluxcorrection(gr):
    xi, xr, n = [], [], 0
    nfro, nbac, nrgt, nlft, nbot, ntop = gr.bc
    imax, jmax, kmax = gr.ii - 2, gr.jj - 2, gr.kk - 2
    if nbac == 7:
        imax = gr.ii - 1
    if nlft == 7:
        jmax = gr.jj - 1
    if ntop == 7:
        kmax = gr.kk - 1
    v = G.v
    wall = lambda t: t in (2, 5, 6)
    for i in range(3, imax + 1):
        for j in range(3, jmax + 1):
            for k in range(3, kmax + 1):
                f = findif(gr, gr.bp, k, j, i)
                if f["found"] != 1:
                    continue
                dx, dy, dz = gr.ddx[i], gr.ddy[j], gr.ddz[k]
                cx2 = float(findif(gr, gr.bu, k, j, i - 1)["found"])
                cx1 = float(findif(gr, gr.bu, k, j, i)["found"])
                cy2 = float(findif(gr, gr.bv, k, j - 1, i)["found"])
                cy1 = float(findif(gr, gr.bv, k, j, i)["found"])
                cz2 = float(findif(gr, gr.bw, k - 1, j, i)["found"])
                cz1 = float(findif(gr, gr.bw, k, j, i)["found"])
                # a stationary body: every body velocity is zero
                xvel = yvel = zvel = 0.0
                acoeff = (1.0 - cx1) * xvel * dy * dz - (1.0 - cx2) * xvel * dy * dz + \
                    (1.0 - cy1) * yvel * dx * dz - (1.0 - cy2) * yvel * dx * dz + \
                    (1.0 - cz1) * zvel * dx * dy - (1.0 - cz2) * zvel * dx * dy
                ax1, ax2, ay1, ay2, az1, az2 = (float(f[q]) for q in ("x1", "x2", "y1", "y2", "z1", "z2"))
                if i == 3 and wall(nfro):
                    ax2 = 0.0
                if i == gr.ii - 2 and wall(nbac):
                    ax1 = 0.0
                if j == 3 and wall(nrgt):
                    ay2 = 0.0
                if j == gr.jj - 2 and wall(nlft):
                    ay1 = 0.0
                if k == 3 and wall(nbot):
                    az2 = 0.0
                if k == gr.kk - 2 and wall(ntop):
                    az1 = 0.0
                au = [v(gr.areau, k, j, i), v(gr.areau, k, j, i - 1), v(gr.areav, k, j, i),
                      v(gr.areav, k, j - 1, i), v(gr.areaw, k, j, i), v(gr.areaw, k - 1, j, i)]
                sarea = ax1 * au[0] + ax2 * au[1] + ay1 * au[2] + ay2 * au[3] + az1 * au[4] + az2 * au[5]
                r3 = (dx + dy + dz) / 3.0
                if sarea > r3 * r3 * MACCUR:
                    ax1, ax2, ay1, ay2, az1, az2 = (q * w for q, w in zip((ax1, ax2, ay1, ay2, az1, az2), au))
                n += 1
                xi += [f["nr"], gr.flat(k, j, i)]
                xr += [ax1, ax2, ay1, ay2, az1, az2, acoeff]
    return n, np.array(xi, dtype=np.int64), np.array(xr)


@pytest.fixture(scope="module")
def small():
    """Two levels around a sphere of 6.4 coarse cells in a 2 x 1 x 1 channel."""
    sc = channel.SphereChannel(tiles=(4, 2, 2), n=8, grid_size=0.5, diameter=0.4,
                               refine_radii=(0.35,))
    return sc


def test_blocking_restriction_and_faces(small):
    case, geo = small.case, small.geo
    v = lambda a, g: a.reshape(case.ngrid, case.ii, case.jj, case.kk)[g]
    bp = geo["bp"]
    n = case.ii - 4
    checked = 0
    for g in range(case.ngrid):
        par = case.iparent[g]
        if not par:
            continue
        fine, coarse = v(bp, g), v(bp, par - 1)
        ip, jp, kp = case.position[g]
        for a in range(n // 2):
            for b in range(n // 2):
                for c in range(n // 2):
                    kids = fine[2 + 2 * a:4 + 2 * a, 2 + 2 * b:4 + 2 * b, 2 + 2 * c:4 + 2 * c]
                    assert coarse[ip - 1 + a, jp - 1 + b, kp - 1 + c] == kids.max()
                    checked += 1
    assert checked > 0
    B = bp.reshape(case.ngrid, case.ii, case.jj, case.kk)
    BU = geo["bu"].reshape(B.shape)
    assert np.array_equal(BU[:, :-1], B[:, :-1] * B[:, 1:])
    assert (bp == 0).any() and geo["icells"].sum() > 0
    # open areas lie between 0 and the face area
    ddy = case.ddy.reshape(case.ngrid, -1)[:, None, :, None]
    ddz = case.ddz.reshape(case.ngrid, -1)[:, None, None, :]
    au = geo["areau"].reshape(B.shape)
    assert np.all(au >= 0) and np.all(au <= ddy * ddz * (1 + 1e-12))


def test_stencils_match_transcription(small):
    """Every grid with a cut cell: the library's lists equal the Python
    transcription of fluxcorrection / fluxstencil bit for bit."""
    case, geo = small.case, small.geo
    lists = small.lists
    grids = [g for g in range(case.ngrid) if geo["icells"][g] > 0]
    assert grids
    for g in grids:
        gr = G(case, geo, g)
        n, fi, fr = fluxcorrection(gr)
        ln, lfi, lfr = lists[g][4]
        assert ln == n and np.array_equal(lfi, fi) and np.array_equal(lfr, fr), g
        for comp, b in ((1, gr.bu), (2, gr.bv), (3, gr.bw)):
            n, xi, xr, xv = fluxstencil(gr, b, comp)
            ln, lxi, lxr, lxv = lists[g][comp]
            assert ln == n, (g, comp)
            assert np.array_equal(lxi, xi), (g, comp)
            assert np.array_equal(lxr, xr), (g, comp)
            assert np.array_equal(lxv, xv), (g, comp)


def test_stencil_entries_are_sane(small):
    """Entries with stencil points: at most 6 points, flux weights summing to
    at most 0.61 (calcfluxu's acceptance limit), velocity weights within
    12, stencil points open and inside the grid."""
    case, geo = small.case, small.geo
    npg = case.kk * case.jj * case.ii
    total = 0
    for g, gl in enumerate(small.lists):
        blk = {1: geo["bu"], 2: geo["bv"], 3: geo["bw"]}
        for comp in (1, 2, 3):
            n, xi, xr, xv = gl[comp]
            p = q = 0
            for _ in range(n):
                m = int(xi[p + 1])
                assert 0 <= m <= 6
                if m:
                    assert xr[q:q + m].sum() <= F061
                    assert np.all(np.abs(xv[q:q + m]) <= 12.0)
                    pts = xi[p + 2:p + 2 + m]
                    assert np.all((pts >= 1) & (pts <= npg))
                    assert np.all(blk[comp][g * npg + pts - 1] == 1.0)
                    total += 1
                p += 2 + m
                q += m + 1
            assert p == len(xi) and q == len(xr)
    assert total > 0


def test_body_refined_hierarchy():
    """The full configuration's hierarchy: 16 x 8 x 8 level-1 grids and
    uneven finer levels, every fine grid inside its parent, faces CON
    exactly where a same-level neighbour exists."""
    case = cases.body_refined(16, 8, 8, n=24, length=(8.0, 4.0, 4.0), center=(2.0, 2.0, 2.0),
                              refine_radii=(1.0, 1.0), walls={1: abi.BC_FIX, 2: abi.BC_OP1})
    counts = [int((case.level == lv).sum()) for lv in (1, 2, 3)]
    assert counts[0] == 1024 and 500 <= counts[1] <= 800 and 1800 <= counts[2] <= 2600
    for g in range(case.ngrid):
        if case.level[g] == 1:
            continue
        assert case.level[case.iparent[g] - 1] == case.level[g] - 1
        for f in range(6):
            nb = case.nbrgrid[g, f]
            assert (case.bctype[g, f] == abi.BC_CON) == (nb > 0)
            assert case.bctype[g, f] in (abi.BC_CON, abi.BC_PAR)


def test_sample_steps_on_the_oracle(oracle_lib):
    """The bounded sample with three levels runs: one RK3 step on the oracle
    keeps every field finite and the CFL number below 1.5 (the flow speeds
    up around the sphere after the impulsive start)."""
    sc = channel.SphereChannel(tiles=(4, 2, 2), n=8, grid_size=0.5, diameter=0.4,
                               refine_radii=(0.35, 0.25))
    prm = sc.flow_params(nouter=6, ninner=5, nouter_min=6)
    o = oracle_lib.Oracle(sc.case, prm)
    sc.setup(o)
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        st = o.timeintegrate_flow(1, 1, 0.0, sc.dt(), irk, rk)
        assert np.isfinite(st.maxrhs)
    info = o.itinfo(sc.dt())
    assert not info.exploded and 0.0 < info.cflmax < 1.5
    for n in "UVWP":
        assert np.all(np.isfinite(o.get(n)))
