"""The scalar ghost-cell list construction (mglet_create_scastencils) on the
CPU: a loop-by-loop Python transcription of tscastencil, tscastencilcoeff,
calcfluxtsca and the area / full / rescue records of
src/scalar/gc_scastencils_mod.F90:127-946 (with wmcheckneighbor and
choosestencil of src/ib/gc_createstencils_mod.F90) must reproduce every
grid's list bit for bit on the two-level sphere case; the cut cells' areas
and body ids are synthetic (two bodies, so the choice of the largest body
id matters).  The lists then drive the oracle's scalar stage."""
import numpy as np

from mglet_gb300 import gpu
from test_sphere_stencils import BALL, G, findif, small  # noqa: F401  (small is a fixture)

F02 = float(np.float32(0.2))
F061 = float(np.float32(0.61))
TINY = np.finfo(np.float64).tiny
HUGE = np.finfo(np.float64).max
NPERI = 6


def _open_points(gr, k, j, i):
    ir = []
    for t in gr.bc:
        ir.append(0 if t in (3, 4, 6) else (1 if t in (7, 8) else 2))
    pts = []
    for (a, b, c) in BALL:
        it, jt, kt = i + a, j + b, k + c
        if it < 3 - ir[0] or it > gr.ii - 2 + ir[1]:
            continue
        if jt < 3 - ir[2] or jt > gr.jj - 2 + ir[3]:
            continue
        if kt < 3 - ir[4] or kt > gr.kk - 2 + ir[5]:
            continue
        if int(round(gr.v(gr.bp, kt, jt, it))) == 1:
            pts.append((kt, jt, it))
    return pts


def _choose(k, j, i, pts):
    face = [p for p in pts if abs(p[0] - k) + abs(p[1] - j) + abs(p[2] - i) == 1]
    if len(face) == 1:
        beyond = (2 * face[0][0] - k, 2 * face[0][1] - j, 2 * face[0][2] - i)
        face += [p for p in pts if p == beyond]
    return [] if len(face) == 1 else face


def _calcfluxtsca(gr, k, j, i, plane, pts):
    a, b, c, dpl = plane
    m = len(pts)
    co, cv = [0.0] * m, [0.0] * m
    ac = 0.0
    dpoint = a * gr.x[i] + b * gr.y[j] + c * gr.z[k] - dpl
    dist, dall = [], 0.0
    for (kt, jt, it) in pts:
        d = a * gr.x[it] + b * gr.y[jt] + c * gr.z[kt] - dpl
        if d < abs(dpoint) * F02:
            d = 0.0
        dist.append(d)
        dall = dall + d * d
    if abs(dall) < TINY:
        return -11, None
    ce = [d / dall for d in dist]
    cesum = 0.0
    for e in ce:
        cesum = cesum + e
    parts = 20
    ddi, ddj, ddk = gr.ddx[i] / parts, gr.ddy[j] / parts, gr.ddz[k] / parts
    xs, ys, zs = gr.xs[i - 1] - ddi / 2.0, gr.ys[j - 1] - ddj / 2.0, gr.zs[k - 1] - ddk / 2.0
    dvol = ddi * ddj * ddk
    nfluid = 0
    for i2 in range(1, parts + 1):
        xm = xs + ddi * float(i2)
        for j2 in range(1, parts + 1):
            ym = ys + ddj * float(j2)
            for k2 in range(1, parts + 1):
                zm = zs + ddk * float(k2)
                d = (a * xm + b * ym + c * zm) - dpl
                if d > 0.0:
                    co = [q + d * e for q, e in zip(co, ce)]
                    ac = ac + (1.0 - d * cesum)
                    nfluid += 1
    if nfluid > 0:
        co = [q * dvol / (nfluid * dvol) for q in co]
        ac = ac * dvol / (nfluid * dvol)
    else:
        co, ac = [0.0] * m, 0.0
    dpoint = a * gr.x[i] + b * gr.y[j] + c * gr.z[k] - dpl
    cv = [dpoint * e for e in ce]
    acv = 1.0 - dpoint * cesum
    s = 0.0
    for q in co:
        s = s + q
    return (-12 if s > F061 else 1), (co, ac, cv, acv)


def transcribe(gr, area, body):
    xi, xr, xv = [], [], []

    def record(cell, bid, pts, aby, co, cv, ac, acv):
        xi.extend([gr.flat(k, j, i) for (k, j, i) in [cell]] + [bid, len(pts)] +
                  [gr.flat(*p) for p in pts] + [-1] * (NPERI - len(pts)))
        xr.extend([aby] + list(co) + [-HUGE] * (NPERI - len(pts)) + [ac])
        xv.extend([aby] + list(cv) + [-HUGE] * (NPERI - len(pts)) + [acv])

    for i in range(3, gr.ii - 1):
        for j in range(3, gr.jj - 1):
            for k in range(3, gr.kk - 1):
                f = findif(gr, gr.bp, k, j, i)
                bz = int(gr.v(gr.bz, k, j, i))
                vol = gr.ddx[i] * gr.ddy[j] * gr.ddz[k]
                if f["found"] == 0:
                    if bz < 0 and gr.v(gr.bp, k, j, i) > 0.5:
                        record((k, j, i), int(body[-bz - 1]), [(k, j, i)], area[-bz - 1] / vol,
                               [1.0], [1.0], 0.0, 0.0)
                    continue
                target = None
                if bz < 0:
                    target = (k, j, i)
                else:
                    best = 0
                    for key, p in (("x1", (k, j, i + 1)), ("x2", (k, j, i - 1)), ("y1", (k, j + 1, i)),
                                   ("y2", (k, j - 1, i)), ("z1", (k + 1, j, i)), ("z2", (k - 1, j, i))):
                        bq = int(gr.v(gr.bz, *p))
                        if f[key] == 1 and bq < 0 and int(body[-bq - 1]) > best:
                            best = int(body[-bq - 1])
                            target = p
                if target is None:
                    record((k, j, i), 0, [], 0.0, [], [], 1.0, 1.0)
                    continue
                bt = int(gr.v(gr.bz, *target))
                aby = area[-bt - 1] / vol if target == (k, j, i) else 0.0
                bid = int(body[-bt - 1])
                pts = _choose(k, j, i, _open_points(gr, k, j, i))
                ok = False
                if 0 < len(pts) <= NPERI:
                    found, res = _calcfluxtsca(gr, k, j, i, gr.nv[-bt - 1], pts)
                    if found == 1 and not any(abs(q) > 12.0 for q in res[2]):
                        co, ac, cv, acv = res
                        record((k, j, i), bid, pts, aby, co, cv, ac, acv)
                        ok = True
                if not ok:
                    record((k, j, i), bid, [], aby, [], [], 1.0, 1.0)
    return np.array(xi, dtype=np.int64), np.array(xr), np.array(xv)


def _cut_data(geo, seed=4):
    rng = np.random.default_rng(seed)
    n = int(geo["icells"].sum())
    return 0.05 + rng.random(n), (1 + np.arange(n) % 2).astype(np.int32)


def test_scalar_stencils_match_transcription(small):
    case, geo = small.case, small.geo
    area, body = _cut_data(geo)
    lists = gpu.create_scastencils(case, geo, area, body)
    grids = [g for g in range(case.ngrid) if geo["icells"][g] > 0]
    assert grids
    kinds = set()
    for g in grids:
        off = int(geo["icells"][:g].sum())
        n = int(geo["icells"][g])
        gr = G(case, geo, g)
        xi, xr, xv = transcribe(gr, area[off:off + n], body[off:off + n])
        lxi, lxr, lxv = lists[g]
        assert np.array_equal(lxi, xi), g
        assert np.array_equal(lxr, xr), g
        assert np.array_equal(lxv, xv), g
        kinds |= set(int(m) for m in xi.reshape(-1, 9)[:, 2])
    # full stencils, rescue records and area records all occur
    assert 0 in kinds and any(m >= 2 for m in kinds)
    for g in range(case.ngrid):
        if geo["icells"][g] == 0:
            assert len(lists[g][0]) == 0


def test_scalar_stencils_drive_the_oracle(small, oracle_lib):
    """The constructed lists with a fixed-value and a fixed-flux body drive
    the oracle's scalar stage on the sphere hierarchy (fields stay finite);
    the GPU's stage on the same lists is compared with the oracle in
    test_gpu_scalar_ib.py."""
    case, geo = small.case, small.geo
    area, body = _cut_data(geo)
    scal = gpu.create_scastencils(case, geo, area, body)
    o = oracle_lib.Oracle(case, small.flow_params(nouter=6, ninner=5, nouter_min=6))
    small.setup(o)
    o.set_scalars([0.71])
    o.set("T1", np.ones(case.idim3d))
    for g, (xi, xr, xv) in enumerate(scal):
        o.set_scastencils(g + 1, xi, xr, xv)
    o.set_scalar_geometry(1, [0, 1], [2.0, 0.5])
    o.timeintegrate_scalar(5e-3, 1, oracle_lib.rk_scheme("williamson"))
    assert np.all(np.isfinite(o.get("T1")))


def test_plane_box_areas():
    """Sections of the unit cube with known areas: a mid plane (1), the
    hexagon normal to a diagonal (3 sqrt(3) / 4), the diagonal rectangle
    (sqrt 2), a corner triangle (sqrt(3) / 8), and a plane that misses."""
    from mglet_gb300.geometry import plane_box_area
    s2, s3 = np.sqrt(2.0), np.sqrt(3.0)
    nv = np.array([[1, 0, 0, 0.5], [1 / s3, 1 / s3, 1 / s3, 1.5 / s3], [1 / s2, 1 / s2, 0, 1 / s2],
                   [1 / s3, 1 / s3, 1 / s3, 0.5 / s3], [0, 0, 1, 2.0]])
    lo, hi = np.zeros((5, 3)), np.ones((5, 3))
    assert np.allclose(plane_box_area(nv, lo, hi), [1.0, 3 * s3 / 4, s2, s3 / 8, 0.0], rtol=1e-12, atol=0)


def test_sphere_interface_area_and_scalar_lists(small):
    """The blocking's interface areas of the finer level (which covers the
    sphere) add up to the sphere's surface within 15 %, and the scalar lists
    built from them carry areabyvol = area / cell volume on the cut cells."""
    case, geo = small.case, small.geo
    r = 0.2
    fine = [g for g in range(case.ngrid) if case.level[g] == case.level.max()]
    off = np.concatenate([[0], np.cumsum(geo["icells"])])
    total = 0.0
    for g in fine:   # interior cells only: ghost layers repeat the neighbours' cells
        bz = geo["bzelltyp"].reshape(case.ngrid, case.ii, case.jj, case.kk)[g, 2:-2, 2:-2, 2:-2]
        total += geo["arealist"][off[g] - bz[bz < 0] - 1].sum()
    assert abs(total / (4 * np.pi * r * r) - 1.0) < 0.15, total
    assert np.all(geo["bodyid"] == 1)
    scal = gpu.create_scastencils(case, geo, geo["arealist"], geo["bodyid"])
    n_area = 0
    for g in fine:
        xi, xr, _ = scal[g]
        rec_i, rec_r = xi.reshape(-1, 9), xr.reshape(-1, 8)
        assert np.all(rec_r[:, 0] >= 0.0)
        n_area += int(np.count_nonzero(rec_r[:, 0] > 0.0))
    assert n_area > 0
