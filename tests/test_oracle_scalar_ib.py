"""The oracle's ghost-cell IB of the scalars against direct numpy
restatements of the reference's loops: blockbt (blockbt_mod.F90:73-91,
bt = the largest bp of a cell and its six face neighbours) and the
set_scastencils walks (gc_scastencils_mod.F90:1036-1125: a fixed-value body
sets the interface cell from its stencil cells and acoeffvel * value, a
fixed-flux body adds areabyvol * value to its QTT).  The GPU path is
compared with the oracle bit for bit in test_gpu_scalar_ib.py."""
import numpy as np

from mglet_gb300 import abi, cases
from test_oracle_ghostcell import gc_case, load

ISIZE, RSIZE, NPERI = 9, 8, 6


def _prm(**kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=6, ninner=5, nouter_min=6)
    base.update(kw)
    return abi.make_flow_params(**base)


def sca_lists(case, bp, seed=3, nobody_every=5):
    """Synthetic scalar lists: every blocked cell of the interior with a
    fluid face neighbour is an interface cell; its stencil cells are fluid
    cells that are no interface cell (its fluid face neighbours first, then
    other fluid cells of the grid), up to six; bodies 1 and 2 alternate,
    every nobody_every-th cell has none.  Returns per grid (xpoli, xpolr,
    xpolrvel) and the interface cells (1-based positions) per grid."""
    rng = np.random.default_rng(seed)
    kk, jj, ii = case.kk, case.jj, case.ii
    v = case.view(bp)
    out, icells = [], []
    for g in range(case.ngrid):
        b = v[g]
        inter = []
        for i in range(2, ii - 2):
            for j in range(2, jj - 2):
                for k in range(2, kk - 2):
                    if b[i, j, k] != 0.0:
                        continue
                    nb = [(i + 1, j, k), (i - 1, j, k), (i, j + 1, k), (i, j - 1, k), (i, j, k + 1), (i, j, k - 1)]
                    fl = [p for p in nb if b[p] == 1.0]
                    if fl:
                        inter.append(((i, j, k), fl))
        pos = lambda p: 1 + p[2] + p[1] * kk + p[0] * kk * jj
        iset = {pos(p) for p, _ in inter}
        fluid = [pos((i, j, k)) for i in range(2, ii - 2) for j in range(2, jj - 2) for k in range(2, kk - 2)
                 if b[i, j, k] == 1.0 and pos((i, j, k)) not in iset]
        xi, xr, xv = [], [], []
        for n, (p, fl) in enumerate(inter):
            st = [pos(q) for q in fl if pos(q) not in iset][:NPERI]
            while len(st) < 3:
                st.append(int(fluid[rng.integers(len(fluid))]))
            m = int(rng.integers(1, len(st) + 1))
            st = st[:m]
            body = 0 if n % nobody_every == nobody_every - 1 else 1 + n % 2
            xi += [pos(p), body, m] + st + [0] * (NPERI - m)
            coef = list(rng.uniform(-0.5, 1.0, m)) + [0.0] * (NPERI - m)
            xr += [float(rng.uniform(0.1, 2.0))] + coef + [float(rng.uniform(0.2, 1.5))]
            coefv = list(rng.uniform(-0.5, 1.0, m)) + [0.0] * (NPERI - m)
            xv += [float(rng.uniform(0.1, 2.0))] + coefv + [float(rng.uniform(0.2, 1.5))]
        out.append((np.array(xi, dtype=np.int64), np.array(xr), np.array(xv)))
        icells.append(sorted(iset))
    return out, icells


def scalar_ib_setup(s, case, bp, lists, fields, scal, geo, t1):
    """Flow ghost-cell lists and blocking, two scalars, their lists and body
    conditions, in the order a caller would use."""
    load(s, case, bp, lists, fields)
    s.set_scalars([0.71, 2.0], source=[0.0, 0.05], prturb=0.9)
    s.set("T1", t1)
    s.set("T2", 0.5 * t1)
    s.connect(0, 2, "U", "V", "W", "P", corners=True)
    s.connect(0, 2, s1="T1", s2="T2", corners=True)
    s.setpointvalues(True)
    for g, (xi, xr, xv) in enumerate(scal):
        s.set_scastencils(g + 1, xi, xr, xv)
    for isca, (fl, va) in enumerate(geo, start=1):
        s.set_scalar_geometry(isca, fl, va)


GEO = [([0, 1], [1.0, 0.5]), ([1, 0], [0.2, -0.3])]


def test_blockbt_matches_numpy(oracle_lib):
    case, bp, lists = gc_case(seed=7)
    u, v, w, p = cases.taylor_green(case)
    o = oracle_lib.Oracle(case, _prm())
    load(o, case, bp, lists, dict(zip("UVWP", (u, v, w, p))))
    o.set_scalars([0.71])
    bt = case.view(o.get("BT"))
    b = case.view(bp)
    for g in range(case.ngrid):
        ref = b[g, 2:-2, 2:-2, 2:-2].copy()
        for sl in ((slice(3, -1), slice(2, -2), slice(2, -2)), (slice(1, -3), slice(2, -2), slice(2, -2)),
                   (slice(2, -2), slice(3, -1), slice(2, -2)), (slice(2, -2), slice(1, -3), slice(2, -2)),
                   (slice(2, -2), slice(2, -2), slice(3, -1)), (slice(2, -2), slice(2, -2), slice(1, -3))):
            ref = np.maximum(ref, b[g][sl])
        assert np.array_equal(bt[g, 2:-2, 2:-2, 2:-2], ref)


def test_value_condition_of_the_bodies(oracle_lib):
    """After a scalar stage every interface cell of a fixed-value body holds
    sum T(stencil) * coeff + acoeffvel * value, formed in the reference's
    order from the final T (no stencil cell is an interface cell, and the
    closing connect touches only ghost layers)."""
    case, bp, lists = gc_case(seed=7)
    u, v, w, p = cases.taylor_green(case)
    fields = dict(zip("UVWP", (u + 0.2, v, w, p)))
    rng = np.random.default_rng(5)
    t1 = 1.0 + 0.1 * rng.standard_normal(case.idim3d)
    scal, icells = sca_lists(case, bp)
    o = oracle_lib.Oracle(case, _prm())
    scalar_ib_setup(o, case, bp, lists, fields, scal, GEO, t1)
    rk = oracle_lib.rk_scheme("williamson")
    o.timeintegrate_scalar(5e-3, 1, rk)
    n_checked = 0
    for isca, name in ((0, "T1"), (1, "T2")):
        flags, values = GEO[isca]
        t = o.get(name)
        for g, (xi, xr, xv) in enumerate(scal):
            base = g * case.ii * case.jj * case.kk
            for cell in range(len(xi) // ISIZE):
                rec, r = xi[cell * ISIZE:(cell + 1) * ISIZE], xv[cell * RSIZE:(cell + 1) * RSIZE]
                body = rec[1]
                if body <= 0 or flags[body - 1] != 0:
                    continue
                val = 0.0
                for n in range(1, rec[2] + 1):
                    val = val + t[base + rec[2 + n] - 1] * r[n]
                val = val + r[1 + NPERI] * values[body - 1]
                assert t[base + rec[0] - 1] == val
                n_checked += 1
    assert n_checked > 10


def test_flux_condition_of_the_bodies(oracle_lib):
    """With every body a fixed-flux body, the first RK stage (frhs = 0, so
    T += dt b1 QTT) moves each interface cell by dt b1 areabyvol value
    against the same stage without lists; every other interior cell is
    unchanged (set_scastencils "P" on QTT, :71-73; maskbt keeps interface
    cells, whose BT is 1)."""
    case, bp, lists = gc_case(seed=7)
    u, v, w, p = cases.taylor_green(case)
    fields = dict(zip("UVWP", (u + 0.2, v, w, p)))
    t1 = 1.0 + 0.1 * np.random.default_rng(5).standard_normal(case.idim3d)
    scal, _ = sca_lists(case, bp)
    geo = [([1, 1], [0.8, -0.4]), ([1, 1], [0.0, 0.0])]
    dt, rk = 5e-3, oracle_lib.rk_scheme("williamson")
    out = []
    for with_lists in (False, True):
        o = oracle_lib.Oracle(case, _prm())
        scalar_ib_setup(o, case, bp, lists, fields, scal if with_lists else [], geo, t1)
        o.timeintegrate_scalar(dt, 1, rk)
        out.append(o.get("T1"))
    dtfu = dt * rk.b[0]
    expect = np.zeros(case.idim3d)
    flags, values = geo[0]
    for g, (xi, xr, xv) in enumerate(scal):
        base = g * case.ii * case.jj * case.kk
        for cell in range(len(xi) // ISIZE):
            body = xi[cell * ISIZE + 1]
            if body > 0:
                expect[base + xi[cell * ISIZE] - 1] += dtfu * xv[cell * RSIZE] * values[body - 1]
    diff = case.interior(out[1] - out[0])
    assert np.count_nonzero(case.interior(expect)) > 10
    assert np.allclose(diff, case.interior(expect), rtol=1e-9, atol=1e-14)
