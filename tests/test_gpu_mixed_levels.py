"""The batched mixed form on grid hierarchies against the FP64 oracle.

The inner SIP iterations run level by level in FP32 on the plane-ordered
arrays, with the level operators of mgpoisl (ctof, parent + bound_pressure,
ftoc of the correction and of the residual) restated on that layout, and
the fluxes of grids with PAR faces corrected by tstle4_par before their RK
update.  With the outer loop converged on both sides the fields agree to
the tolerances stated per test.
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_levels import prepare_levels

pytestmark = pytest.mark.gpu

HIERARCHIES = [
    dict(nx=2, ny=2, nz=2, n=8, refine=(1,)),
    dict(nx=3, ny=2, nz=2, n=12, refine=(1, 3)),
]


def _prm(form, gmol=1e-2, **kw):
    base = dict(gmol=gmol, epcorr=1e-10, nouter=40, ninner=5, nouter_min=0, form=form)
    base.update(kw)
    return abi.make_flow_params(**base)


def _errors(case, a, b):
    """Relative L2 of the velocity vector and of the pressure (mean removed)
    over the interior of every grid."""
    num = sum(np.sum((case.interior(a.get(n)) - case.interior(b.get(n))) ** 2) for n in "UVW")
    den = sum(np.sum(case.interior(b.get(n)) ** 2) for n in "UVW")
    pa, pb = case.interior(a.get("P")), case.interior(b.get("P"))
    pa, pb = pa - pa.mean(), pb - pb.mean()
    return float(np.sqrt(num / den)), float(np.linalg.norm(pa - pb) / np.linalg.norm(pb))


def _run(case, solvers, rks, dt, steps):
    """Runs both solvers stage by stage; returns per stage the relative
    residual maxrhs / prefak each reached."""
    hist = []
    for it in range(1, steps + 1):
        for irk in (1, 2, 3):
            stats = [s.timeintegrate_flow(it, it, 0.0, dt, irk, rk) for s, rk in zip(solvers, rks)]
            for st in stats:
                assert np.isfinite(st.maxrhs)
                assert st.maxrhs / st.prefak < 1e-10 or st.nouter_done == 40
            hist.append([st.maxrhs / st.prefak for st in stats])
    return np.array(hist)


@pytest.mark.parametrize("h", HIERARCHIES)
def test_mixed_hierarchy_against_oracle(gpu_lib, oracle_lib, h):
    """Two-level periodic hierarchies (cases.refined_box), Taylor-Green with
    noise, two RK3 steps: velocity to relative L2 <= 1e-7, pressure to 1e-5."""
    case = cases.refined_box(h["nx"], h["ny"], h["nz"], n=h["n"], refine=h["refine"])
    g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED))
    o = oracle_lib.Oracle(case, _prm(abi.FORM_PLAIN))
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=1e-2, seed=42)
    for s in (g, o):
        for nm, a in zip("UVWP", (u, v, w, p)):
            s.set(nm, a)
        s.set_hierarchy(case.iparent, case.position)
        for lvl in (1, 2):
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        prepare_levels(s, case)
    _run(case, (g, o), (gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")), 2e-3, 2)
    ev, ep = _errors(case, g, o)
    print(f"refined_box {h}: velocity {ev:.3e}, pressure {ep:.3e}")
    assert ev <= 1e-7, ev
    assert ep <= 1e-5, ep
    ig, io = g.itinfo(2e-3), o.itinfo(2e-3)
    assert abs(ig.cflmax - io.cflmax) <= 1e-6 * io.cflmax
    g.close()


def test_mixed_channel_hierarchy_against_oracle(gpu_lib, oracle_lib):
    """The sphere channel's hierarchy without the body: 4 x 2 x 2 level-1
    grids of 8^3 cells refined twice around the channel's quarter point
    (16 + 64 + 224 grids), FIX inflow u = 1, OP1 outflow, periodic in y and
    z, a Taylor-Green perturbation on the mean flow; three RK3 steps at CFL
    0.5 on the finest level.  On this hierarchy the reference's outer loop
    leaves a relative residual of 0.04 to 0.5 after 40 iterations (both
    forms, the same residual in every stage to 1e-3), so the outer loop does
    not wash out the FP32 sweeps' rounding: velocity to relative L2 <= 1e-6,
    pressure to 5e-5."""
    case = cases.body_refined(4, 2, 2, n=8, length=(2.0, 1.0, 1.0), center=(0.5, 0.5, 0.5),
                              refine_radii=(0.35, 0.25), walls={1: abi.BC_FIX, 2: abi.BC_OP1})
    assert [int((case.level == lv).sum()) for lv in (1, 2, 3)] == [16, 64, 224]
    gmol = 0.4 / 300.0
    g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, gmol=gmol))
    o = oracle_lib.Oracle(case, _prm(abi.FORM_PLAIN, gmol=gmol))
    u, v, w, p = cases.taylor_green(case)
    one = np.ones(case.kk * case.jj)
    for s in (g, o):
        s.set_hierarchy(case.iparent, case.position)
        for gi in range(case.ngrid):
            if case.bctype[gi, 0] == abi.BC_FIX:
                s.set_buffer("U", gi + 1, 1, one)
        for nm, a in zip("UVWP", (1.0 + 0.1 * u, 0.1 * v, 0.1 * w, 0.01 * p)):
            s.set(nm, a)
        for lvl in (1, 2, 3):
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        prepare_levels(s, case)
    dt = 0.5 * float(case.ddx.min())
    hist = _run(case, (g, o), (gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")),
                dt, 3)
    assert np.all(np.abs(hist[:, 0] - hist[:, 1]) <= 1e-3 * hist[:, 1]), hist
    ev, ep = _errors(case, g, o)
    print(f"channel hierarchy: velocity {ev:.3e}, pressure {ep:.3e}")
    assert ev <= 1e-6, ev
    assert ep <= 5e-5, ep
    g.close()


def test_mixed_hierarchy_graph_matches_eager(gpu_lib):
    """On a hierarchy the captured stage graph (level loops, tstle4_par, the
    RK update of PAR grids, the level operators) gives the same bits as the
    stage issued kernel by kernel."""
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,))
    out = []
    for profile in (False, True):
        g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=6))
        u, v, w, p = cases.taylor_green(case)
        for nm, a in zip("UVWP", (u, v, w, p)):
            g.set(nm, a)
        g.set_hierarchy(case.iparent, case.position)
        for lvl in (1, 2):
            g.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        prepare_levels(g, case)
        g.profile(profile)
        rk = gpu_lib.rk_scheme("williamson")
        for irk in (1, 2, 3):
            g.timeintegrate_flow(1, 1, 0.0, 2e-3, irk, rk)
        out.append([g.get(nm) for nm in "UVWP"])
        g.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
