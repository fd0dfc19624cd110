"""The sphere-in-channel configuration (multi-level, ghost-cell immersed
boundary built from the sphere's signed distance) on the GPU, plain FP64
form, against the oracle bit for bit: a bounded sample of the full case --
4 x 2 x 2 level-1 grids of 8^3 cells, two refinement levels around a sphere
of 0.4 (16 + 64 + 224 grids), FIX inflow u = 1, OP1 outflow, periodic in y
and z -- for three RK3 time steps with the outer pressure iterations
fixed.  Both sides consume the same geometry and the same lists from
mglet_create_flowstencils."""
import numpy as np
import pytest

from mglet_gb300 import abi, channel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sample():
    return channel.SphereChannel(tiles=(4, 2, 2), n=8, grid_size=0.5, diameter=0.4,
                                 refine_radii=(0.35, 0.25))


def test_sphere_channel_steps_bit_exact(gpu_lib, oracle_lib, sample):
    case = sample.case
    assert [int((case.level == lv).sum()) for lv in (1, 2, 3)] == [16, 64, 224]
    prm = sample.flow_params(nouter=6, ninner=5, nouter_min=6)
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    for s in (gs, o):
        sample.setup(s)
    for n in ("U", "V", "W", "P", "PWU", "PWV", "PWW", "SDIV"):
        assert np.array_equal(gs.get(n), o.get(n)), n
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    dt = sample.dt()
    for it in range(1, 4):
        for irk in (1, 2, 3):
            sg = gs.timeintegrate_flow(it, it, 0.0, dt, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, dt, irk, rko)
            assert (sg.ipc, sg.maxrhs) == (so.ipc, so.maxrhs), (it, irk)
            assert np.isfinite(sg.maxrhs)
        for n in ("U", "V", "W", "P", "PWU", "PWV", "PWW"):
            assert np.array_equal(gs.get(n), o.get(n)), (it, n)
    ig, io = gs.itinfo(dt), o.itinfo(dt)
    assert ig.cflmax == io.cflmax and ig.divmax == io.divmax
    # an impulsive start: the flow speeds up around the sphere (up to 1.5 U
    # in potential flow), so the CFL number rises above the 0.5 of the
    # inflow; it stays finite and below 1.5
    assert not ig.exploded and 0.0 < ig.cflmax < 1.5
    gs.close()


def test_sphere_channel_mixed_against_oracle(gpu_lib, oracle_lib, sample):
    """The same bounded sample in the batched mixed form (hierarchy, FIX /
    OP1 faces and the ghost-cell IB together) against the oracle, three RK3
    steps with six outer iterations per stage on both sides.  The relative
    residual of every stage agrees to 1e-3; the velocity to relative L2
    <= 3e-5 and the pressure (mean removed) to 1e-4.  These are wider than
    on one level (1e-7): with six outer iterations the multi-level outer
    loop leaves relative residuals of order one, so the FP32 rounding of the
    sweeps and fluxes stays in the correction, and this flow amplifies small
    differences on the finest level (the FP64 form itself, started from a
    state perturbed by 2^-24, drifts by a growing amount too)."""
    case = sample.case
    kw = dict(nouter=6, ninner=5, nouter_min=6)
    gs = gpu_lib.Solver(case, sample.flow_params(abi.FORM_MIXED, **kw))
    o = oracle_lib.Oracle(case, sample.flow_params(**kw))
    for s in (gs, o):
        sample.setup(s)
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    dt = sample.dt()
    for it in range(1, 4):
        for irk in (1, 2, 3):
            sg = gs.timeintegrate_flow(it, it, 0.0, dt, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, dt, irk, rko)
            assert np.isfinite(sg.maxrhs)
            assert abs(sg.maxrhs / sg.prefak - so.maxrhs / so.prefak) <= 1e-3 * so.maxrhs / so.prefak, \
                (it, irk, sg.maxrhs, so.maxrhs)
    num = sum(np.sum((case.interior(gs.get(n)) - case.interior(o.get(n))) ** 2) for n in "UVW")
    den = sum(np.sum(case.interior(o.get(n)) ** 2) for n in "UVW")
    ev = float(np.sqrt(num / den))
    pg, po = case.interior(gs.get("P")), case.interior(o.get("P"))
    pg, po = pg - pg.mean(), po - po.mean()
    ep = float(np.linalg.norm(pg - po) / np.linalg.norm(po))
    print(f"mixed sphere sample: velocity {ev:.3e}, pressure {ep:.3e}")
    assert ev <= 3e-5, ev
    assert ep <= 1e-4, ep
    gs.close()
