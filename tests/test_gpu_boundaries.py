"""FIX / OP1 / NOS / SLI faces on the GPU against the oracle: in the plain
FP64 form bound_flow alone and whole stages bit for bit, tstle4 with the
Werner-Wengle wall function of NOS walls (bit for bit in its laminar branch,
to CUDA's pow in the turbulent one); in the batched mixed form whole stages
within stated tolerances."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_boundaries import face_plane_shape, random_bc_case

pytestmark = pytest.mark.gpu

WALLS = [
    {1: abi.BC_FIX, 2: abi.BC_OP1},
    {3: abi.BC_OP1, 4: abi.BC_FIX, 5: abi.BC_NOS, 6: abi.BC_SLI},
    {1: abi.BC_SLI, 2: abi.BC_NOS, 5: abi.BC_OP1, 6: abi.BC_OP1},
    {5: abi.BC_FIX, 6: abi.BC_FIX, 3: abi.BC_NOS, 4: abi.BC_SLI},
]


def _prm(form=abi.FORM_PLAIN, **kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=6, ninner=5, nouter_min=6, form=form)
    base.update(kw)
    return abi.make_flow_params(**base)


def _load(solvers, case, fields, bufs, pinf):
    for s in solvers:
        for nm, a in fields.items():
            s.set(nm, a)
        for (nm, g, f), b in bufs.items():
            s.set_buffer(nm, g + 1, f, b)
        for (g, f), val in pinf.items():
            s.set_bc_real(g + 1, f, val)


@pytest.mark.parametrize("walls", WALLS)
def test_bound_flow_bit_exact(gpu_lib, oracle_lib, walls):
    case, fields, bufs = random_bc_case(walls, seed=len(walls) * 11 + 3)
    pinf = {(g, f): 0.1 * (g + f) for (nm, g, f) in bufs if case.bctype[g, f - 1] == abi.BC_OP1}
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    _load((gs, o), case, fields, bufs, pinf)
    gs.bound_flow()
    o.bound_flow()
    for nm in "UVWP":
        assert np.array_equal(gs.get(nm), o.get(nm)), nm


@pytest.mark.parametrize("walls", WALLS)
def test_wall_stages_bit_exact(gpu_lib, oracle_lib, walls):
    """Two time steps (six stages) with the pressure solve, bound_flow before
    it and after the projection, on a 2x2x1 tiling."""
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0), walls=walls)
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u + 0.5, v, w), amplitude=1e-2, seed=9)
    fields = dict(zip("UVWP", (u, v, w, p)))
    rng = np.random.default_rng(17)
    bufs, pinf = {}, {}
    for g in range(case.ngrid):
        for f in range(1, 7):
            t = case.bctype[g, f - 1]
            if t == abi.BC_FIX:
                bufs[("U", g, f)] = 0.5 + 0.01 * rng.standard_normal(face_plane_shape(case, f))
            if t == abi.BC_OP1:
                pinf[(g, f)] = 0.05
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    _load((gs, o), case, fields, bufs, pinf)
    for s in (gs, o):
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for it in range(1, 3):
        for irk in range(1, 4):
            sg = gs.timeintegrate_flow(it, it, 0.0, 2e-3, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, 2e-3, irk, rko)
            assert sg.ipc == so.ipc and sg.maxrhs == so.maxrhs
    for nm in "UVWP":
        assert np.array_equal(gs.get(nm), o.get(nm)), nm


@pytest.mark.parametrize("gmol,amplitude", [(1e-2, 0.3), (1e-3, 1.0), (1e-5, 1.0)])
def test_wall_function_tstle4(gpu_lib, oracle_lib, gmol, amplitude):
    """tstle4 with the Werner-Wengle wall function on six NOS walls.  In the
    laminar sublayer (gmol 1e-2) the result is bit for bit the oracle's; the
    turbulent branch raises a base to the power 2/(1+1/7) with CUDA's pow
    (at most 2 ulp from the correctly rounded value) where the oracle uses
    the C library's, so there each wall term agrees to a relative 1e-15 and
    every other point bit for bit."""
    from test_oracle_wallfunction import ww_constants, wall_case, wall_fields, wall_terms
    case = wall_case()
    prm = abi.make_flow_params(gmol=gmol, epcorr=1e-12, nouter=4, ninner=2, nouter_min=0)
    fields = wall_fields(case, amplitude, 33, gmol)
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    _load((gs, o), case, fields, {}, {})
    gs.tstle4()
    o.tstle4()
    _, M, nturb, _ = wall_terms(case, ww_constants(gmol, 1.0), fields["U"], fields["V"], fields["W"])
    for nm in ("UO", "VO", "WO"):
        a, b = gs.get(nm), o.get(nm)
        m = M[nm[0]]
        assert np.array_equal(a[~m], b[~m]), nm
        if nturb == 0:
            assert np.array_equal(a, b), nm
        else:
            assert np.abs(a[m] - b[m]).max() <= 1e-14 * np.abs(b).max(), nm


def test_turbulent_wall_stage(gpu_lib, oracle_lib):
    """Three stages with NOS walls in the wall function's turbulent branch
    (gmol 1e-5), the pressure solve's six outer iterations fixed: the fields
    follow the oracle's to a relative 1e-12 (the pow difference above,
    carried through the solve)."""
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0), walls={5: abi.BC_NOS, 6: abi.BC_NOS})
    u, v, w, p = cases.taylor_green(case)
    fields = dict(zip("UVWP", (u + 0.5, v, w, p)))
    prm = _prm(gmol=1e-5)
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    _load((gs, o), case, fields, {}, {})
    for s in (gs, o):
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for irk in range(1, 4):
        gs.timeintegrate_flow(1, 1, 0.0, 2e-3, irk, rkg)
        o.timeintegrate_flow(1, 1, 0.0, 2e-3, irk, rko)
    for nm in "UVWP":
        a, b = gs.get(nm), o.get(nm)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), nm


@pytest.mark.parametrize("walls", WALLS)
def test_viscosity_field_at_start(gpu_lib, oracle_lib, walls):
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0), walls=walls)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    assert np.array_equal(gs.get("G"), o.get("G"))


MIXED_WALLS = [
    {1: abi.BC_FIX, 2: abi.BC_OP1},
    {5: abi.BC_FIX, 6: abi.BC_FIX, 3: abi.BC_NOS, 4: abi.BC_SLI},
    {1: abi.BC_SLI, 2: abi.BC_NOS, 5: abi.BC_NOS, 6: abi.BC_OP1},
    {3: abi.BC_NOS, 4: abi.BC_NOS},
]


@pytest.mark.parametrize("walls", MIXED_WALLS)
def test_mixed_form_with_walls(gpu_lib, oracle_lib, walls):
    """The batched mixed form on grids with FIX, OP1, NOS and SLI faces
    against the FP64 oracle: two RK3 steps with the outer loop run to
    convergence (epcorr 1e-11, at most 40 outer iterations) on both sides.
    The velocity vector agrees to relative L2 <= 1e-7, the pressure (mean
    removed) to 1e-5: FP32 fluxes and SIP sweeps under the float-float
    outer loop.  With gmol = 1e-3 and u = 0.5 + Taylor-Green the NOS walls'
    wall function runs in both of its branches."""
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0), walls=walls)
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u + 0.5, v, w), amplitude=1e-2, seed=9)
    fields = dict(zip("UVWP", (u, v, w, p)))
    rng = np.random.default_rng(17)
    bufs, pinf = {}, {}
    for g in range(case.ngrid):
        for f in range(1, 7):
            t = case.bctype[g, f - 1]
            if t == abi.BC_FIX:
                bufs[("U", g, f)] = 0.5 + 0.01 * rng.standard_normal(face_plane_shape(case, f))
            if t == abi.BC_OP1:
                pinf[(g, f)] = 0.05
    kw = dict(gmol=1e-3, epcorr=1e-11, nouter=40, nouter_min=0)
    gs = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, **kw))
    o = oracle_lib.Oracle(case, _prm(**kw))
    _load((gs, o), case, fields, bufs, pinf)
    for s in (gs, o):
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.bound_flow()
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for it in range(1, 3):
        for irk in range(1, 4):
            sg = gs.timeintegrate_flow(it, it, 0.0, 2e-3, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, 2e-3, irk, rko)
            assert np.isfinite(sg.maxrhs)
            assert sg.maxrhs / sg.prefak < 1e-11 or sg.nouter_done == 40
    num = sum(np.sum((case.interior(gs.get(n)) - case.interior(o.get(n))) ** 2) for n in "UVW")
    den = sum(np.sum(case.interior(o.get(n)) ** 2) for n in "UVW")
    ev = float(np.sqrt(num / den))
    pg, po = case.interior(gs.get("P")), case.interior(o.get("P"))
    pg, po = pg - pg.mean(), po - po.mean()
    ep = float(np.linalg.norm(pg - po) / np.linalg.norm(po))
    print(f"walls {walls}: velocity {ev:.3e}, pressure {ep:.3e}")
    assert ev <= 1e-7, ev
    assert ep <= 1e-5, ep
    ig, io = gs.itinfo(2e-3), o.itinfo(2e-3)
    assert abs(ig.cflmax - io.cflmax) <= 1e-6 * io.cflmax
    gs.close()


def test_mixed_form_refuses_low_outflow(gpu_lib):
    """tstle4 extends the flux range of an outflow face on a low side (1, 3,
    5) over the ghost plane, which the mixed form's interior sweep does not
    visit: such a case is refused loudly, not run approximately."""
    case = cases.periodic_box(2, 1, 1, n=8, walls={1: abi.BC_OP1, 2: abi.BC_FIX})
    with pytest.raises(gpu_lib.MgletError) as e:
        gpu_lib.Solver(case, _prm(abi.FORM_MIXED))
    assert e.value.code == abi.MGLET_ERR_UNSUPPORTED
