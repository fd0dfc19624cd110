"""Inter-level operators on the GPU (plain FP64 form) against the oracle, bit
for bit: parent, ftoc (every restriction kind), ctof, bound_pressure (with
and without BP), bound_flow on PAR faces (BP = 1 and with blocked cells),
tstle4 with tstle4_par, the multi-level pressure solve and the multi-level
RK stage, on the two-level hierarchies of cases.refined_box."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_levels import _buf_shape, _fine, _random_bp, prepare_levels

pytestmark = pytest.mark.gpu

HIERARCHIES = [
    dict(nx=2, ny=2, nz=2, n=8, refine=(1,)),
    dict(nx=3, ny=2, nz=2, n=12, refine=(1, 3)),
]


def _prm():
    return abi.make_flow_params(gmol=1e-2, epcorr=1e-12, nouter=4, ninner=2, nouter_min=0)


def _pair(gpu_lib, oracle_lib, h):
    case = cases.refined_box(h["nx"], h["ny"], h["nz"], n=h["n"], refine=h["refine"])
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        s.set_hierarchy(case.iparent, case.position)
    return case, gs, o


def _set(solvers, fields):
    for s in solvers:
        for n, a in fields.items():
            s.set(n, a)


@pytest.mark.parametrize("h", HIERARCHIES)
def test_ctof_and_ftoc(gpu_lib, oracle_lib, h):
    case, gs, o = _pair(gpu_lib, oracle_lib, h)
    rng = np.random.default_rng(11)
    _set((gs, o), {n: rng.standard_normal(case.idim3d) for n in ("HILF", "RES", "RHS", "U", "V", "W", "P")})
    for s in (gs, o):
        s.ctof(2, "HILF", "RES")
        s.ctof(1, "RES", "HILF")          # nothing on the coarsest level
    for n in ("HILF", "RES"):
        assert np.array_equal(gs.get(n), o.get(n)), n
    # sibling grids restrict a shared staggered face into the same coarse
    # face; connect makes their values equal, as in the reference's sequence
    for s in (gs, o):
        s.connect(2, 2, v1="U", v2="V", v3="W")
    for flag, ff, fc in (("R", "RHS", "RHS"), ("P", "HILF", "RES"), ("U", "U", "RES"), ("V", "V", "HILF"),
                         ("W", "W", "RHS")):
        for s in (gs, o):
            s.ftoc(2, ff, fc, flag)
        assert np.array_equal(gs.get(fc), o.get(fc)), flag
    for s in (gs, o):
        s.ftoc_multiple(2, v=("U", "V", "W"), s=("P",))
    for n in "UVWP":
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("h", HIERARCHIES)
@pytest.mark.parametrize("normal", [False, True])
def test_parent_buffers(gpu_lib, oracle_lib, h, normal):
    case, gs, o = _pair(gpu_lib, oracle_lib, h)
    rng = np.random.default_rng(12)
    _set((gs, o), {n: rng.standard_normal(case.idim3d) for n in ("U", "V", "W", "P", "DP")})
    for s in (gs, o):
        s.parent(2, v=("U", "V", "W"), s=("P", "DP"), normal=normal)
    n = 0
    for g in _fine(case):
        for iface in range(1, 7):
            if case.bctype[g, iface - 1] != abi.BC_PAR:
                continue
            for name in ("U", "V", "W", "P", "DP"):
                a = gs.get_buffer(name, g + 1, iface, _buf_shape(case, iface))
                b = o.get_buffer(name, g + 1, iface, _buf_shape(case, iface))
                assert np.array_equal(a, b), (g, iface, name)
                n += 1
    assert n > 0


@pytest.mark.parametrize("h", HIERARCHIES)
@pytest.mark.parametrize("withbp", [False, True])
def test_bound_pressure(gpu_lib, oracle_lib, h, withbp):
    case, gs, o = _pair(gpu_lib, oracle_lib, h)
    rng = np.random.default_rng(13)
    _set((gs, o), {"DP": rng.standard_normal(case.idim3d), "BP": _random_bp(case, 14)})
    for s in (gs, o):
        s.parent(2, s=("DP",))              # the parent's values into the DP buffers
        s.bound_pressure(2, "DP", with_bp=withbp)
    assert np.array_equal(gs.get("DP"), o.get("DP"))


@pytest.mark.parametrize("h", HIERARCHIES)
@pytest.mark.parametrize("blocked", [False, True])
def test_bound_flow_par(gpu_lib, oracle_lib, h, blocked):
    case, gs, o = _pair(gpu_lib, oracle_lib, h)
    rng = np.random.default_rng(15)
    bp = _random_bp(case, 16) if blocked else np.ones(case.idim3d)
    _set((gs, o), {**{n: rng.standard_normal(case.idim3d) for n in "UVWP"}, "BP": bp})
    for s in (gs, o):
        s.parent(2, v=("U", "V", "W"), s=("P",))
        s.bound_flow(2)
        s.bound_flow(1)                     # coarse level: CON faces only, nothing to do
    for n in "UVWP":
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("h", HIERARCHIES)
@pytest.mark.parametrize("psolver", [abi.PSOLVER_SIP, abi.PSOLVER_SOR])
def test_multilevel_mgpoisl_bit_exact(gpu_lib, oracle_lib, h, psolver):
    """The pressure solve over both levels, six outer iterations fixed, after
    the calls that precede it in the stage; every field bit for bit."""
    case = cases.refined_box(h["nx"], h["ny"], h["nz"], n=h["n"], refine=h["refine"])
    prm = abi.make_flow_params(gmol=1e-2, epcorr=1e-12, nouter=6, ninner=5, nouter_min=6,
                               psolver=psolver)
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    rng = np.random.default_rng(17)
    _set((gs, o), {n: rng.standard_normal(case.idim3d) for n in "UVWP"})
    for s in (gs, o):
        s.set_hierarchy(case.iparent, case.position)
        for lvl in (1, 2):
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        prepare_levels(s, case)
    sg, so = gs.mgpoisl(2e-3), o.mgpoisl(2e-3)
    assert (sg.ipc, sg.nouter_done) == (so.ipc, so.nouter_done) == (30, 6)
    assert sg.maxrhs == so.maxrhs
    for n in ("U", "V", "W", "P", "DP"):
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("h", HIERARCHIES)
def test_viscosity_on_par_faces(gpu_lib, oracle_lib, h):
    """G after set_hierarchy: the parent's values on the PAR ghost planes."""
    case, gs, o = _pair(gpu_lib, oracle_lib, h)
    assert np.array_equal(gs.get("G"), o.get("G"))


@pytest.mark.parametrize("h", HIERARCHIES)
def test_tstle4_par_bit_exact(gpu_lib, oracle_lib, h):
    """tstle4 with tstle4_par on every grid with PAR faces."""
    case, gs, o = _pair(gpu_lib, oracle_lib, h)
    rng = np.random.default_rng(18)
    _set((gs, o), {**{n: rng.standard_normal(case.idim3d) for n in "UVWP"},
                   "G": 1e-2 * (1.0 + rng.random(case.idim3d))})
    for s in (gs, o):
        s.tstle4()
    for n in ("UO", "VO", "WO"):
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("h", HIERARCHIES)
def test_multilevel_stage_bit_exact(gpu_lib, oracle_lib, h):
    """Three RK stages of timeintegrate_flow on the hierarchy, six outer
    iterations of the pressure solve fixed per stage; every field bit for
    bit."""
    from oracle.binding import rk_scheme
    case = cases.refined_box(h["nx"], h["ny"], h["nz"], n=h["n"], refine=h["refine"])
    prm = abi.make_flow_params(gmol=1e-2, epcorr=1e-12, nouter=6, ninner=5, nouter_min=6)
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    rng = np.random.default_rng(19)
    _set((gs, o), {**{n: rng.standard_normal(case.idim3d) for n in "UVW"},
                   "G": np.full(case.idim3d, 1e-2)})
    rk = rk_scheme("williamson")
    for s in (gs, o):
        s.set_hierarchy(case.iparent, case.position)
        for lvl in (1, 2):
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        prepare_levels(s, case)
    for irk in (1, 2, 3):
        sg = gs.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
        so = o.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
        assert (sg.ipc, sg.nouter_done, sg.maxrhs) == (so.ipc, so.nouter_done, so.maxrhs)
        for n in ("U", "V", "W", "P", "DU", "DV", "DW", "UO", "VO", "WO"):
            assert np.array_equal(gs.get(n), o.get(n)), (irk, n)


def test_mixed_form_refuses_sor_on_hierarchies(gpu_lib):
    """The mixed form's inner solver is SIP on every level: SOR on the finer
    levels (pressuresolver_mod.F90's psolver choice) is refused loudly."""
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,))
    prm = abi.make_flow_params(gmol=1e-2, epcorr=1e-12, nouter=4, ninner=2, nouter_min=0,
                               form=abi.FORM_MIXED, psolver=abi.PSOLVER_SOR)
    with pytest.raises(gpu_lib.MgletError) as e:
        gpu_lib.Solver(case, prm)
    assert e.value.code == abi.MGLET_ERR_UNSUPPORTED
