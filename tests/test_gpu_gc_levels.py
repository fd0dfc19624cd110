"""Grid hierarchies with the ghost-cell IB on the GPU (plain FP64 form)
against the oracle, bit for bit: the BP-weighted restrictions, par_ftoc_norm,
the multi-level setibvalues / setpointvalues / setsdivfield schedules and
whole multi-level ghost-cell stages."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_gc_levels import gc_hierarchy, load_gc
from test_oracle_levels import _fine, _g3, prepare_levels

pytestmark = pytest.mark.gpu

OCTANTS = [None, [(0, 0, 0)], [(1, 1, 1)], [(1, 0, 1)]]


def _prm(**kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=4, ninner=2, nouter_min=0)
    base.update(kw)
    return abi.make_flow_params(**base)


def _pair(gpu_lib, oracle_lib, octants=None, body=True, prm=None, fields=None):
    case, bp, lists = gc_hierarchy(octants=octants, body=body)
    prm = prm or _prm()
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    for s in (gs, o):
        load_gc(s, case, bp, lists, fields)
    return case, bp, gs, o


@pytest.mark.parametrize("flag", ["P", "R", "S"])
def test_gc_ftoc(gpu_lib, oracle_lib, flag):
    """The scalar restrictions (U, V, W are the no-IB means, checked with the
    other level operators)."""
    case, bp, lists = gc_hierarchy()
    bp = bp.copy()
    rng = np.random.default_rng(3)
    bp[rng.random(case.idim3d) < 0.3] = 0.0
    for g in _fine(case):
        _g3(case, bp, g)[2:4, 2:4, 2:4] = 0.0
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    ff, fc = rng.standard_normal(case.idim3d), rng.standard_normal(case.idim3d)
    for s in (gs, o):
        load_gc(s, case, bp, lists, {"RHS": ff, "RES": fc})
        s.ftoc(2, "RHS", "RES", flag)
    assert np.array_equal(gs.get("RES"), o.get("RES"))


def test_gc_t_restriction_is_refused(gpu_lib):
    case, bp, lists = gc_hierarchy()
    gs = gpu_lib.Solver(case, _prm())
    load_gc(gs, case, bp, lists)
    with pytest.raises(gpu_lib.MgletError):
        gs.ftoc(2, "RHS", "RES", "T")


@pytest.mark.parametrize("octants", OCTANTS)
@pytest.mark.parametrize("use_sum", [False, True])
def test_par_ftoc_norm(gpu_lib, oracle_lib, octants, use_sum):
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,), octants=octants)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    rng = np.random.default_rng(4)
    f = {n: rng.standard_normal(case.idim3d) for n in "UVW"}
    for s in (gs, o):
        s.set_hierarchy(case.iparent, case.position)
        for n, a in f.items():
            s.set(n, a)
        s.par_ftoc_norm(2, sum=use_sum)
    for n in "UVW":
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("octants", OCTANTS[:2])
def test_multilevel_setibvalues_and_setpointvalues(gpu_lib, oracle_lib, octants):
    rng = np.random.default_rng(7)
    case, _, _ = gc_hierarchy(octants=octants)
    fields = {n: rng.standard_normal(case.idim3d) for n in "UVWP"}
    case, bp, gs, o = _pair(gpu_lib, oracle_lib, octants=octants, fields=fields)
    for s in (gs, o):
        assert np.array_equal(gs.get("SDIV"), o.get("SDIV"))
        s.setpointvalues(True)
    for n in ("PWU", "PWV", "PWW"):
        assert np.array_equal(gs.get(n), o.get(n)), n
    for s in (gs, o):
        s.gc_mode("I")
    for n in "UVW":
        assert np.array_equal(gs.get(n), o.get(n)), n
    for s in (gs, o):
        s.setpointvalues(False)
        s.gc_mode("R")
    for n in ("U", "V", "W", "PWU", "PWV", "PWW"):
        assert np.array_equal(gs.get(n), o.get(n)), n


def test_restore_before_save_is_refused(gpu_lib):
    case, bp, lists = gc_hierarchy()
    gs = gpu_lib.Solver(case, _prm())
    load_gc(gs, case, bp, lists)
    with pytest.raises(gpu_lib.MgletError):
        gs.gc_mode("R")
    with pytest.raises(gpu_lib.MgletError):
        gs.setpointvalues(False)


@pytest.mark.parametrize("octants", OCTANTS[:2])
@pytest.mark.parametrize("body", [False, True])
def test_multilevel_ghostcell_stages_bit_exact(gpu_lib, oracle_lib, octants, body):
    """Three RK stages with the multi-level ghost-cell schedule, six outer
    iterations of the pressure solve fixed; every field bit for bit."""
    from oracle.binding import rk_scheme
    rng = np.random.default_rng(8)
    case, _, _ = gc_hierarchy(octants=octants, body=body)
    fields = {n: 0.1 * rng.standard_normal(case.idim3d) for n in "UVW"}
    fields["U"] = fields["U"] + 1.0
    prm = _prm(nouter=6, ninner=5, nouter_min=6)
    case, bp, gs, o = _pair(gpu_lib, oracle_lib, octants=octants, body=body, prm=prm, fields=fields)
    for s in (gs, o):
        for lvl in (1, 2):
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        prepare_levels(s, case)
        s.setpointvalues(True)
    rk = rk_scheme("williamson")
    for irk in (1, 2, 3):
        sg = gs.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
        so = o.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
        assert (sg.ipc, sg.nouter_done, sg.maxrhs) == (so.ipc, so.nouter_done, so.maxrhs)
        for n in ("U", "V", "W", "P", "PWU", "PWV", "PWW"):
            assert np.array_equal(gs.get(n), o.get(n)), (irk, n)
