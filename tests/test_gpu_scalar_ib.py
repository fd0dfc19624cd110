"""The ghost-cell IB of the scalars on the GPU (plain FP64 form) against the
oracle, bit for bit: BT from BP (blockbt, also behind PAR faces on a
hierarchy), and scalar stages with the bodies' flux and value conditions
(set_scastencils "P" on QTT and T, maskbt; timeintegrate_scalar_mod.F90:
71-90) interleaved with the flow stages of the ghost-cell case."""
import numpy as np
import pytest

from mglet_gb300 import cases
from test_oracle_ghostcell import gc_case
from test_oracle_levels import prepare_levels
from test_oracle_scalar_ib import GEO, _prm, sca_lists, scalar_ib_setup

pytestmark = pytest.mark.gpu


def test_scalar_ghostcell_stages_bit_exact(gpu_lib, oracle_lib):
    case, bp, lists = gc_case(seed=7)
    u, v, w, p = cases.taylor_green(case)
    fields = dict(zip("UVWP", (u + 0.2, v, w, p)))
    t1 = 1.0 + 0.1 * np.random.default_rng(5).standard_normal(case.idim3d)
    scal, _ = sca_lists(case, bp)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        scalar_ib_setup(s, case, bp, lists, fields, scal, GEO, t1)
    assert np.array_equal(gs.get("BT"), o.get("BT"))
    assert np.any(gs.get("BT") != 1.0)
    rk = oracle_lib.rk_scheme("williamson")
    for it in (1, 2):
        for irk in (1, 2, 3):
            for s in (gs, o):
                s.timeintegrate_scalar(5e-3, irk, rk)
                s.timeintegrate_flow(it, it, 0.0, 5e-3, irk, rk)
    for n in ("T1", "T2", "DT1", "DT2", "U", "V", "W", "P"):
        assert np.array_equal(gs.get(n), o.get(n)), n
    gs.close()


def test_scalar_ghostcell_on_a_hierarchy_bit_exact(gpu_lib, oracle_lib):
    """A two-level hierarchy with blocked cells: BT from BP with the cells
    behind the PAR faces opened from the coarse BT, and one scalar stage
    whose fine-to-coarse restriction of T weighs by BT."""
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,))
    rng = np.random.default_rng(9)
    # the lower half (k <= 6, ghosts included) of every fine grid blocked:
    # BT closes its inside and blockbt reopens the cells behind the PAR
    # faces, where the coarse grid is open
    bp = np.ones(case.idim3d)
    for g in range(case.ngrid):
        if case.iparent[g] != 0:
            case.view(bp)[g, :, :, :6] = 0.0
    u, v, w, p = cases.taylor_green(case)
    t1 = 1.0 + 0.1 * rng.standard_normal(case.idim3d)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        s.set_hierarchy(case.iparent, case.position)
        for nm, a in zip("UVWP", (u + 0.2, v, w, p)):
            s.set(nm, a)
        s.set("BP", bp)
        for lvl in (1, 2):
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        prepare_levels(s, case)
        s.set_ghostcell()
        s.set_scalars([0.71])
        s.set("T1", t1)
        for lvl in (1, 2):
            s.connect(lvl, 2, s1="T1", corners=True)
    bt = o.get("BT")
    assert np.any(bt == 0.0)
    assert np.array_equal(gs.get("BT"), bt)
    rk = oracle_lib.rk_scheme("williamson")
    for s in (gs, o):
        s.timeintegrate_scalar(5e-3, 1, rk)
    for n in ("T1", "DT1"):
        assert np.array_equal(gs.get(n), o.get(n)), n
    gs.close()


def test_scalar_body_without_condition_is_refused(gpu_lib):
    case, bp, lists = gc_case(seed=7)
    u, v, w, p = cases.taylor_green(case)
    scal, _ = sca_lists(case, bp)
    g = gpu_lib.Solver(case, _prm())
    scalar_ib_setup(g, case, bp, lists, dict(zip("UVWP", (u, v, w, p))), scal,
                    [([0], [1.0]), ([1, 0], [0.2, -0.3])], np.ones(case.idim3d))
    with pytest.raises(gpu_lib.MgletError):
        g.timeintegrate_scalar(5e-3, 1, gpu_lib.rk_scheme("williamson"))
    g.close()


def test_constructed_scalar_lists_on_the_sphere_bit_exact(gpu_lib, oracle_lib):
    """The lists of mglet_create_scastencils on the two-level sphere case
    (synthetic cut-cell areas and body ids): one scalar stage and one flow
    stage on the GPU and on the oracle, bit for bit."""
    from mglet_gb300 import channel
    sc = channel.SphereChannel(tiles=(4, 2, 2), n=8, grid_size=0.5, diameter=0.4, refine_radii=(0.35,))
    ncut = int(sc.geo["icells"].sum())
    area = 0.05 + np.random.default_rng(4).random(ncut)
    body = (1 + np.arange(ncut) % 2).astype(np.int32)
    scal = gpu_lib.create_scastencils(sc.case, sc.geo, area, body)
    prm = sc.flow_params(nouter=6, ninner=5, nouter_min=6)
    gs, o = gpu_lib.Solver(sc.case, prm), oracle_lib.Oracle(sc.case, prm)
    t1 = 1.0 + 0.1 * np.random.default_rng(6).standard_normal(sc.case.idim3d)
    for s in (gs, o):
        sc.setup(s)
        s.set_scalars([0.71])
        s.set("T1", t1)
        for lvl in (1, 2):
            s.connect(lvl, 2, s1="T1", corners=True)
        for g, (xi, xr, xv) in enumerate(scal):
            s.set_scastencils(g + 1, xi, xr, xv)
        s.set_scalar_geometry(1, [0, 1], [2.0, 0.5])
    rk = oracle_lib.rk_scheme("williamson")
    for s in (gs, o):
        s.timeintegrate_scalar(sc.dt(), 1, rk)
        s.timeintegrate_flow(1, 1, 0.0, sc.dt(), 1, rk)
    for n in ("BT", "T1", "DT1", "U", "P"):
        assert np.array_equal(gs.get(n), o.get(n)), n
    gs.close()
