"""Scalar transport on the GPU (plain FP64 form) against the oracle: RK
stages of two scalars interleaved with the flow stages, bit for bit on one
level and on a two-level hierarchy (PAR fluxes from the parent), and with
an LES model (within 1e-12 where the Kays/Crawford fit takes CUDA's exp)."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_levels import prepare_levels

pytestmark = pytest.mark.gpu


def _prm(**kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=6, ninner=5, nouter_min=6)
    base.update(kw)
    return abi.make_flow_params(**base)


def _run(gs, o, case, rk, les=0, kc=(0, 0), stages=3, levels=False):
    rng = np.random.default_rng(12)
    u, v, w, p = cases.taylor_green(case)
    f = dict(zip("UVWP", (u + 0.2, v, w, p)))
    t1 = 1.0 + 0.1 * rng.standard_normal(case.idim3d)
    t2 = rng.standard_normal(case.idim3d)
    for s in (gs, o):
        if levels:
            s.set_hierarchy(case.iparent, case.position)
        for n, a in f.items():
            s.set(n, a)
        s.set_scalars([0.71, 2.0], kayscrawford=list(kc), source=[0.0, 0.05], prturb=0.9)
        s.set("T1", t1)
        s.set("T2", t2)
        if levels:
            for lvl in (1, 2):
                s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", s2="T1", s3="T2", corners=True)
            prepare_levels(s, case)
        else:
            s.connect(0, 2, "U", "V", "W", "P", corners=True)
            s.connect(0, 2, s1="T1", s2="T2", corners=True)
        if les:
            s.set_lesmodel(les)
    for irk in range(1, stages + 1):
        for s in (gs, o):
            s.timeintegrate_scalar(5e-3, irk, rk)
            s.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)


def test_scalar_stages_bit_exact(gpu_lib, oracle_lib):
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0))
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    _run(gs, o, case, oracle_lib.rk_scheme("williamson"))
    for n in ("T1", "T2", "DT1", "DT2", "U", "P"):
        assert np.array_equal(gs.get(n), o.get(n)), n


def test_scalar_on_a_hierarchy_bit_exact(gpu_lib, oracle_lib):
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,))
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    _run(gs, o, case, oracle_lib.rk_scheme("williamson"), levels=True)
    for n in ("T1", "T2", "U"):
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("kc", [(0, 0), (1, 1)])
def test_scalar_with_les(gpu_lib, oracle_lib, kc):
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    prm = _prm(gmol=1e-4)
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    _run(gs, o, case, oracle_lib.rk_scheme("williamson"), les=1, kc=kc)
    for n in ("T1", "T2"):
        a, b = gs.get(n), o.get(n)
        if kc == (0, 0):
            assert np.array_equal(a, b), n
        else:
            assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), n


def test_buoyancy_and_coriolis_bit_exact(gpu_lib, oracle_lib):
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0))
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        s.set_scalars([0.71, 2.0])
    for s in (gs, o):
        s.set_buoyancy([0.3, -0.2, -9.81], 3e-3, iscalar=2)
        s.set_coriolis([0.1, -0.2, 0.25])
    _run(gs, o, case, oracle_lib.rk_scheme("williamson"))
    for n in ("T1", "T2", "U", "V", "W", "P"):
        assert np.array_equal(gs.get(n), o.get(n)), n


def _run_bc(gs, o, case, rk, les=0, gmol=1e-2):
    """Two scalars behind SIO faces (x, FIX inflow and OP1 outflow) and SWA
    walls (z, NOS), value and flux conditions mixed, random buffers."""
    rng = np.random.default_rng(21)
    u, v, w, p = cases.taylor_green(case)
    f = dict(zip("UVWP", (u + 1.0, v, w, p)))
    t1 = 1.0 + 0.1 * rng.standard_normal(case.idim3d)
    t2 = rng.standard_normal(case.idim3d)
    bc = {(1, 1): (2, [0, 1]), (2, 2): (2, [0, 0]),
          (1, 5): (1, [0, 1]), (2, 5): (1, [1, 0]), (1, 6): (1, [0, 0]), (2, 6): (1, [1, 1])}
    shape = {1: (case.kk, case.jj), 2: (case.kk, case.jj), 5: (case.jj, case.ii), 6: (case.jj, case.ii)}
    planes = {(g, fc, n): rng.uniform(-1, 2, shape[fc]) for (g, fc) in bc for n in ("T1", "T2")}
    inflow = np.ones((case.kk, case.jj))
    for s in (gs, o):
        for n, a in f.items():
            s.set(n, a)
        s.set_buffer("U", 1, 1, inflow)
        s.set_scalars([0.71, 2.0], source=[0.0, 0.05], prturb=0.9)
        s.set("T1", t1)
        s.set("T2", t2)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.connect(0, 2, s1="T1", s2="T2", corners=True)
        for (g, fc), (kind, types) in bc.items():
            s.set_scalar_bc(g, fc, kind, types)
        for (g, fc, n), a in planes.items():
            s.set_buffer(n, g, fc, a)
        if les:
            s.set_lesmodel(les)
    for irk in (1, 2, 3):
        for s in (gs, o):
            s.timeintegrate_scalar(5e-3, irk, rk)
            s.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)


_BC_WALLS = {1: abi.BC_FIX, 2: abi.BC_OP1, 5: abi.BC_NOS, 6: abi.BC_NOS}


def test_scalar_walls_and_inflow_bit_exact(gpu_lib, oracle_lib):
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0), walls=_BC_WALLS)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    _run_bc(gs, o, case, oracle_lib.rk_scheme("williamson"))
    for n in ("T1", "T2", "DT1", "DT2", "U", "P"):
        assert np.array_equal(gs.get(n), o.get(n)), n


def test_scalar_wall_model_with_les(gpu_lib, oracle_lib):
    """The wall model's turbulent branch (gmol 1e-4, speeds near 1) takes
    CUDA's pow: the scalars agree within 1e-12 of their range; the flow is
    bit for bit apart from what the scalars do not touch."""
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0), walls=_BC_WALLS)
    gs, o = gpu_lib.Solver(case, _prm(gmol=1e-4)), oracle_lib.Oracle(case, _prm(gmol=1e-4))
    _run_bc(gs, o, case, oracle_lib.rk_scheme("williamson"), les=1)
    for n in ("T1", "T2"):
        a, b = gs.get(n), o.get(n)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), n


def test_scalar_field_sources_bit_exact(gpu_lib, oracle_lib):
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0))
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    rng = np.random.default_rng(17)
    u, v, w, p = cases.taylor_green(case)
    t1, t2 = rng.standard_normal(case.idim3d), rng.standard_normal(case.idim3d)
    rk = oracle_lib.rk_scheme("williamson")
    for s in (gs, o):
        for n, a in zip("UVWP", (u, v, w, p)):
            s.set(n, a)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.set_scalars([0.71, 2.0], source=[0.05, 0.0])
        s.set("T1", t1)
        s.set("T2", t2)
        s.connect(0, 2, s1="T1", s2="T2", corners=True)
        s.add_scalar_source(1, -0.75, "T2")
        s.add_scalar_source(1, 0.01)
        s.add_scalar_source(2, 0.3, "P")
    for irk in (1, 2, 3):
        for s in (gs, o):
            s.timeintegrate_scalar(5e-3, irk, rk)
            s.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
    for n in ("T1", "T2", "DT1", "DT2"):
        assert np.array_equal(gs.get(n), o.get(n)), n
