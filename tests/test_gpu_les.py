"""LES models on the GPU (plain FP64 form) against the oracle, bit for bit:
the effective viscosity of set_lesmodel (Smagorinsky, WALE; with the NOS
wall-model gradients), and whole stages with the LES update after the
pressure solve and the cross term of tstle4_diff, on periodic boxes, walls
and the ghost-cell IB (setginbody)."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_ghostcell import gc_case, load

pytestmark = pytest.mark.gpu


def _prm(**kw):
    base = dict(gmol=1e-4, epcorr=1e-12, nouter=6, ninner=5, nouter_min=6)
    base.update(kw)
    return abi.make_flow_params(**base)


def _fields(case, seed=3):
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u + 0.3, v, w), amplitude=5e-2, seed=seed)
    return dict(zip("UVWP", (u, v, w, p)))


CASES = {
    "periodic": lambda: cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0)),
    "walls": lambda: cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0),
                                        walls={5: abi.BC_NOS, 6: abi.BC_NOS, 3: abi.BC_SLI, 4: abi.BC_NOS}),
}


# gmol keeps the wall function of the NOS walls in its laminar branch
# (|u| < cpo6/dds); its turbulent branch raises to a real power with CUDA's
# pow, within 2 ulp of the C library's, which the last test covers
GMOL = {"periodic": 1e-4, "walls": 2e-2}


@pytest.mark.parametrize("model", [1, 2])
@pytest.mark.parametrize("name", list(CASES))
def test_les_viscosity_and_stages_bit_exact(gpu_lib, oracle_lib, model, name):
    case = CASES[name]()
    fields = _fields(case)
    prm = _prm(gmol=GMOL[name])
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    for s in (gs, o):
        for n, a in fields.items():
            s.set(n, a)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.set_lesmodel(model)
    assert np.array_equal(gs.get("G"), o.get("G"))
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        sg = gs.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
        so = o.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
        assert sg.maxrhs == so.maxrhs
    for n in ("U", "V", "W", "P", "G"):
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("model", [1, 2])
def test_les_with_ghostcells_bit_exact(gpu_lib, oracle_lib, model):
    case, bp, lists = gc_case()
    fields = _fields(case)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        load(s, case, bp, lists, fields)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.setpointvalues(True)
        s.set_lesmodel(model)
    assert np.array_equal(gs.get("G"), o.get("G"))
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        gs.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
        o.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
    for n in ("U", "V", "W", "P", "G"):
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("model", [1, 2])
def test_les_turbulent_walls(gpu_lib, oracle_lib, model):
    """NOS walls in the wall function's turbulent branch (gmol 1e-4): three
    stages agree with the oracle to a relative 1e-12."""
    case = CASES["walls"]()
    fields = _fields(case)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        for n, a in fields.items():
            s.set(n, a)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.set_lesmodel(model)
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        gs.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
        o.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
    for n in ("U", "V", "W", "P", "G"):
        a, b = gs.get(n), o.get(n)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), n


def test_mixed_form_refuses_les(gpu_lib):
    case = cases.periodic_box(2, 2, 2, n=8)
    s = gpu_lib.Solver(case, _prm(form=abi.FORM_MIXED, nouter_min=0))
    with pytest.raises(gpu_lib.MgletError):
        s.set_lesmodel(1)


def test_sigma_model(gpu_lib, oracle_lib):
    """The sigma model takes pow, acos and cos, CUDA's on the GPU and the C
    library's in the oracle: G and three stages agree to a relative 1e-10."""
    case = CASES["periodic"]()
    fields = _fields(case)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        for n, a in fields.items():
            s.set(n, a)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.set_lesmodel(5)
    a, b = gs.get("G"), o.get("G")
    assert np.abs(a - b).max() <= 1e-10 * np.abs(b - 1e-4).max()
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        gs.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
        o.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
    for n in ("U", "V", "W", "P"):
        a, b = gs.get(n), o.get(n)
        assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max(), n
