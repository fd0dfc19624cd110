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


def _converged(a, b):
    """Relative L2 of a - b over the interior (pressure: mean removed)."""
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("model", [1, 2, 5])
@pytest.mark.parametrize("name", list(CASES))
def test_mixed_form_with_les(gpu_lib, oracle_lib, model, name):
    """The batched mixed form with an LES model against the FP64 oracle: the
    LES kernel (FP64) sets G after every pressure solve, and the FP32 fluxes
    read the face viscosities of tstle4_diff from G at every point.  Two RK3
    steps with the outer loop converged on both sides: velocity to relative
    L2 <= 1e-7, pressure (mean removed) and G to 1e-5."""
    case = CASES[name]()
    fields = _fields(case)
    kw = dict(gmol=GMOL[name], epcorr=1e-11, nouter=40, nouter_min=0)
    gs = gpu_lib.Solver(case, _prm(form=abi.FORM_MIXED, **kw))
    o = oracle_lib.Oracle(case, _prm(**kw))
    for s in (gs, o):
        for n, a in fields.items():
            s.set(n, a)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.set_lesmodel(model)
    # sigma takes pow, acos and cos: CUDA's against the C library's
    eg0 = _converged(gs.get("G"), o.get("G"))
    print(f"G of set_lesmodel({model}) {name}: {eg0:.3e}")
    assert eg0 <= 1e-9, eg0
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for it in (1, 2):
        for irk in (1, 2, 3):
            sg = gs.timeintegrate_flow(it, it, 0.0, 5e-3, irk, rkg)
            o.timeintegrate_flow(it, it, 0.0, 5e-3, irk, rko)
            assert np.isfinite(sg.maxrhs)
    iv = [case.interior(gs.get(n)) for n in "UVW"]
    ov = [case.interior(o.get(n)) for n in "UVW"]
    ev = float(np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(iv, ov)) / sum(np.sum(b ** 2) for b in ov)))
    pg, po = case.interior(gs.get("P")), case.interior(o.get("P"))
    ep = _converged(pg - pg.mean(), po - po.mean())
    eg = _converged(case.interior(gs.get("G")), case.interior(o.get("G")))
    print(f"mixed LES model {model} {name}: velocity {ev:.3e}, pressure {ep:.3e}, G {eg:.3e}")
    assert ev <= 1e-7, ev
    assert ep <= 1e-5, ep
    assert eg <= 1e-5, eg
    gs.close()


def test_mixed_form_with_a_viscosity_field(gpu_lib, oracle_lib):
    """A G field set by the caller (no LES model) in the mixed form: the
    fluxes read it at every point; against the FP64 oracle as above."""
    case = CASES["periodic"]()
    fields = _fields(case)
    rng = np.random.default_rng(5)
    fields["G"] = 1e-3 * (1.0 + 0.5 * rng.random(case.idim3d))
    kw = dict(gmol=1e-3, epcorr=1e-11, nouter=40, nouter_min=0)
    gs = gpu_lib.Solver(case, _prm(form=abi.FORM_MIXED, **kw))
    o = oracle_lib.Oracle(case, _prm(**kw))
    for s in (gs, o):
        for n, a in fields.items():
            s.set(n, a)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.connect(0, 2, s1="G", corners=True)
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        gs.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rkg)
        o.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rko)
    iv = [case.interior(gs.get(n)) for n in "UVW"]
    ov = [case.interior(o.get(n)) for n in "UVW"]
    ev = float(np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(iv, ov)) / sum(np.sum(b ** 2) for b in ov)))
    print(f"mixed, caller-set G: velocity {ev:.3e}")
    assert ev <= 1e-7, ev
    gs.close()
