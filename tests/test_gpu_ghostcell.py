"""Ghost-cell IB on the GPU (plain FP64 form) against the oracle, bit for
bit: the rebuilt Poisson coefficients, every list operation, and whole
stages with the ghost-cell sequence."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_ghostcell import gc_case, load, random_fields

pytestmark = pytest.mark.gpu


def _prm(form=abi.FORM_PLAIN, **kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=6, ninner=5, nouter_min=6, form=form)
    base.update(kw)
    return abi.make_flow_params(**base)


def _pair(gpu_lib, oracle_lib, fields, seed=7):
    case, bp, lists = gc_case(seed=seed)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        load(s, case, bp, lists, fields(case))
    return case, gs, o


def test_ghostcell_coefficients(gpu_lib, oracle_lib):
    case, gs, o = _pair(gpu_lib, oracle_lib, lambda c: random_fields(c, 1))
    for nm in ("GSAP", "SIPLW", "SIPLS", "SIPLB", "SIPLPR", "SIPUE", "SIPUN", "SIPUT", "SDIV"):
        assert np.array_equal(gs.get(nm), o.get(nm)), nm


@pytest.mark.parametrize("op", ["I", "R", "M", "X", "Y"])
def test_ghostcell_ops(gpu_lib, oracle_lib, op):
    case, gs, o = _pair(gpu_lib, oracle_lib, lambda c: random_fields(c, 2))
    for s in (gs, o):
        if op in "IRM":
            if op == "R":
                s.gc_mode("I")          # saves the lists' values ('S')
                s.set("U", np.ones(case.idim3d))
            s.gc_mode(op)
        else:
            s.setpointvalues(True)
            if op == "Y":
                s.set("U", np.full(case.idim3d, 2.0))
                s.setpointvalues(False)
    names = ("PWU", "PWV", "PWW") if op in "XY" else ("U", "V", "W", "P")
    for nm in names:
        assert np.array_equal(gs.get(nm), o.get(nm)), nm


def test_ghostcell_stages_bit_exact(gpu_lib, oracle_lib):
    """Two time steps (six stages): setibvalues on the first stage of each
    step, maskbp + getibvalues after the RK update, the ghost-cell divcal
    and bp projection, setpointvalues at the end of every stage."""
    def tg(case):
        u, v, w, p = cases.taylor_green(case)
        return dict(zip("UVWP", (u, v, w, p)))
    case, gs, o = _pair(gpu_lib, oracle_lib, tg)
    for s in (gs, o):
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.setpointvalues(True)
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for it in range(1, 3):
        for irk in range(1, 4):
            sg = gs.timeintegrate_flow(it, it, 0.0, 1e-2, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, 1e-2, irk, rko)
            assert sg.maxrhs == so.maxrhs
    for nm in ("U", "V", "W", "P", "PWU", "PWV", "PWW"):
        assert np.array_equal(gs.get(nm), o.get(nm)), nm


def test_mixed_form_refuses_ghostcell(gpu_lib):
    case = cases.periodic_box(2, 2, 2, n=8)
    s = gpu_lib.Solver(case, _prm(abi.FORM_MIXED))
    with pytest.raises(gpu_lib.MgletError) as e:
        s.set_ghostcell()
    assert e.value.code == abi.MGLET_ERR_UNSUPPORTED
