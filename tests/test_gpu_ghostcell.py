"""Ghost-cell IB on the GPU against the oracle: in the plain FP64 form bit
for bit (the rebuilt Poisson coefficients, every list operation, whole
stages with the ghost-cell sequence), in the batched mixed form whole
stages within stated tolerances."""
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


def _chained(case, lists):
    """The synthetic lists with three cells appended to the first grid's u
    list that depend on each other and on the list: cell A writes a, reading
    b and the first cell's ghost value; cell B writes c, reading a (after A);
    cell C writes b (after A read it).  The level-parallel walk must give the
    values of the ordered walk."""
    kk, jj = case.kk, case.jj
    flat = lambda i, j, k: (k - 1) + (j - 1) * kk + (i - 1) * kk * jj + 1
    n, xi, xr, xv = lists[0][1]
    first = int(xi[0])
    a, b, cc = flat(4, 4, 4), flat(4, 5, 4), flat(5, 4, 4)
    xi2 = list(xi) + [a, 2, b, first] + [cc, 1, a] + [b, 1, flat(5, 5, 5)]
    xr2 = list(xr) + [0.5, 0.25, 0.1] + [0.7, -0.2] + [0.3, 0.05]
    xv2 = list(xv) + [0.4, 0.3, 0.0] + [0.6, 0.0] + [0.2, 0.0]
    out = [dict(gl) for gl in lists]
    out[0][1] = (n + 3, np.array(xi2, dtype=np.int64), np.array(xr2), np.array(xv2))
    return out


@pytest.mark.parametrize("op", ["I", "X"])
def test_ghostcell_dependent_cells_bit_exact(gpu_lib, oracle_lib, op):
    """Cells of one list that read values earlier cells write (and write
    values earlier cells read) come out as the reference's ordered walk
    gives them, bit for bit, in setibvalues and setpointvalues."""
    case, bp, lists = gc_case(seed=7)
    lists = _chained(case, lists)
    fields = random_fields(case, 5)
    gs, o = gpu_lib.Solver(case, _prm()), oracle_lib.Oracle(case, _prm())
    for s in (gs, o):
        load(s, case, bp, lists, fields)
        if op == "I":
            s.gc_mode("I")
        else:
            s.setpointvalues(True)
    names = ("U", "V", "W") if op == "I" else ("PWU", "PWV", "PWW")
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


def test_mixed_ghostcell_stages(gpu_lib, oracle_lib):
    """The batched mixed form with the ghost-cell IB against the FP64
    oracle: the stage sequence of test_ghostcell_stages_bit_exact with the
    outer loop run to convergence (epcorr 1e-10, at most 40 outer
    iterations) on both sides.  The grids next to the body take the FP64
    fluxes of the point values, the Poisson couplings BP closes are masked in
    the FP32 sweeps' records and the float-float outer step; velocity to
    relative L2 <= 1e-7, pressure (mean removed) to 1e-5."""
    case, bp, lists = gc_case(seed=7)
    u, v, w, p = cases.taylor_green(case)
    fields = dict(zip("UVWP", (u, v, w, p)))
    kw = dict(epcorr=1e-10, nouter=40, nouter_min=0)
    gs = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, **kw))
    o = oracle_lib.Oracle(case, _prm(**kw))
    for s in (gs, o):
        load(s, case, bp, lists, fields)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        s.setpointvalues(True)
    assert "uniform classes: no" in gs.tuning()
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for it in range(1, 3):
        for irk in range(1, 4):
            sg = gs.timeintegrate_flow(it, it, 0.0, 1e-2, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, 1e-2, irk, rko)
            assert np.isfinite(sg.maxrhs)
    num = sum(np.sum((case.interior(gs.get(n)) - case.interior(o.get(n))) ** 2) for n in "UVW")
    den = sum(np.sum(case.interior(o.get(n)) ** 2) for n in "UVW")
    ev = float(np.sqrt(num / den))
    pg, po = case.interior(gs.get("P")), case.interior(o.get("P"))
    pg, po = pg - pg.mean(), po - po.mean()
    ep = float(np.linalg.norm(pg - po) / np.linalg.norm(po))
    print(f"mixed ghost-cell: velocity {ev:.3e}, pressure {ep:.3e}")
    assert ev <= 1e-7, ev
    assert ep <= 1e-5, ep
    gs.close()
