"""The plain form's performance build (MGLET_FORM_PLAIN_FMA): the flux and
Poisson kernels compiled with multiply-add contraction.  Each a*b + c is
rounded once instead of twice, so the fields are not the reference's bits
but stay within a relative 1e-12 of the FP64 oracle; the parity build
(MGLET_FORM_PLAIN) stays bit-exact."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_boundaries import face_plane_shape

pytestmark = pytest.mark.gpu


def _prm(form, **kw):
    base = dict(gmol=1.0 / 1600, epcorr=1e-10, nouter=40, ninner=5, nouter_min=0, form=form)
    base.update(kw)
    return abi.make_flow_params(**base)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _run(gpu_lib, oracle_lib, case, kw, steps, dt, shift=0.0, walls=False):
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u + shift, v, w), amplitude=1e-2, seed=42)
    gs = gpu_lib.Solver(case, _prm(abi.FORM_PLAIN_FMA, **kw))
    o = oracle_lib.Oracle(case, _prm(abi.FORM_PLAIN, **kw))
    rng = np.random.default_rng(17)
    bufs = {}
    if walls:
        for g in range(case.ngrid):
            for f in range(1, 7):
                if case.bctype[g, f - 1] == abi.BC_FIX:
                    bufs[(g, f)] = 0.5 + 0.01 * rng.standard_normal(face_plane_shape(case, f))
    for s in (gs, o):
        for nm, a in zip("UVWP", (u, v, w, p)):
            s.set(nm, a)
        for (g, f), b in bufs.items():
            s.set_buffer("U", g + 1, f, b)
        for g in range(case.ngrid):
            for f in range(1, 7):
                if case.bctype[g, f - 1] == abi.BC_OP1:
                    s.set_bc_real(g + 1, f, 0.05)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
        if walls:
            s.bound_flow()
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for it in range(1, steps + 1):
        for irk in (1, 2, 3):
            gs.timeintegrate_flow(it, it, 0.0, dt, irk, rkg)
            o.timeintegrate_flow(it, it, 0.0, dt, irk, rko)
    errs = {}
    for nm in "UVWP":
        a, b = case.interior(gs.get(nm)), case.interior(o.get(nm))
        if nm == "P":
            a, b = a - a.mean(), b - b.mean()
        errs[nm] = _rel(a, b)
    same = all(np.array_equal(gs.get(nm), o.get(nm)) for nm in "UVW")
    gs.close()
    return errs, same


@pytest.mark.parametrize("tiles,n,steps", [((1, 1, 1), 32, 10), ((3, 2, 2), 12, 4)])
def test_contracted_build_within_1e12(gpu_lib, oracle_lib, tiles, n, steps):
    """Taylor-Green with noise on periodic tilings: u, v, w and p (mean
    removed) within a relative 1e-12 of the oracle, and not the same bits
    (the contracted kernels are the ones that ran)."""
    case = cases.periodic_box(*tiles, n=n)
    errs, same = _run(gpu_lib, oracle_lib, case, {}, steps, 1e-3)
    print(f"plain FMA build {tiles} n={n}, {steps} steps: {errs}")
    assert not same
    for nm, e in errs.items():
        assert e <= 1e-12, (nm, e)


def test_contracted_build_with_walls(gpu_lib, oracle_lib):
    """FIX inflow, OP1 outflow, NOS and SLI walls on a stretched tiling."""
    walls = {1: abi.BC_FIX, 2: abi.BC_OP1, 3: abi.BC_NOS, 4: abi.BC_SLI}
    case = cases.stretch(cases.periodic_box(3, 2, 2, n=8, length=(2.0, 2.0, 1.0), walls=walls))
    errs, same = _run(gpu_lib, oracle_lib, case, dict(gmol=1e-3), 2, 2e-3, shift=0.5, walls=True)
    print(f"plain FMA build, walls: {errs}")
    assert not same
    for nm, e in errs.items():
        assert e <= 1e-12, (nm, e)
