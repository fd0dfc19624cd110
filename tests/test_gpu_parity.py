"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Tolerance: relative L2 <= 1e-12 on every FP64 field of the plain form (the
bar of the FP64 form); the plain kernels evaluate the reference's
expressions in the reference's order without FMA contraction, so most
comparisons are in fact bit-exact, and the tests record that too.
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _prm(**kw):
    base = dict(gmol=1.0 / 1600, epcorr=1e-10, nouter=9, ninner=5, nouter_min=0)
    base.update(kw)
    return abi.make_flow_params(**base)


def _pair(gpu_lib, oracle_lib, case, prm, noise=0.0, seed=42):
    g = gpu_lib.Solver(case, prm)
    o = oracle_lib.Oracle(case, prm)
    u, v, w, p = cases.taylor_green(case)
    if noise:
        u, v, w = cases.add_noise(case, (u, v, w), amplitude=noise, seed=seed)
    for nm, a in zip("UVWP", (u, v, w, p)):
        g.set(nm, a)
        o.set(nm, a)
    g.connect(0, 2, "U", "V", "W", "P", corners=True)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    return g, o


CASES = {
    "tg32": lambda: cases.periodic_box(1, 1, 1, n=32),
    "tiles8": lambda: cases.periodic_box(2, 2, 2, n=8),
    "tiles24": lambda: cases.periodic_box(3, 2, 2, n=24),
    "aniso": lambda: cases.periodic_box(2, 1, 3, n=10, nj=12, nk=6),
    "stretched": lambda: cases.stretch(cases.periodic_box(2, 2, 1, n=10, nj=9, nk=8)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_setup_coefficients(gpu_lib, oracle_lib, name):
    case = CASES[name]()
    g, o = _pair(gpu_lib, oracle_lib, case, _prm())
    for f in ("GSAP", "SIPLW", "SIPLS", "SIPLB", "SIPLPR", "SIPUE", "SIPUN", "SIPUT"):
        a, b = g.get(f), o.get(f)
        assert np.array_equal(a, b), f
    for f, n in (("GSAW", case.ngrid * case.ii), ("GSAE", case.ngrid * case.ii),
                 ("GSAS", case.ngrid * case.jj), ("GSAN", case.ngrid * case.jj),
                 ("GSAB", case.ngrid * case.kk), ("GSAT", case.ngrid * case.kk)):
        assert np.array_equal(g.get(f, n), o.get(f, n)), f


def test_classic_coefficients(gpu_lib, oracle_lib):
    case = CASES["tiles8"]()
    g, o = _pair(gpu_lib, oracle_lib, case, _prm(psolver=abi.PSOLVER_CLASSIC))
    for f in ("SIPLW", "SIPLS", "SIPLB", "SIPLPR", "SIPUE", "SIPUN", "SIPUT"):
        assert np.array_equal(g.get(f), o.get(f)), f


@pytest.mark.parametrize("layers,corners,normal,forward", [
    (1, False, False, 0), (2, False, False, 0), (2, True, False, 0), (1, True, False, 0),
    (1, False, True, 1), (1, False, False, -1), (1, False, False, 1)])
def test_connect(gpu_lib, oracle_lib, layers, corners, normal, forward):
    case = CASES["tiles8"]()
    g, o = _pair(gpu_lib, oracle_lib, case, _prm())
    rng = np.random.default_rng(5)
    for nm in "UVWP":
        a = rng.normal(size=case.idim3d)
        g.set(nm, a)
        o.set(nm, a)
    if normal:
        g.connect(0, layers, "U", "V", "W", corners=corners, normal=True, forward=forward)
        o.connect(0, layers, "U", "V", "W", corners=corners, normal=True, forward=forward)
    else:
        g.connect(0, layers, "U", "V", "W", "P", corners=corners, forward=forward)
        o.connect(0, layers, "U", "V", "W", "P", corners=corners, forward=forward)
    for nm in "UVWP":
        assert np.array_equal(g.get(nm), o.get(nm)), nm


@pytest.mark.parametrize("name", ["tg32", "tiles8", "aniso", "stretched"])
def test_tstle4_rkstep(gpu_lib, oracle_lib, name):
    case = CASES[name]()
    g, o = _pair(gpu_lib, oracle_lib, case, _prm(gradp=(0.3, -0.2, 0.1)), noise=1e-2)
    g.tstle4()
    o.tstle4()
    for nm in ("UO", "VO", "WO"):
        a, b = g.get(nm), o.get(nm)
        assert rel_l2(a, b) <= RTOL, nm
        assert np.array_equal(a, b), nm
    g.rkstep("U", "DU", "UO", -5.0 / 9.0, 1e-3 * 15 / 16)
    o.rkstep("U", "DU", "UO", -5.0 / 9.0, 1e-3 * 15 / 16)
    assert np.array_equal(g.get("U"), o.get("U"))
    assert np.array_equal(g.get("DU"), o.get("DU"))


@pytest.mark.parametrize("name", ["tg32", "tiles8", "aniso", "stretched"])
def test_divcal_laplacephi(gpu_lib, oracle_lib, name):
    case = CASES[name]()
    g, o = _pair(gpu_lib, oracle_lib, case, _prm(), noise=1e-2)
    g.divcal("RHS", 1234.5)
    o.divcal("RHS", 1234.5)
    assert np.array_equal(g.get("RHS"), o.get("RHS"))
    g.laplacephi("RES", "P")
    o.laplacephi("RES", "P")
    assert np.array_equal(g.get("RES"), o.get("RES"))


@pytest.mark.parametrize("psolver", [abi.PSOLVER_SIP, abi.PSOLVER_CLASSIC])
@pytest.mark.parametrize("name", ["tg32", "tiles8", "tiles24"])
def test_mgpoisl(gpu_lib, oracle_lib, name, psolver):
    case = CASES[name]()
    prm = _prm(psolver=psolver, nouter=3, ninner=4)
    g, o = _pair(gpu_lib, oracle_lib, case, prm, noise=1e-2)
    sg = g.mgpoisl(1e-3 / 3)
    so = o.mgpoisl(1e-3 / 3)
    assert (sg.ipc, sg.nouter_done) == (so.ipc, so.nouter_done)
    assert sg.maxrhs == so.maxrhs
    for nm in ("U", "V", "W", "P", "DP", "RHS"):
        a, b = g.get(nm), o.get(nm)
        assert rel_l2(a, b) <= RTOL, nm


@pytest.mark.parametrize("name,steps", [("tg32", 3), ("tiles8", 3), ("tiles24", 2), ("aniso", 2),
                                        ("stretched", 2)])
def test_stage_parity(gpu_lib, oracle_lib, name, steps):
    case = CASES[name]()
    prm = _prm(nouter_min=9)      # fixed iteration counts: parity independent of epcorr
    g, o = _pair(gpu_lib, oracle_lib, case, prm, noise=1e-2)
    rkg = gpu_lib.rk_scheme("williamson")
    rko = oracle_lib.rk_scheme("williamson")
    dt = 1e-3
    for it in range(1, steps + 1):
        for irk in range(1, 4):
            sg = g.timeintegrate_flow(it, it, 0.0, dt, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, dt, irk, rko)
            assert sg.ipc == so.ipc
    worst = 0.0
    for nm in ("U", "V", "W", "P", "DU", "DV", "DW"):
        e = rel_l2(g.get(nm), o.get(nm))
        worst = max(worst, e)
        assert e <= RTOL, (nm, e)
    ig, io = g.itinfo(dt), o.itinfo(dt)
    assert abs(ig.cflmax - io.cflmax) <= 1e-14 * io.cflmax
    assert abs(ig.divmax - io.divmax) <= 1e-12 * max(io.divmax, 1e-300)
    # enerfg sums in parallel on the GPU (different summation order)
    assert abs(ig.energy - io.energy) <= 1e-11 * io.energy


def test_taylor_green_32_hundred_steps(gpu_lib, oracle_lib):
    """The CPU-runnable configuration: 32^3 Taylor-Green, nu = 1/1600,
    Williamson RK3, dt = 1e-3, 100 steps, SIP to 1e-10."""
    case = CASES["tg32"]()
    prm = _prm(epcorr=1e-10)
    g, o = _pair(gpu_lib, oracle_lib, case, prm)
    rkg = gpu_lib.rk_scheme("williamson")
    rko = oracle_lib.rk_scheme("williamson")
    for it in range(1, 101):
        for irk in range(1, 4):
            sg = g.timeintegrate_flow(it, it, 0.0, 1e-3, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, 1e-3, irk, rko)
            assert sg.ipc == so.ipc
    for nm in "UVWP":
        assert rel_l2(g.get(nm), o.get(nm)) <= RTOL, nm


def test_exploded_flag(gpu_lib):
    """A NaN placed in the velocity field (on the host) is reported by itinfo
    as 'exploded', the reference's stop criterion (itinfo_mod.F90:296-320)."""
    case = CASES["tiles8"]()
    g = gpu_lib.Solver(case, _prm())
    u, v, w, p = cases.taylor_green(case)
    case.interior(u)[3, 2, 1, 4] = np.nan      # an interior cell of grid 4
    for nm, a in zip("UVWP", (u, v, w, p)):
        g.set(nm, a)
    info = g.itinfo(1e-3)
    assert info.exploded == 1
    case.interior(u)[3, 2, 1, 4] = 0.0
    g.set("U", u)
    assert g.itinfo(1e-3).exploded == 0
