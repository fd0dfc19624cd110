"""The persistent solve of the mixed form: the whole outer loop of one
single-level mgpoisl (pressuresolver_mod.F90:218-302) as one cooperative
launch with grid-wide barriers between its phases.

It computes every point with the arithmetic of the per-phase kernels, so the
fields, the outer-iteration count and the residual must be the same bits in
every variant, whether the loop stops on the residual or at the outer cap,
and whether a CTA owns one grid or several.  Its barrier waits are bounded:
with the test switch one CTA never arrives, the others give up after about a
second, and the stage reports the time-out through its status without
faulting the GPU.
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_boundaries import face_plane_shape
from test_oracle_ghostcell import gc_case, load

pytestmark = pytest.mark.gpu

NVARIANTS = 6


def _prm(**kw):
    base = dict(gmol=1.0 / 1600, epcorr=1e-10, nouter=4, ninner=5, nouter_min=0,
                form=abi.FORM_MIXED)
    base.update(kw)
    return abi.make_flow_params(**base)


def _tg(solver, case, shift=0.0):
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u + shift, v, w), amplitude=1e-2, seed=42)
    for nm, a in zip("UVWP", (u, v, w, p)):
        solver.set(nm, a)
    solver.connect(0, 2, "U", "V", "W", "P", corners=True)


def _periodic(gpu_lib, case, prm):
    g = gpu_lib.Solver(case, prm)
    _tg(g, case)
    return g


def _walls(gpu_lib, case, prm):
    g = gpu_lib.Solver(case, prm)
    _tg(g, case, shift=0.5)
    rng = np.random.default_rng(17)
    for gi in range(case.ngrid):
        for f in range(1, 7):
            t = case.bctype[gi, f - 1]
            if t == abi.BC_FIX:
                g.set_buffer("U", gi + 1, f, 0.5 + 0.01 * rng.standard_normal(face_plane_shape(case, f)))
            if t == abi.BC_OP1:
                g.set_bc_real(gi + 1, f, 0.05)
    g.bound_flow()
    return g


def _stages(gpu_lib, g, steps, dt):
    rk = gpu_lib.rk_scheme("williamson")
    stats = []
    for it in range(1, steps + 1):
        for irk in range(1, 4):
            st = g.timeintegrate_flow(it, it, 0.0, dt, irk, rk)
            stats.append((st.nouter_done, st.maxrhs))
    return stats


def _compare(gpu_lib, make, steps=2, dt=5e-4, names="UVWP"):
    """The per-phase kernels, then every persistent variant that applies:
    same fields, outer counts and residuals."""
    g = make(-1)
    ref_stats = _stages(gpu_lib, g, steps, dt)
    ref = [g.get(nm) for nm in names]
    assert "mx_sip_solve: per-phase kernels" in g.tuning()
    g.close()
    ran = 0
    for v in range(NVARIANTS):
        g = make(v)
        if g is None:
            continue
        assert "mx_sip_solve: 256 threads" in g.tuning()
        stats = _stages(gpu_lib, g, steps, dt)
        assert stats == ref_stats, (v, stats, ref_stats)
        for nm, a in zip(names, ref):
            assert np.array_equal(g.get(nm), a), (v, nm)
        g.close()
        ran += 1
    assert ran >= 3
    return ref_stats


def _forced(gpu_lib, case, prm, build):
    def make(v):
        g = build(gpu_lib, case, prm)
        try:
            g.force_variant("mx_sip_solve", v)
        except gpu_lib.MgletError:
            g.close()
            return None
        return g
    return make


@pytest.mark.parametrize("tiles,n", [((3, 2, 2), 24), ((16, 8, 8), 8)])
def test_persistent_solve_matches_per_phase(gpu_lib, tiles, n):
    """Periodic tilings: 12 grids of 24^3 (one grid per CTA) and 1024 grids
    of 8^3 (more grids than resident CTAs, so every CTA walks several)."""
    case = cases.periodic_box(*tiles, n=n)
    stats = _compare(gpu_lib, _forced(gpu_lib, case, _prm(), _periodic))
    assert all(k == 4 for k, _ in stats)      # the outer cap in every stage


def test_persistent_solve_stops_on_the_residual(gpu_lib):
    """With a loose epcorr the stopping test ends the loop early, after the
    same outer iteration in both forms."""
    case = cases.periodic_box(2, 2, 2, n=24)
    stats = _compare(gpu_lib, _forced(gpu_lib, case, _prm(epcorr=1e-5, nouter=30), _periodic))
    assert all(k < 30 for k, _ in stats)


def test_persistent_solve_with_walls_and_stretching(gpu_lib):
    """FIX inflow, OP1 outflow, NOS and SLI walls on a stretched tiling: the
    per-point records of the pre-pass (no uniform classes)."""
    walls = {1: abi.BC_FIX, 2: abi.BC_OP1, 3: abi.BC_NOS, 4: abi.BC_SLI}
    case = cases.stretch(cases.periodic_box(3, 2, 2, n=8, length=(2.0, 2.0, 1.0), walls=walls))
    _compare(gpu_lib, _forced(gpu_lib, case, _prm(gmol=1e-3), _walls), dt=2e-3)


def test_persistent_solve_with_ghostcell(gpu_lib):
    """The ghost-cell IB on one level: masked couplings in the records and
    the outer step, SDIV and BP in divcal."""
    case, bp, lists = gc_case(seed=7)
    u, v, w, p = cases.taylor_green(case)
    fields = dict(zip("UVWP", (u, v, w, p)))

    def build(gpu_lib_, case_, prm):
        g = gpu_lib_.Solver(case_, prm)
        load(g, case_, bp, lists, fields)
        g.connect(0, 2, "U", "V", "W", "P", corners=True)
        g.setpointvalues(True)
        return g

    _compare(gpu_lib, _forced(gpu_lib, case, _prm(gmol=1e-2), build), dt=1e-2)


def test_persistent_barrier_wait_runs_out_and_recovers(gpu_lib):
    """Failure detection without a fault: with the test switch one CTA of
    the persistent solve leaves before its first arrival, the others' barrier
    wait gives up after about a second, the stage returns MGLET_ERR_CUDA, and
    the next stage on the same context runs normally."""
    case = cases.periodic_box(2, 2, 1, n=24)
    g = _periodic(gpu_lib, case, _prm())
    g.force_variant("mx_sip_solve", 2)
    rk = gpu_lib.rk_scheme("williamson")
    g.test_barrier_timeout()
    with pytest.raises(gpu_lib.MgletError) as err:
        g.timeintegrate_flow(1, 1, 0.0, 5e-4, 1, rk)
    assert err.value.code == abi.MGLET_ERR_CUDA and "timed out" in str(err.value)
    st = g.timeintegrate_flow(1, 1, 0.0, 5e-4, 1, rk)
    assert np.isfinite(st.maxrhs) and st.nouter_done == 4
    assert np.all(np.isfinite(g.get("U")))
    g.close()


def test_barrier_switch_needs_the_persistent_solve(gpu_lib):
    case = cases.periodic_box(2, 1, 1, n=8)
    g = _periodic(gpu_lib, case, _prm())
    g.force_variant("mx_sip_solve", -1)
    with pytest.raises(gpu_lib.MgletError):
        g.test_barrier_timeout()
    with pytest.raises(gpu_lib.MgletError):
        g.force_variant("mx_sip_solve", 6)
    g.close()


def test_persistent_solve_refused_on_hierarchies(gpu_lib):
    """Hierarchies keep the per-phase kernels (the levels' ctof, parent and
    ftoc sit between the phases)."""
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,))
    g = gpu_lib.Solver(case, _prm())
    for v in range(NVARIANTS):
        with pytest.raises(gpu_lib.MgletError):
            g.force_variant("mx_sip_solve", v)
    g.close()
