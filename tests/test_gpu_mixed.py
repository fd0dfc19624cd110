"""The batched mixed-precision form (MGLET_FORM_MIXED) against the FP64 oracle.

The inner SIP iterations run in FP32 under the FP64 defect-correction outer
loop, so results are not bit-identical to the reference; with the outer loop
converged they agree to the convergence level.  Tolerances are stated per
test.
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_levels import prepare_levels

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def vel_err(case, ga, gb):
    """Relative L2 error of the velocity vector (u, v, w) on the interior.
    Taylor-Green starts with w = 0, so a per-component norm of w would
    measure noise against noise."""
    num = sum(np.sum((case.interior(ga(nm)) - case.interior(gb(nm))) ** 2) for nm in "UVW")
    den = sum(np.sum(case.interior(gb(nm)) ** 2) for nm in "UVW")
    return float(np.sqrt(num / den))


def _prm(form, **kw):
    base = dict(gmol=1.0 / 1600, epcorr=1e-11, nouter=40, ninner=5, nouter_min=0, form=form)
    base.update(kw)
    return abi.make_flow_params(**base)


def _init(solver, case, noise=1e-2):
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=noise, seed=42)
    for nm, a in zip("UVWP", (u, v, w, p)):
        solver.set(nm, a)
    solver.connect(0, 2, "U", "V", "W", "P", corners=True)


@pytest.mark.parametrize("tiles,n", [((2, 2, 2), 8), ((2, 2, 1), 24), ((1, 1, 1), 32)])
def test_mixed_stage_against_oracle(gpu_lib, oracle_lib, tiles, n):
    """Three RK3 steps with up to 40 outer iterations: the velocity vector
    agrees to relative L2 <= 5e-9, the pressure (mean removed) to 1e-6."""
    case = cases.periodic_box(*tiles, n=n)
    g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED))
    o = oracle_lib.Oracle(case, _prm(abi.FORM_PLAIN))
    _init(g, case)
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=1e-2, seed=42)
    for nm, a in zip("UVWP", (u, v, w, p)):
        o.set(nm, a)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    rkg, rko = gpu_lib.rk_scheme("williamson"), oracle_lib.rk_scheme("williamson")
    for it in range(1, 4):
        for irk in range(1, 4):
            sg = g.timeintegrate_flow(it, it, 0.0, 1e-3, irk, rkg)
            so = o.timeintegrate_flow(it, it, 0.0, 1e-3, irk, rko)
            assert sg.maxrhs / sg.prefak < 1e-11 or sg.nouter_done == 40
    e = vel_err(case, g.get, o.get)
    assert e <= 5e-9, e
    # pressure is defined up to a constant; compare after removing the mean
    pg, po = case.interior(g.get("P")), case.interior(o.get("P"))
    assert rel_l2(pg - pg.mean(), po - po.mean()) <= 1e-6
    info_g, info_o = g.itinfo(1e-3), o.itinfo(1e-3)
    assert info_g.divmax < 10 * info_o.divmax + 1e-9


def test_mixed_device_convergence_flag(gpu_lib):
    """The outer loop stops on the device as soon as max|rhs|/prefak < epcorr
    (pressuresolver_mod.F90:294-301): a loose tolerance needs fewer outer
    iterations than a tight one, and ipc = nouter_done * ninner."""
    case = cases.periodic_box(2, 2, 2, n=8)
    res = {}
    for eps in (1e-4, 1e-12):
        g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=eps, nouter=30))
        _init(g, case)
        st = g.timeintegrate_flow(1, 1, 0.0, 1e-3, 1, gpu_lib.rk_scheme("williamson"))
        assert st.ipc == st.nouter_done * 5
        res[eps] = st
    assert res[1e-4].nouter_done < res[1e-12].nouter_done
    assert res[1e-4].maxrhs / res[1e-4].prefak < 1e-4


def test_graph_replay_matches_eager(gpu_lib):
    """A stage replayed from its CUDA graph gives the same bits as the same
    stage issued kernel by kernel (per-kernel profiling forces eager issue)."""
    case = cases.periodic_box(2, 2, 1, n=24)
    out = []
    for profile in (False, True):
        g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=9))
        _init(g, case)
        g.profile(profile)
        rk = gpu_lib.rk_scheme("williamson")
        for it in range(1, 3):
            for irk in range(1, 4):
                g.timeintegrate_flow(it, it, 0.0, 5e-4, irk, rk)
        out.append([g.get(nm) for nm in "UVWP"])
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_graph_serves_changing_dt(gpu_lib):
    """A time step size that changes every step (as targetcflmax does,
    timeloop_mod.F90:105-121) replays the one captured stage graph: the
    stage scalars come from device memory, so the result equals eager issue
    bit for bit and every stage launches the same number of kernels."""
    case = cases.periodic_box(2, 2, 1, n=24)
    out, per_stage = [], []
    dts = [5e-4, 4.3e-4, 6.1e-4, 5.7e-4]
    for profile in (False, True):
        g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=9))
        _init(g, case)
        g.profile(profile)
        rk = gpu_lib.rk_scheme("williamson")
        counts = []
        for it, dt in enumerate(dts, start=1):
            for irk in range(1, 4):
                n0 = g.launches
                g.timeintegrate_flow(it, it, 0.0, dt, irk, rk)
                counts.append(g.launches - n0)
        out.append([g.get(nm) for nm in "UVWP"])
        per_stage.append(counts)
    for a, b in zip(*out):
        assert np.array_equal(a, b)
    assert len(set(per_stage[0])) == 1, per_stage[0]


def test_mixed_matches_plain_gpu(gpu_lib):
    """Mixed against the plain FP64 GPU form on the 4-grid 24^3 tiling."""
    case = cases.periodic_box(2, 2, 1, n=24)
    gm = gpu_lib.Solver(case, _prm(abi.FORM_MIXED))
    gp = gpu_lib.Solver(case, _prm(abi.FORM_PLAIN))
    _init(gm, case)
    _init(gp, case)
    rk = gpu_lib.rk_scheme("williamson")
    for it in range(1, 3):
        for irk in range(1, 4):
            gm.timeintegrate_flow(it, it, 0.0, 5e-4, irk, rk)
            gp.timeintegrate_flow(it, it, 0.0, 5e-4, irk, rk)
    assert vel_err(case, gm.get, gp.get) <= 5e-9


def test_mixed_precision_solenoidal_field(gpu_lib):
    """The precision configuration at small scale: a projected solenoidal
    random field, nu = 1e-3, 30 RK3 steps at dt = 2e-4, pressure to 1e-10.
    Against the plain FP64 form (bit-identical to the oracle) the velocity
    vector stays within relative L2 1e-8 and the pressure within 1e-6."""
    case = cases.periodic_box(2, 2, 2, n=16)
    u, v, w = cases.divergence_free_modes(case, nmodes=24, kpeak=4.0, urms=1.0, seed=4242)
    prm = lambda form: abi.make_flow_params(gmol=1e-3, epcorr=1e-10, nouter=40, ninner=5,
                                            nouter_min=0, form=form)
    ref = gpu_lib.Solver(case, prm(abi.FORM_PLAIN))
    for nm, a in zip("UVWP", (u, v, w, np.zeros_like(u))):
        ref.set(nm, a)
    ref.connect(0, 2, "U", "V", "W", "P", corners=True)
    ref.mgpoisl(1.0)
    ref.set("P", np.zeros_like(u))
    mix = gpu_lib.Solver(case, prm(abi.FORM_MIXED))
    for nm in "UVWP":
        mix.set(nm, ref.get(nm))
    mix.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = gpu_lib.rk_scheme("williamson")
    for it in range(1, 31):
        for irk in range(1, 4):
            ref.timeintegrate_flow(it, it, 0.0, 2e-4, irk, rk)
            mix.timeintegrate_flow(it, it, 0.0, 2e-4, irk, rk)
    assert vel_err(case, mix.get, ref.get) <= 1e-8
    pm, pr = case.interior(mix.get("P")), case.interior(ref.get("P"))
    assert rel_l2(pm - pm.mean(), pr - pr.mean()) <= 1e-6


def test_pre_pass_variants_agree(gpu_lib):
    """Every launch variant of the pre-pass the tuner may pick (loads ahead,
    CTAs per SM, uniform-coefficient records) gives the same bits."""
    case = cases.periodic_box(2, 2, 1, n=24)
    out = []
    g0 = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=3))
    assert "mx_sip_pre" in g0.tuning() and "uniform classes: yes" in g0.tuning()
    g0.close()
    for v in range(10):
        g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=3))
        g.force_variant("mx_sip_pre", v)
        _init(g, case)
        rk = gpu_lib.rk_scheme("williamson")
        for irk in range(1, 4):
            g.timeintegrate_flow(1, 1, 0.0, 5e-4, irk, rk)
        out.append([g.get(nm) for nm in "UVWP"])
        g.close()
    for o in out[1:]:
        for a, b in zip(out[0], o):
            assert np.array_equal(a, b)


def test_uniform_variant_refused_without_uniform_classes(gpu_lib):
    case = cases.stretch(cases.periodic_box(2, 1, 1, n=8))
    g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED))
    assert "uniform classes: no" in g.tuning()
    with pytest.raises(gpu_lib.MgletError):
        g.force_variant("mx_sip_pre", 5)
    g.force_variant("mx_sip_pre", 2)


@pytest.mark.parametrize("n", [24, 8])
def test_flux_tma_variant_agrees(gpu_lib, n):
    """The flux kernel with its planes staged by TMA tensor copies gives the
    same bits as the plane-load kernel (same windows, same arithmetic)."""
    case = cases.periodic_box(2, 2, 1, n=n)
    out = []
    for v in (0, 1):
        g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=3))
        assert "mx_flux" in g.tuning()
        g.force_variant("mx_flux", v)
        _init(g, case)
        rk = gpu_lib.rk_scheme("williamson")
        for it in (1, 2):
            for irk in range(1, 4):
                st = g.timeintegrate_flow(it, it, 0.0, 5e-4, irk, rk)
                assert np.isfinite(st.maxrhs)
        out.append([g.get(nm) for nm in ("U", "V", "W", "P", "DU", "DV", "DW")])
        g.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_sweep_variants_agree(gpu_lib):
    """The packed forward and backward sweeps in every launch variant the
    tuner may pick (ranks per thread, CTAs per SM) give the same bits."""
    case = cases.periodic_box(2, 2, 1, n=24)
    out = []
    for v in range(5):
        g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=3))
        assert "sweeps:" in g.tuning()
        g.force_variant("mx_sip_sweep", v)
        _init(g, case)
        rk = gpu_lib.rk_scheme("williamson")
        for irk in range(1, 4):
            g.timeintegrate_flow(1, 1, 0.0, 5e-4, irk, rk)
        out.append([g.get(nm) for nm in "UVWP"])
        g.close()
    for o in out[1:]:
        for a, b in zip(out[0], o):
            assert np.array_equal(a, b)


def test_bounded_wait_runs_out_and_recovers(gpu_lib):
    """Failure detection without a fault: with the test switch the TMA flux
    kernel leaves one plane's copy out, its mbarrier wait gives up after
    about a second, the stage returns MGLET_ERR_CUDA, and the next stage on
    the same context runs normally."""
    case = cases.periodic_box(1, 1, 1, n=24)
    g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=3))
    _init(g, case)
    g.force_variant("mx_flux", 1)
    rk = gpu_lib.rk_scheme("williamson")
    g.test_wait_timeout()
    with pytest.raises(gpu_lib.MgletError) as err:
        g.timeintegrate_flow(1, 1, 0.0, 5e-4, 1, rk)
    assert err.value.code == abi.MGLET_ERR_CUDA and "timed out" in str(err.value)
    st = g.timeintegrate_flow(1, 1, 0.0, 5e-4, 1, rk)
    assert np.isfinite(st.maxrhs)
    assert np.all(np.isfinite(g.get("U")))
    g.close()


@pytest.mark.parametrize("walls", [False, True])
def test_outer_step_writes_the_next_pre_pass(gpu_lib, walls):
    """On one level the outer step writes the pre-pass of the next outer
    iteration's first inner iteration (hilf = 0: rhs * lpr), which is then
    not launched: the same bits as launching it, with and without walls
    (per-point records), at the outer cap and with an early stop."""
    kw = {"walls": {1: abi.BC_NOS, 2: abi.BC_SLI}} if walls else {}
    case = cases.periodic_box(2, 2, 1, n=24, **kw)
    for eps, nouter in ((1e-10, 4), (1e-5, 30)):
        out = []
        for v in (0, 1):
            g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=eps, nouter=nouter))
            g.force_variant("mx_outer_pre", v)
            assert ("writes the next pre-pass" in g.tuning()) == (v == 1)
            _init(g, case)
            rk = gpu_lib.rk_scheme("williamson")
            stats = []
            for it in (1, 2):
                for irk in range(1, 4):
                    st = g.timeintegrate_flow(it, it, 0.0, 5e-4, irk, rk)
                    stats.append((st.nouter_done, st.maxrhs))
            out.append((stats, [g.get(nm) for nm in "UVWP"]))
            g.close()
        assert out[0][0] == out[1][0]
        for a, b in zip(out[0][1], out[1][1]):
            assert np.array_equal(a, b)


def _init_any(g, case):
    """Taylor-Green with noise on a single level or a hierarchy."""
    if case.iparent is None or all(p == 0 for p in case.iparent):
        _init(g, case)
        return
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=1e-2, seed=42)
    for nm, a in zip("UVWP", (u, v, w, p)):
        g.set(nm, a)
    g.set_hierarchy(case.iparent, case.position)
    for lvl in (1, 2):
        g.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
    prepare_levels(g, case)


def test_natural_order_divcal_and_scatter_same_bits(gpu_lib):
    """divcal and the scatter of dp in natural order (the default) and in
    plane order give the same bits: one level, and a two-level hierarchy."""
    for case in (cases.periodic_box(2, 2, 1, n=24), cases.refined_box(2, 2, 2, n=8, refine=(1,))):
        out = []
        for v in (0, 1):
            g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=4))
            g.force_variant("mx_order", v)
            _init_any(g, case)
            rk = gpu_lib.rk_scheme("williamson")
            for irk in range(1, 4):
                g.timeintegrate_flow(1, 1, 0.0, 5e-4, irk, rk)
            out.append([g.get(nm) for nm in ("U", "V", "W", "P", "DP")])
            g.close()
        for a, b in zip(*out):
            assert np.array_equal(a, b)


def test_outer_step_variants_same_bits(gpu_lib):
    """The outer step with hilf staged by a bulk copy and the two direct-load
    variants give the same bits: one level, walls, and a hierarchy (PAR
    ghost planes)."""
    for case in (cases.periodic_box(2, 2, 1, n=24),
                 cases.periodic_box(2, 2, 1, n=8, walls={1: abi.BC_NOS, 2: abi.BC_SLI}),
                 cases.refined_box(2, 2, 2, n=8, refine=(1,))):
        out = []
        for v in range(3):
            g = gpu_lib.Solver(case, _prm(abi.FORM_MIXED, epcorr=1e-10, nouter=4))
            assert "mx_outer:" in g.tuning()
            g.force_variant("mx_outer", v)
            _init_any(g, case)
            rk = gpu_lib.rk_scheme("williamson")
            for irk in range(1, 4):
                g.timeintegrate_flow(1, 1, 0.0, 5e-4, irk, rk)
            out.append([g.get(nm) for nm in "UVWP"])
            g.close()
        for o in out[1:]:
            for a, b in zip(out[0], o):
                assert np.array_equal(a, b)
