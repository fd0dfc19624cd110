"""Scalar transport in the oracle (no GPU): tstsca4 + fluxbalance
(src/scalar/timeintegrate_scalar_mod.F90:164-545) pinned against a
vectorised numpy transcription of one RK stage; the scalar content of a
periodic box is conserved; a diffusing sine mode decays at the rate of the
discrete Laplacian."""
import math

import numpy as np
import pytest

from mglet_gb300 import abi, cases


def _prm(**kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=20, ninner=5, nouter_min=0)
    base.update(kw)
    return abi.make_flow_params(**base)


def _stage_ref(case, u, v, w, t, dtf, frhs, dtfu, gmol, prmol, source):
    """One RK stage of one scalar on a periodic single-level case, no LES."""
    kk, jj, ii = case.kk, case.jj, case.ii
    sh = (case.ngrid, ii, jj, kk)
    U, V, W, Tt = (a.reshape(sh) for a in (u, v, w, t))
    out_t, out_d = t.copy().reshape(sh), dtf.copy().reshape(sh)
    h = [case.ddx[0], case.ddy[0], case.ddz[0]]
    rd = [1.0 / case.dx[0], 1.0 / case.dy[0], 1.0 / case.dz[0]]
    rdd = [1.0 / x for x in h]
    gs = gmol / 1.0 / prmol
    for g in range(case.ngrid):
        q = [np.zeros((ii, jj, kk)) for _ in range(3)]
        T = Tt[g]
        # every face CON: fluxes on 2..n-2 along their direction, 3..n-2 across
        s = slice(2, -2)
        f = slice(1, -2)
        adv = (h[1] * h[2]) * U[g][f, s, s] * 0.5 * (T[f, s, s] + T[2:-1, s, s])
        area = 1.0 * 1.0 * (h[1] * h[2])
        q[0][f, s, s] = adv + (-gs * rd[0] * (T[2:-1, s, s] - T[f, s, s]) * area)
        adv = (h[0] * h[2]) * V[g][s, f, s] * 0.5 * (T[s, f, s] + T[s, 2:-1, s])
        area = 1.0 * 1.0 * (h[0] * h[2])
        q[1][s, f, s] = adv + (-gs * rd[1] * (T[s, 2:-1, s] - T[s, f, s]) * area)
        adv = (h[0] * h[1]) * W[g][s, s, f] * 0.5 * (T[s, s, f] + T[s, s, 2:-1])
        area = 1.0 * 1.0 * (h[0] * h[1])
        q[2][s, s, f] = adv + (-gs * rd[2] * (T[s, s, 2:-1] - T[s, s, f]) * area)
        net = (q[0][1:-3, s, s] - q[0][s, s, s] + q[1][s, 1:-3, s] - q[1][s, s, s]
               + q[2][s, s, 1:-3] - q[2][s, s, s])
        qtt = np.zeros((ii, jj, kk))
        qtt[s, s, s] = rdd[2] * rdd[1] * rdd[0] * net
        if source:
            qtt[s, s, s] = qtt[s, s, s] + source
        d = frhs * out_d[g] + qtt
        out_d[g] = d
        out_t[g] = out_t[g] + dtfu * d
    return out_t.ravel(), out_d.ravel()


def test_scalar_stage_matches_transcription(oracle_lib):
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    o = oracle_lib.Oracle(case, _prm())
    rng = np.random.default_rng(41)
    u, v, w = (rng.standard_normal(case.idim3d) for _ in range(3))
    t = rng.standard_normal(case.idim3d)
    for n, a in zip("UVW", (u, v, w)):
        o.set(n, a)
    o.set_scalars([0.71], source=[0.3])
    o.set("T1", t)
    o.connect(0, 2, "U", "V", "W", "T1", corners=True)
    u, v, w, t = (o.get(n) for n in ("U", "V", "W", "T1"))
    rk = oracle_lib.rk_scheme("williamson")
    o.timeintegrate_scalar(1e-2, 1, rk)
    rt, rd = _stage_ref(case, u, v, w, t, np.zeros(case.idim3d), rk.a[0], 1e-2 * rk.b[0], 1e-2, 0.71, 0.3)
    inner = case.interior(np.arange(case.idim3d))
    assert np.array_equal(o.get("DT1")[inner.ravel()], rd[inner.ravel()])
    # after the corner connect the ghosts are the neighbours' interior values
    ref = oracle_lib.Oracle(case, _prm())
    ref.set_scalars([0.71])
    ref.set("T1", rt)
    ref.connect(0, 2, s1="T1", corners=True)
    assert np.array_equal(o.get("T1"), ref.get("T1"))


def test_scalar_content_is_conserved(oracle_lib):
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0))
    o = oracle_lib.Oracle(case, _prm())
    u, v, w, p = cases.taylor_green(case)
    for n, a in zip("UVWP", (u, v, w, p)):
        o.set(n, a)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    o.set_scalars([0.71, 2.0])
    rng = np.random.default_rng(5)
    for n in ("T1", "T2"):
        o.set(n, 1.0 + 0.1 * rng.standard_normal(case.idim3d))
    o.connect(0, 2, s1="T1", s2="T2", corners=True)
    tot0 = [case.interior(o.get(n)).sum() for n in ("T1", "T2")]
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        o.timeintegrate_scalar(5e-3, irk, rk)
        o.timeintegrate_flow(1, 1, 0.0, 5e-3, irk, rk)
    for n, t0 in zip(("T1", "T2"), tot0):
        assert abs(case.interior(o.get(n)).sum() - t0) <= 1e-12 * abs(t0), n


def test_diffusing_mode_decays_at_the_discrete_rate(oracle_lib):
    """Fluid at rest: dT/dt = kappa L T with kappa = gmol / (rho prmol); a
    sine mode along x is an eigenvector of the discrete Laplacian with
    eigenvalue -(2 - 2 cos(k h)) / h^2, so one RK3 step multiplies it by the
    stability polynomial of that eigenvalue."""
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    gmol, prmol, dt = 1e-2, 0.5, 1e-2
    o = oracle_lib.Oracle(case, _prm(gmol=gmol))
    o.set_scalars([prmol])
    xg, _, _ = case.coords()
    kx = 2 * np.pi / 2.0
    t = np.sin(kx * xg)[:, :, None, None] * np.ones((1, 1, case.jj, case.kk))
    o.set("T1", t.ravel())
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        o.timeintegrate_scalar(dt, irk, rk)
    h = case.dx[0]
    lam = -(gmol / prmol) * (2 - 2 * math.cos(kx * h)) / h ** 2
    z = lam * dt
    amp = 1 + z + z * z / 2 + z ** 3 / 6          # RK3 on a linear problem
    got = case.interior(o.get("T1"))
    want = case.interior(t.ravel()) * amp
    assert np.allclose(got, want, rtol=0, atol=1e-13)


def test_buoyancy_of_a_uniform_scalar_accelerates_uniformly(oracle_lib):
    """-gravity beta T of a uniform scalar is a uniform force, which the
    pressure of a periodic box cannot take up: after one time step the fluid
    moves against gravity at dt g beta T (RK3 integrates a constant force
    exactly), and not across it (boussinesqterm_mod.F90)."""
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    o = oracle_lib.Oracle(case, _prm())
    o.set_scalars([0.71])
    o.set("T1", np.full(case.idim3d, 2.0))
    o.set_buoyancy([0.0, 0.0, -9.81], 3e-3)
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        o.timeintegrate_scalar(1e-2, irk, rk)
        o.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
    for n in "UV":
        assert np.abs(case.interior(o.get(n))).max() < 1e-14, n
    assert np.allclose(case.interior(o.get("W")), 1e-2 * 9.81 * 3e-3 * 2.0, rtol=1e-12, atol=0)


def test_coriolis_turns_a_uniform_stream(oracle_lib):
    """-2 omega x u of a uniform stream u0 along x with omega along z
    accelerates v by -2 omega u0 (coriolisterm_mod.F90): after the first RK
    stage v = dt b1 (-2 omega u0) everywhere inside."""
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    o = oracle_lib.Oracle(case, _prm())
    o.set("U", np.full(case.idim3d, 1.5))
    o.set_coriolis([0.0, 0.0, 0.25])
    rk = oracle_lib.rk_scheme("williamson")
    o.timeintegrate_flow(1, 1, 0.0, 1e-2, 1, rk)
    want = 1e-2 * rk.b[0] * (-2.0 * 0.25 * 1.5)
    assert np.allclose(case.interior(o.get("V")), want, rtol=1e-12, atol=0)
    assert np.allclose(case.interior(o.get("U")), 1.5, rtol=0, atol=1e-14)


def test_sources_apply_in_order(oracle_lib):
    """sourceterm (timeintegrate_scalar_mod.F90:549-634): a constant source
    and value * field sources add to the balance in the order given; at rest
    with a uniform scalar the first stage's DT is exactly that sum."""
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    o = oracle_lib.Oracle(case, _prm())
    o.set_scalars([0.7, 1.0], source=[0.25, 0.0])
    rng = np.random.default_rng(9)
    f = rng.standard_normal(case.idim3d)
    o.set("T1", np.full(case.idim3d, 2.0))
    o.set("T2", f)
    o.add_scalar_source(1, -1.5, "T2")
    o.add_scalar_source(1, 0.125)
    rk = oracle_lib.rk_scheme("williamson")
    o.timeintegrate_scalar(1e-2, 1, rk)
    want = (0.0 + 0.25) + -1.5 * f
    want = want + 0.125
    assert np.array_equal(case.interior(o.get("DT1")), case.interior(want))
    # a field of ones times c is the constant source c, bit for bit
    a, b = (oracle_lib.Oracle(case, _prm()) for _ in range(2))
    for s in (a, b):
        s.set_scalars([0.7, 1.0])
        s.set("T1", f)
    a.add_scalar_source(1, 0.3)
    b.set("T2", np.ones(case.idim3d))
    b.add_scalar_source(1, 0.3, "T2")
    for s in (a, b):
        s.timeintegrate_scalar(1e-2, 1, rk)
    assert np.array_equal(a.get("T1"), b.get("T1"))
    with pytest.raises(RuntimeError):
        o.add_scalar_source(3, 1.0)
    with pytest.raises(RuntimeError):
        o.add_scalar_source(1, 1.0, "NOPE")
