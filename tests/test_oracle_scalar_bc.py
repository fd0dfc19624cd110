"""Scalar wall and in/outflow conditions in the oracle (no GPU): SWA and
SIO of bound_scalar_mod.F90:124-210 (and the twins of the other faces).
The linear conduction profile between two fixed-value walls is steady;
fixed-flux walls change the scalar content at the set rate; an inflow face
carries its value in by advection and diffusion, an outflow face by
advection alone; the wall model of an LES run at rest gives the molecular
wall flux."""
import numpy as np
import pytest

from mglet_gb300 import abi, cases


def _prm(**kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=20, ninner=5, nouter_min=0)
    base.update(kw)
    return abi.make_flow_params(**base)


def _channel(oracle_lib, gmol=1e-2, prmol=0.5):
    case = cases.periodic_box(1, 1, 1, n=8, length=(1.0, 1.0, 1.0),
                              walls={5: abi.BC_NOS, 6: abi.BC_NOS})
    o = oracle_lib.Oracle(case, _prm(gmol=gmol))
    o.set_scalars([prmol])
    return case, o


def _plane(case, value):
    return np.full((case.jj, case.ii), value)


def _content(case, o):
    return case.interior(o.get("T1")).sum() * case.dx[0] * case.dy[0] * case.dz[0]


def test_conduction_profile_is_steady(oracle_lib):
    case, o = _channel(oracle_lib)
    for f, tb in ((5, 1.0), (6, 0.0)):
        o.set_scalar_bc(1, f, 1, [0])
        o.set_buffer("T1", 1, f, _plane(case, tb))
    _, _, zg = case.coords()
    t = (1.0 - zg)[:, None, None, :] * np.ones((1, case.ii, case.jj, 1))
    o.set("T1", t.ravel())
    t0 = case.interior(o.get("T1")).copy()
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        o.timeintegrate_scalar(1e-2, irk, rk)
    assert np.abs(case.interior(o.get("T1")) - t0).max() < 1e-14
    # a uniform field between the same walls is not steady: heat enters below
    o.set("T1", np.full(case.idim3d, 0.5))
    o.timeintegrate_scalar(1e-2, 1, rk)
    t = case.interior(o.get("T1")).reshape(case.ngrid, case.ii - 4, case.jj - 4, case.kk - 4)
    assert np.all(t[..., 0] > 0.5) and np.all(t[..., -1] < 0.5)


def test_fixed_flux_walls_change_content_at_the_set_rate(oracle_lib):
    case, o = _channel(oracle_lib)
    q1, q2 = 0.3, -0.1                       # fluxes into the domain
    for f, q in ((5, q1), (6, q2)):
        o.set_scalar_bc(1, f, 1, [1])
        o.set_buffer("T1", 1, f, _plane(case, q))
    rng = np.random.default_rng(3)
    o.set("T1", 1.0 + 0.1 * rng.standard_normal(case.idim3d))
    o.connect(0, 2, s1="T1", corners=True)
    c0 = _content(case, o)
    rk = oracle_lib.rk_scheme("williamson")
    dt = 1e-2
    for irk in (1, 2, 3):
        o.timeintegrate_scalar(dt, irk, rk)
    assert abs(_content(case, o) - c0 - dt * (q1 + q2) * 1.0) < 1e-14


def test_inflow_and_outflow_faces(oracle_lib):
    gmol, prmol, w0, tin = 1e-2, 0.5, 0.7, 1.0
    case, o = _channel(oracle_lib, gmol, prmol)
    for f in (5, 6):
        o.set_scalar_bc(1, f, 2, [0])
        o.set_buffer("T1", 1, f, _plane(case, tin))
    o.set("W", np.full(case.idim3d, w0))
    # a uniform field at the inflow value is steady
    o.set("T1", np.full(case.idim3d, tin))
    rk = oracle_lib.rk_scheme("williamson")
    o.timeintegrate_scalar(1e-2, 1, rk)
    assert np.all(case.interior(o.get("T1")) == tin)
    # an empty domain takes in w0 tin + 2 gamma tin / h per unit area in the
    # first stage (the ghost value 2 tin - 0 mirrors the inflow value); the
    # outflow face (zero gradient) carries out the advective flux of 0
    o.set("T1", case.zeros())
    o.set("DT1", case.zeros())
    dt = 1e-2
    o.timeintegrate_scalar(dt, 1, rk)
    h = case.dz[0]
    rate = w0 * tin + 2 * (gmol / prmol) * tin / h
    assert abs(_content(case, o) - dt * rk.b[0] * rate) < 1e-14
    # reversed flow: the upper face takes in, the lower one lets out
    o.set("W", np.full(case.idim3d, -w0))
    o.set("T1", case.zeros())
    o.set("DT1", case.zeros())
    o.timeintegrate_scalar(dt, 1, rk)
    t = case.interior(o.get("T1")).reshape(case.ngrid, case.ii - 4, case.jj - 4, case.kk - 4)
    assert np.all(t[..., -1] > 0) and np.all(t[..., :-1] == 0)


def test_wall_model_at_rest_gives_the_molecular_flux(oracle_lib):
    """With the fluid at rest the wall model of an LES run stays in its
    laminar branch, 2 gmol / (rho prmol) (T_wall - T) / h, the flux of the
    run without LES; G stays gmol at rest."""
    out = []
    for les in (0, 1):
        case, o = _channel(oracle_lib)
        for f, tb in ((5, 1.0), (6, -0.5)):
            o.set_scalar_bc(1, f, 1, [0])
            o.set_buffer("T1", 1, f, _plane(case, tb))
        rng = np.random.default_rng(8)
        o.set("T1", rng.standard_normal(case.idim3d))
        o.connect(0, 2, s1="T1", corners=True)
        if les:
            o.set_lesmodel(1)
        rk = oracle_lib.rk_scheme("williamson")
        for irk in (1, 2, 3):
            o.timeintegrate_scalar(1e-2, irk, rk)
        out.append(case.interior(o.get("T1")))
    assert np.allclose(out[0], out[1], rtol=0, atol=1e-14)


def test_scalar_bc_refuses_interior_faces(oracle_lib):
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    o = oracle_lib.Oracle(case, _prm())
    o.set_scalars([0.7])
    with pytest.raises(RuntimeError):
        o.set_scalar_bc(1, 2, 1, [0])        # CON face between the grids
