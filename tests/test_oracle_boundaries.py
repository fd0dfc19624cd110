"""Boundary conditions FIX, OP1, NOS and SLI in the CPU oracle (no GPU).

bound_flow (src/flow/bound_flow_mod.F90) is pinned two ways:

* against a second, loop-by-loop numpy transcription of bfront / bright /
  bbottom, written independently of the oracle's face-generic C++ (so an
  index or staggering slip in either shows up);
* by flow properties: a uniform inflow through a FIX/OP1 channel is steady
  to the last bit; after a stage with NOS or SLI walls the projected field
  is discretely divergence free; the OP1 ghost pressure is the far-field
  value for outflow and loses the dynamic pressure for inflow.
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases


def _prm(**kw):
    base = dict(gmol=1e-2, epcorr=1e-13, nouter=40, ninner=5, nouter_min=0)
    base.update(kw)
    return abi.make_flow_params(**base)


def _sign(a, b):
    return np.copysign(abs(a), b)


def bound_reference(case, g, iface, typ, u, v, w, p, ub, vb, wb, pinf, rho):
    """bound_flow_mod.F90 loops for one face of grid g (0-based), arrays
    indexed [i, j, k] 1-based through offsets (ghost layers included)."""
    kk, jj, ii = case.kk, case.jj, case.ii
    U = u[g].reshape(ii, jj, kk)
    V = v[g].reshape(ii, jj, kk)
    W = w[g].reshape(ii, jj, kk)
    P = p[g].reshape(ii, jj, kk)
    A = lambda arr, k, j, i: arr[i - 1, j - 1, k - 1]

    def S(arr, k, j, i, val):
        arr[i - 1, j - 1, k - 1] = val
    B = lambda buf, a, b: buf[a - 1, b - 1]
    if iface in (1, 2):
        i2, i3, s1, s2, d = (2, 3, 1, 2, -1.0) if iface == 1 else (ii - 1, ii - 2, ii - 1, ii - 2, 1.0)
        if typ == abi.BC_FIX:
            for j in range(1, jj + 1):
                for k in range(1, kk + 1):
                    S(U, k, j, s2, B(ub, k, j))
                    S(V, k, j, i2, 2.0 * B(vb, k, j) - A(V, k, j, i3))
                    S(W, k, j, i2, 2.0 * B(wb, k, j) - A(W, k, j, i3))
        elif typ == abi.BC_OP1:
            for j in range(1, jj):
                for k in range(1, kk):
                    S(U, k, j, s1, A(U, k, j, s2))
                    f = 0.5 * (_sign(1.0, d * (A(U, k, j, s2) + A(U, k, j + 1, s2))) + 1.0)
                    S(V, k, j, i2, f * A(V, k, j, i3) + (1.0 - f) * (2.0 * B(vb, k, j) - A(V, k, j, i3)))
                    f = 0.5 * (_sign(1.0, d * (A(U, k, j, s2) + A(U, k + 1, j, s2))) + 1.0)
                    S(W, k, j, i2, f * A(W, k, j, i3) + (1.0 - f) * (2.0 * B(wb, k, j) - A(W, k, j, i3)))
        elif typ == abi.BC_NOS:
            U[s2 - 1, :, :] = 0.0
            V[i2 - 1, :, :] = 0.0
            W[i2 - 1, :, :] = 0.0
        elif typ == abi.BC_SLI:
            U[s2 - 1, :, :] = 0.0
            V[i2 - 1, :, :] = V[i3 - 1, :, :]
            W[i2 - 1, :, :] = W[i3 - 1, :, :]
        if typ == abi.BC_OP1:
            for j in range(2, jj + 1):
                for k in range(2, kk + 1):
                    vi = 0.25 * (A(V, k, j - 1, i2) + A(V, k, j, i2) + A(V, k, j - 1, i3) + A(V, k, j, i3))
                    wi = 0.25 * (A(W, k - 1, j, i2) + A(W, k, j, i2) + A(W, k - 1, j, i3) + A(W, k, j, i3))
                    um = A(U, k, j, s2) ** 2 + vi ** 2 + wi ** 2
                    S(P, k, j, i2, pinf + min(0.0, 0.5 * rho * _sign(um, d * A(U, k, j, s2))))
        else:
            P[i2 - 1, :, :] = P[i3 - 1, :, :]
    elif iface in (3, 4):
        j2, j3, s1, s2, d = (2, 3, 1, 2, -1.0) if iface == 3 else (jj - 1, jj - 2, jj - 1, jj - 2, 1.0)
        if typ == abi.BC_FIX:
            for i in range(1, ii + 1):
                for k in range(1, kk + 1):
                    S(U, k, j2, i, 2.0 * B(ub, k, i) - A(U, k, j3, i))
                    S(V, k, s2, i, B(vb, k, i))
                    S(W, k, j2, i, 2.0 * B(wb, k, i) - A(W, k, j3, i))
        elif typ == abi.BC_OP1:
            for i in range(1, ii):
                for k in range(1, kk):
                    f = 0.5 * (_sign(1.0, d * (A(V, k, s2, i) + A(V, k, s2, i + 1))) + 1.0)
                    S(U, k, j2, i, f * A(U, k, j3, i) + (1.0 - f) * (2.0 * B(ub, k, i) - A(U, k, j3, i)))
                    S(V, k, s1, i, A(V, k, s2, i))
                    f = 0.5 * (_sign(1.0, d * (A(V, k, s2, i) + A(V, k + 1, s2, i))) + 1.0)
                    S(W, k, j2, i, f * A(W, k, j3, i) + (1.0 - f) * (2.0 * B(wb, k, i) - A(W, k, j3, i)))
        elif typ == abi.BC_NOS:
            U[:, j2 - 1, :] = 0.0
            V[:, s2 - 1, :] = 0.0
            W[:, j2 - 1, :] = 0.0
        elif typ == abi.BC_SLI:
            U[:, j2 - 1, :] = U[:, j3 - 1, :]
            V[:, s2 - 1, :] = 0.0
            W[:, j2 - 1, :] = W[:, j3 - 1, :]
        if typ == abi.BC_OP1:
            for i in range(2, ii + 1):
                for k in range(2, kk + 1):
                    ui = 0.25 * (A(U, k, j2, i - 1) + A(U, k, j2, i) + A(U, k, j3, i - 1) + A(U, k, j3, i))
                    wi = 0.25 * (A(W, k - 1, j2, i) + A(W, k, j2, i) + A(W, k - 1, j3, i) + A(W, k, j3, i))
                    um = ui ** 2 + A(V, k, s2, i) ** 2 + wi ** 2
                    S(P, k, j2, i, pinf + min(0.0, 0.5 * rho * _sign(um, d * A(V, k, s2, i))))
        else:
            P[:, j2 - 1, :] = P[:, j3 - 1, :]
    else:
        k2, k3, s1, s2, d = (2, 3, 1, 2, -1.0) if iface == 5 else (kk - 1, kk - 2, kk - 1, kk - 2, 1.0)
        if typ == abi.BC_FIX:
            for i in range(1, ii + 1):
                for j in range(1, jj + 1):
                    S(U, k2, j, i, 2.0 * B(ub, j, i) - A(U, k3, j, i))
                    S(V, k2, j, i, 2.0 * B(vb, j, i) - A(V, k3, j, i))
                    S(W, s2, j, i, B(wb, j, i))
        elif typ == abi.BC_OP1:
            for i in range(1, ii):
                for j in range(1, jj):
                    f = 0.5 * (_sign(1.0, d * (A(W, s2, j, i) + A(W, s2, j, i + 1))) + 1.0)
                    S(U, k2, j, i, f * A(U, k3, j, i) + (1.0 - f) * (2 * B(ub, j, i) - A(U, k3, j, i)))
                    f = 0.5 * (_sign(1.0, d * (A(W, s2, j, i) + A(W, s2, j + 1, i))) + 1.0)
                    S(V, k2, j, i, f * A(V, k3, j, i) + (1.0 - f) * (2.0 * B(vb, j, i) - A(V, k3, j, i)))
                    S(W, s1, j, i, A(W, s2, j, i))
        elif typ == abi.BC_NOS:
            U[:, :, k2 - 1] = 0.0
            V[:, :, k2 - 1] = 0.0
            W[:, :, s2 - 1] = 0.0
        elif typ == abi.BC_SLI:
            U[:, :, k2 - 1] = U[:, :, k3 - 1]
            V[:, :, k2 - 1] = V[:, :, k3 - 1]
            W[:, :, s2 - 1] = 0.0
        if typ == abi.BC_OP1:
            for i in range(2, ii + 1):
                for j in range(2, jj + 1):
                    ui = 0.25 * (A(U, k2, j, i - 1) + A(U, k2, j, i) + A(U, k3, j, i - 1) + A(U, k3, j, i))
                    vi = 0.25 * (A(V, k2, j - 1, i) + A(V, k2, j, i) + A(V, k3, j - 1, i) + A(V, k3, j, i))
                    um = ui ** 2 + vi ** 2 + A(W, s2, j, i) ** 2
                    S(P, k2, j, i, pinf + min(0.0, 0.5 * rho * _sign(um, d * A(W, s2, j, i))))
        else:
            P[:, :, k2 - 1] = P[:, :, k3 - 1]


def face_plane_shape(case, iface):
    return ((case.kk, case.jj), (case.kk, case.ii), (case.jj, case.ii))[(iface - 1) // 2]


def random_bc_case(walls, seed):
    case = cases.periodic_box(2, 1, 1, n=6, nj=5, nk=4, length=(2.0, 1.0, 1.0), walls=walls)
    rng = np.random.default_rng(seed)
    fields = {nm: rng.standard_normal(case.idim3d) for nm in "UVWP"}
    bufs = {}
    for g in range(case.ngrid):
        for f in range(1, 7):
            if case.bctype[g, f - 1] in (abi.BC_FIX, abi.BC_OP1):
                for nm in "UVW":
                    bufs[(nm, g, f)] = rng.standard_normal(face_plane_shape(case, f))
    return case, fields, bufs


@pytest.mark.parametrize("walls", [
    {1: abi.BC_FIX, 2: abi.BC_OP1},
    {3: abi.BC_OP1, 4: abi.BC_FIX, 5: abi.BC_NOS, 6: abi.BC_SLI},
    {1: abi.BC_SLI, 2: abi.BC_NOS, 5: abi.BC_OP1, 6: abi.BC_OP1},
    {5: abi.BC_FIX, 6: abi.BC_FIX, 3: abi.BC_NOS, 4: abi.BC_SLI},
])
def test_bound_flow_matches_loop_transcription(oracle_lib, walls):
    case, fields, bufs = random_bc_case(walls, seed=len(walls) * 7 + 1)
    o = oracle_lib.Oracle(case, _prm())
    for nm, a in fields.items():
        o.set(nm, a)
    zero = {f: np.zeros(face_plane_shape(case, f)) for f in range(1, 7)}
    pinf = {}
    for (nm, g, f), b in bufs.items():
        o.set_buffer(nm, g + 1, f, b)
        if case.bctype[g, f - 1] == abi.BC_OP1 and (g, f) not in pinf:
            pinf[(g, f)] = 0.1 * (g + f)
            o.set_bc_real(g + 1, f, pinf[(g, f)])
    o.bound_flow()
    ref = {nm: a.copy().reshape(case.ngrid, -1) for nm, a in fields.items()}
    for g in range(case.ngrid):
        for f in range(1, 7):
            typ = case.bctype[g, f - 1]
            if typ in (abi.BC_FIX, abi.BC_OP1, abi.BC_NOS, abi.BC_SLI):
                bb = [bufs.get((nm, g, f), zero[f]) for nm in "UVW"]
                bound_reference(case, g, f, typ, ref["U"], ref["V"], ref["W"], ref["P"], *bb,
                                pinf.get((g, f), 0.0), 1.0)
    for nm in "UVWP":
        assert np.array_equal(o.get(nm), ref[nm].ravel()), nm


def _channel(oracle_lib, nx=3, n=8, walls=None):
    walls = walls or {1: abi.BC_FIX, 2: abi.BC_OP1}
    case = cases.periodic_box(nx, 1, 1, n=n, length=(float(nx), 1.0, 1.0), walls=walls)
    o = oracle_lib.Oracle(case, _prm())
    return case, o


def test_uniform_channel_flow_is_steady(oracle_lib):
    """u = 1 entering through FIX and leaving through OP1, periodic in y and
    z: the stage leaves the field exactly unchanged."""
    case, o = _channel(oracle_lib)
    n = case.idim3d
    o.set("U", np.ones(n))
    for nm in "VWP":
        o.set(nm, np.zeros(n))
    for g in range(case.ngrid):
        if case.bctype[g, 0] == abi.BC_FIX:
            o.set_buffer("U", g + 1, 1, np.ones((case.kk, case.jj)))
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = oracle_lib.rk_scheme("williamson")
    for it in range(1, 4):
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, 1e-2, irk, rk)
    assert np.array_equal(case.interior(o.get("U")), np.ones_like(case.interior(o.get("U"))))
    for nm in "VWP":
        assert not np.any(case.interior(o.get(nm)))


@pytest.mark.parametrize("walls", [{5: abi.BC_NOS, 6: abi.BC_NOS}, {3: abi.BC_SLI, 4: abi.BC_NOS},
                                   {1: abi.BC_NOS, 2: abi.BC_SLI, 5: abi.BC_SLI, 6: abi.BC_NOS}])
def test_wall_stage_is_divergence_free(oracle_lib, walls):
    """After a stage with no-slip / free-slip walls the divergence of the
    projected field equals the pressure solver's own residual: bound_flow
    keeps the wall-normal velocity fixed where giteig removed the wall
    coefficient, so the operator the solver inverts is the one the
    projection applies.  (With walls in two directions the singular Neumann
    problem converges more slowly; the tolerance is on the residual.)"""
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0), walls=walls)
    o = oracle_lib.Oracle(case, _prm())
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=1e-2, seed=5)
    for nm, a in zip("UVWP", (u, v, w, p)):
        o.set(nm, a)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    st = o.timeintegrate_flow(1, 1, 0.0, 1e-2, 1, oracle_lib.rk_scheme("williamson"))
    res = st.maxrhs / st.prefak
    assert res < 1e-8
    assert o.itinfo(1e-2).divmax <= 1.01 * res + 1e-13


@pytest.mark.parametrize("udir,expect", [(1.0, 0.25), (-1.0, 0.25 - 0.5)])
def test_op1_ghost_pressure(oracle_lib, udir, expect):
    """OP1 far-field pressure: outflow keeps pinf, inflow subtracts
    rho |u|^2 / 2 (bound_flow_mod.F90:236-248)."""
    case, o = _channel(oracle_lib, nx=1, n=6)
    n = case.idim3d
    o.set("U", np.full(n, udir))
    for nm in "VWP":
        o.set(nm, np.zeros(n))
    o.set_bc_real(1, 2, 0.25)
    o.bound_flow()
    P = o.get("P").reshape(case.ii, case.jj, case.kk)
    ghost = P[case.ii - 2, 1:, 1:]   # i2 = ii-1, j, k = 2..
    assert np.allclose(ghost, expect, rtol=0, atol=1e-15)


@pytest.mark.parametrize("walls", [{5: abi.BC_NOS, 6: abi.BC_SLI}, {1: abi.BC_FIX, 2: abi.BC_OP1}, None])
def test_viscosity_field_at_start(oracle_lib, walls):
    """G as init_lesmodel leaves it for the model "none" (lesmodel_mod.F90:
    63-80): gmol inside, 0 on the ghost layers, then connected with corners,
    so the ghost layers of a CON face hold gmol and those of a boundary face
    stay 0 on the coarsest level (no viscous flux through it; NOS walls carry
    the wall function instead)."""
    gmol = 0.02
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0), walls=walls)
    o = oracle_lib.Oracle(case, _prm(gmol=gmol))
    G = o.get("G").reshape(case.ngrid, case.ii, case.jj, case.kk)
    assert np.all(G[:, 2:-2, 2:-2, 2:-2] == gmol)
    for g in range(case.ngrid):
        for f in range(1, 7):
            d, hi = (f - 1) // 2, (f - 1) % 2
            ghost = [slice(2, -2)] * 3
            ghost[d] = slice(-2, None) if hi else slice(0, 2)
            plane = G[g][tuple(ghost)]
            want = gmol if case.bctype[g, f - 1] == abi.BC_CON else 0.0
            assert np.all(plane == want), (g, f)
