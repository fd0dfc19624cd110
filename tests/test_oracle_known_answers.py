"""Known-answer checks that pin the CPU oracle (no GPU needed).

The reference ships no golden field vectors (its tests are whole-program
runs that pass on a clean exit), so the oracle is pinned by properties the
reference's discretisation must satisfy exactly or to a known order:

* hyperplane SIP index lists cover the interior once, plane m = i+j+k
  (the self-checks of src/flow/sip_hyperplane_mod.F90:398-447);
* connect fills every ghost cell from the periodic image, with the message
  sizes of src/core/connect/connect_core_mod.F90:605-637;
* laplacephi reproduces the discrete Fourier eigenvalue of the 7-point
  operator built by giteig (src/ib/noib_mod.F90:81-250);
* the convective term of tstle4_kon is skew-symmetric: it conserves kinetic
  energy for a discretely solenoidal field (src/flow/tstle4_mod.F90:123-138);
* a pure shear mode decays at the discrete diffusion rate with 3rd-order
  time accuracy of Williamson's RK3 (src/core/rungekutta_mod.F90:70-95);
* the 2-D Taylor-Green vortex (tests/TaylorGreen, tests/Taylorvortex_2D of
  the reference) decays like exp(-2 nu k^2 t) with second-order spatial
  error;
* periodic boxes conserve the bulk velocity (the GeostrophicWind check.py
  criterion of the reference, bulk velocity constant to 1e-5).
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases


def _prm(**kw):
    base = dict(gmol=1.0 / 1600, epcorr=1e-12, nouter=9, ninner=5, nouter_min=0)
    base.update(kw)
    return abi.make_flow_params(**base)


def test_sip_hyperplane_tables(oracle_lib):
    case = cases.periodic_box(1, 1, 1, n=8, nj=6, nk=5)
    o = oracle_lib.Oracle(case, _prm())
    mip, idx = o.sip_index()
    kk, jj, ii = case.kk, case.jj, case.ii
    n3dmax = (ii - 2) + (jj - 2) + (kk - 2)
    seen = np.zeros((ii, jj, kk), dtype=int)
    for m in range(9, n3dmax + 1):
        lo, hi = mip[m - 1], mip[m]
        plane = idx[lo:hi]
        assert np.all(np.diff(plane) > 0), "plane not sorted"
        for lin in plane:
            r = lin - 1
            k, j, i = r % kk + 1, (r // kk) % jj + 1, r // (kk * jj) + 1
            assert k + j + i == m
            seen[i - 1, j - 1, k - 1] += 1
    assert seen[2:ii - 2, 2:jj - 2, 2:kk - 2].min() == 1
    assert seen.sum() == (ii - 4) * (jj - 4) * (kk - 4)


def _global_index_field(case):
    """Every point holds the global (periodic) cell number of its position."""
    nx = case.gridpos[:, 0].max() + 1
    ny = case.gridpos[:, 1].max() + 1
    nz = case.gridpos[:, 2].max() + 1
    ni, nj, nk = case.ii - 4, case.jj - 4, case.kk - 4
    f = np.empty((case.ngrid, case.ii, case.jj, case.kk))
    i = np.arange(case.ii) - 2
    j = np.arange(case.jj) - 2
    k = np.arange(case.kk) - 2
    for g in range(case.ngrid):
        gx, gy, gz = case.gridpos[g]
        I = (gx * ni + i) % (nx * ni)
        J = (gy * nj + j) % (ny * nj)
        K = (gz * nk + k) % (nz * nk)
        f[g] = (I[:, None, None] * (ny * nj) + J[None, :, None]) * (nz * nk) + K[None, None, :]
    return f.ravel()


@pytest.mark.parametrize("layers,corners", [(1, False), (2, False), (2, True), (1, True)])
def test_connect_periodic_images(oracle_lib, layers, corners):
    case = cases.periodic_box(2, 3, 2, n=6)
    o = oracle_lib.Oracle(case, _prm())
    ref = _global_index_field(case)
    f = ref.copy()
    v = case.view(f)
    v[:, :2] = -1; v[:, -2:] = -1; v[:, :, :2] = -1; v[:, :, -2:] = -1
    v[:, :, :, :2] = -1; v[:, :, :, -2:] = -1
    o.set("P", f)
    ncopied = o.connect(0, layers, s1="P", corners=corners)
    n = 6
    face = 6 * n * n * layers
    edges = 12 * n * layers * layers
    corn = 8 * layers ** 3
    assert ncopied == case.ngrid * (face + (edges + corn if corners else 0))
    got = case.view(o.get("P"))
    want = case.view(ref)
    lo, hi = 2 - layers, case.ii - 2 + layers
    sl = slice(lo, hi)
    if corners:
        assert np.array_equal(got[:, sl, sl, sl], want[:, sl, sl, sl])
    else:
        # faces only: the six slabs next to the interior
        it = slice(2, case.ii - 2)
        for a in range(3):
            idx = [slice(None), it, it, it]
            idx[1 + a] = sl
            assert np.array_equal(got[tuple(idx)], want[tuple(idx)])


def test_connect_normal_forward(oracle_lib):
    """connect(1, v1=u, v2=v, v3=w, normal, forward=1) touches exactly the
    low-face ghost plane of the face-normal component (timeintegration_mod.F90:121)."""
    case = cases.periodic_box(2, 2, 2, n=6)
    o = oracle_lib.Oracle(case, _prm())
    ref = _global_index_field(case)
    for nm in "UVW":
        o.set(nm, np.full(case.idim3d, -7.0))
    o.set("U", ref)
    o.set("V", ref * 2)
    o.set("W", ref * 3)
    u0, v0, w0 = ref.copy(), ref * 2, ref * 3
    n = o.connect(0, 1, "U", "V", "W", normal=True, forward=1)
    assert n == case.ngrid * 3 * 36
    for nm, base in zip("UVW", (u0, v0, w0)):
        got = o.get(nm)
        diff = np.nonzero(got != base)[0]
        assert diff.size == 0   # the periodic image values equal the global index field


def test_laplacephi_fourier_eigenvalue(oracle_lib):
    n = 16
    case = cases.periodic_box(2, 1, 1, n=n)
    o = oracle_lib.Oracle(case, _prm())
    xg, yg, zg = case.coords()
    kx, ky, kz = 1.0, 2.0, 3.0
    phi = np.empty((case.ngrid, case.ii, case.jj, case.kk))
    for g in range(case.ngrid):
        phi[g] = (np.cos(kx * xg[g])[:, None, None] * np.cos(ky * yg[g])[None, :, None]
                  * np.cos(kz * zg[g])[None, None, :])
    o.set("HILF", phi.ravel())
    o.laplacephi("RES", "HILF")
    res = case.interior(o.get("RES"))
    hs = (case.dx[0], case.dy[0], case.dz[0])
    lam = sum((2 * np.cos(kq * hq) - 2) / hq ** 2 for kq, hq in zip((kx, ky, kz), hs))
    want = -lam * case.interior(phi.ravel())
    assert np.max(np.abs(res - want)) < 1e-11 * np.max(np.abs(want))


def _solenoidal_streamfunction(case, seed=3):
    """Discretely divergence-free u, v from a stream function psi(x, y) on the
    cell edges, w from a second one in (x, z)."""
    rng = np.random.default_rng(seed)
    ni = case.ii - 4
    nx = case.gridpos[:, 0].max() + 1
    N = nx * ni
    h = case.dx[0]
    modes = [(rng.integers(1, 4), rng.integers(1, 4), rng.normal(), rng.uniform(0, 6.28))
             for _ in range(4)]
    xg, yg, zg = case.coords()
    u = np.zeros((case.ngrid, case.ii, case.jj, case.kk))
    v = np.zeros_like(u)
    w = np.zeros_like(u)

    def psi(X, Y):
        return sum(a * np.sin(p * X + q * Y + ph) for p, q, a, ph in modes)

    for g in range(case.ngrid):
        X = xg[g][:, None, None]
        Y = yg[g][None, :, None]
        Z = zg[g][None, None, :]
        # psi lives at (x+h/2, y+h/2); u at (x+h/2, y), v at (x, y+h/2)
        u[g] = (psi(X + h / 2, Y + h / 2) - psi(X + h / 2, Y - h / 2)) / h + 0 * Z
        v[g] = -(psi(X + h / 2, Y + h / 2) - psi(X - h / 2, Y + h / 2)) / h + 0 * Z
    return u.ravel(), v.ravel(), w.ravel()


def test_convection_conserves_energy(oracle_lib):
    case = cases.periodic_box(2, 2, 1, n=12)
    # gmol tiny: the harmonic face viscosity g*g/max(2g, gmol) stays finite
    o = oracle_lib.Oracle(case, _prm(gmol=1e-300))
    u, v, w = _solenoidal_streamfunction(case)
    for nm, a in zip("UVW", (u, v, w)):
        o.set(nm, a)
    o.set("P", case.zeros())
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    o.divcal("RHS", 1.0)
    assert np.max(np.abs(case.interior(o.get("RHS")))) < 1e-12
    o.tstle4()
    U, V, W = (case.interior(o.get(n)) for n in "UVW")
    UO, VO, WO = (case.interior(o.get(n)) for n in ("UO", "VO", "WO"))
    dke = np.sum(U * UO) + np.sum(V * VO) + np.sum(W * WO)
    scale = np.sum(np.abs(U * UO)) + np.sum(np.abs(V * VO)) + np.sum(np.abs(W * WO))
    assert scale > 1.0
    assert abs(dke) < 1e-13 * scale


def _shear_run(oracle_lib, nsteps, dt, nu=0.05, n=8):
    case = cases.periodic_box(1, 1, 1, n=n)
    o = oracle_lib.Oracle(case, _prm(gmol=nu, epcorr=1e-14, nouter=2, ninner=2))
    xg, yg, zg = case.coords()
    u = np.sin(zg[0])[None, None, :] + 0 * xg[0][:, None, None] + 0 * yg[0][None, :, None]
    o.set("U", u.ravel())
    for nm in "VWP":
        o.set(nm, case.zeros())
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = oracle_lib.rk_scheme("williamson")
    for it in range(1, nsteps + 1):
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, dt, irk, rk)
    h = case.dz[0]
    lam = (2 - 2 * np.cos(h)) / h ** 2
    exact = np.exp(-nu * lam * nsteps * dt) * case.interior(u.ravel())
    return np.max(np.abs(case.interior(o.get("U")) - exact))


def test_rk3_third_order(oracle_lib):
    e1 = _shear_run(oracle_lib, 4, 0.4)
    e2 = _shear_run(oracle_lib, 8, 0.2)
    e3 = _shear_run(oracle_lib, 16, 0.1)
    assert e1 > e2 > e3
    assert 6.0 < e1 / e2 < 10.0
    assert 6.5 < e2 / e3 < 9.5


def _tg2d_error(oracle_lib, n, nu=0.01, t_end=0.2, dt=0.0125):
    case = cases.periodic_box(1, 1, 1, n=n, nk=4)
    o = oracle_lib.Oracle(case, _prm(gmol=nu, epcorr=1e-13, nouter=20, ninner=5))
    xg, yg, zg, xs, ys, zs = cases._stag(case)
    u = cases._eval(case, lambda X, Y, Z: np.sin(X) * np.cos(Y) + 0 * Z, xs, yg, zg)
    v = cases._eval(case, lambda X, Y, Z: -np.cos(X) * np.sin(Y) + 0 * Z, xg, ys, zg)
    p = cases._eval(case, lambda X, Y, Z: 0.25 * (np.cos(2 * X) + np.cos(2 * Y)) + 0 * Z, xg, yg, zg)
    o.set("U", u); o.set("V", v); o.set("W", case.zeros()); o.set("P", p)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = oracle_lib.rk_scheme("williamson")
    nsteps = int(round(t_end / dt))
    for it in range(1, nsteps + 1):
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, dt, irk, rk)
    decay = np.exp(-2 * nu * nsteps * dt)
    return np.max(np.abs(case.interior(o.get("U")) - decay * case.interior(u)))


def test_taylor_green_2d_second_order(oracle_lib):
    e16 = _tg2d_error(oracle_lib, 16)
    e32 = _tg2d_error(oracle_lib, 32)
    assert e32 < e16
    assert 3.0 < e16 / e32 < 5.0


def test_bulk_velocity_conserved(oracle_lib):
    case = cases.periodic_box(2, 2, 2, n=8)
    o = oracle_lib.Oracle(case, _prm(gmol=1e-3))
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=0.05)
    for nm, a in zip("UVWP", (u, v, w, p)):
        o.set(nm, a)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    m0 = [case.interior(o.get(nm)).mean() for nm in "UVW"]
    rk = oracle_lib.rk_scheme("williamson")
    for it in range(1, 4):
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, 2e-3, irk, rk)
    m1 = [case.interior(o.get(nm)).mean() for nm in "UVW"]
    assert np.max(np.abs(np.array(m1) - np.array(m0))) < 1e-13


def test_rk_schemes_consistent(oracle_lib):
    for name, nrk in (("williamson", 3), ("berland", 6), ("carpenter", 5), ("bernardini", 5)):
        rk = oracle_lib.rk_scheme(name)
        assert rk.nrk == nrk
        # consistency: a 2N scheme integrates du/dt = 1 exactly (sum of weights)
        du, u = 0.0, 0.0
        for irk in range(1, nrk + 1):
            frhs, fu, dtrk, dtrki = oracle_lib.rk_coeffs(rk, irk)
            du = frhs * du + 1.0
            u = u + fu * du
            assert abs(u - dtrk) < 1e-9   # stage time of the next stage
        assert abs(u - 1.0) < 1e-9


def test_laplacephi_exact_for_quadratics_on_stretched_grid(oracle_lib):
    """On non-uniform spacing the giteig coefficients form the standard
    three-point second derivative, exact for quadratics: -A (x^2+y^2+z^2) = -6."""
    case = cases.stretch(cases.periodic_box(2, 1, 1, n=10, nj=8, nk=7))
    o = oracle_lib.Oracle(case, _prm())
    xg, yg, zg = case.coords()
    phi = np.empty((case.ngrid, case.ii, case.jj, case.kk))
    for g in range(case.ngrid):
        phi[g] = (xg[g][:, None, None] ** 2 + yg[g][None, :, None] ** 2
                  + zg[g][None, None, :] ** 2)
    o.set("HILF", phi.ravel())
    o.laplacephi("RES", "HILF")
    res = case.interior(o.get("RES"))
    assert np.max(np.abs(res - (-6.0))) < 1e-9
