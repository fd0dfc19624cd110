"""The body-force source term and the discrete adjoint on the GPU.

* The body force enters tstle4 after gradp: stages with it match the oracle
  bit for bit.
* dJ/df of the final kinetic energy, from mglet_gpu_energy_gradient (the
  adjoint with checkpoint-and-recompute), against central finite
  differences of the oracle's forward solver along seeded random directions
  (h = 1e-6, relative error <= 1e-6), on a Taylor-Green field with noise so
  that the linearised convection, diffusion, pressure solve and projection
  all carry weight.  The pressure solve runs a fixed number of outer
  iterations, so that J is a smooth function of f.
* Two runs give the same gradient bit for bit (no atomics).
* The same gradient through a thin torch.autograd.Function, as a gradient
  check harness would use it.
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases

pytestmark = pytest.mark.gpu


def _prm(gmol=5e-3, nouter=20):
    return abi.make_flow_params(gmol=gmol, epcorr=1e-30, nouter=nouter, ninner=5, nouter_min=nouter)


def _case():
    return cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))


def _fields(case, seed=3):
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=5e-2, seed=seed)
    return dict(zip("UVWP", (u, v, w, p)))


def _force(case, seed=4, rms=0.1):
    rng = np.random.default_rng(seed)
    return [rms * rng.standard_normal(case.idim3d) for _ in range(3)]


def _load(s, fields, f):
    for n, a in fields.items():
        s.set(n, a)
    s.set_body_force(*f)
    s.connect(0, 2, "U", "V", "W", "P", corners=True)


def _oracle_energy(oracle_lib, case, prm, fields, f, nsteps, dt):
    o = oracle_lib.Oracle(case, prm)
    _load(o, fields, f)
    rk = oracle_lib.rk_scheme("williamson")
    for it in range(1, nsteps + 1):
        for irk in (1, 2, 3):
            o.timeintegrate_flow(it, it, 0.0, dt, irk, rk)
    return o.itinfo(dt).energy


def test_body_force_stages_bit_exact(gpu_lib, oracle_lib):
    case = _case()
    prm = _prm(nouter=6)
    fields, f = _fields(case), _force(case)
    gs, o = gpu_lib.Solver(case, prm), oracle_lib.Oracle(case, prm)
    for s in (gs, o):
        _load(s, fields, f)
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        gs.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
        o.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
    for n in "UVWP":
        assert np.array_equal(gs.get(n), o.get(n)), n


@pytest.mark.parametrize("nsteps,ncheck", [(3, 2), (4, 1)])
def test_energy_gradient_matches_finite_differences(gpu_lib, oracle_lib, nsteps, ncheck):
    case = _case()
    prm = _prm()
    dt = 2e-2
    fields, f = _fields(case), _force(case)
    gs = gpu_lib.Solver(case, prm)
    _load(gs, fields, f)
    J, grad = gs.energy_gradient(nsteps, ncheck, dt, oracle_lib.rk_scheme("williamson"))
    # the run leaves the final forward state: J equals the oracle's energy
    J0 = _oracle_energy(oracle_lib, case, prm, fields, f, nsteps, dt)
    assert abs(J - J0) <= 1e-13 * abs(J0)
    assert gs.itinfo(dt).energy == J
    rng = np.random.default_rng(9)
    h = 1e-6
    for _ in range(3):
        d = [rng.standard_normal(case.idim3d) for _ in range(3)]
        fp = [a + h * b for a, b in zip(f, d)]
        fm = [a - h * b for a, b in zip(f, d)]
        fd = (_oracle_energy(oracle_lib, case, prm, fields, fp, nsteps, dt)
              - _oracle_energy(oracle_lib, case, prm, fields, fm, nsteps, dt)) / (2 * h)
        ad = sum(float(np.dot(g, b)) for g, b in zip(grad, d))
        assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)


def test_energy_gradient_is_reproducible(gpu_lib, oracle_lib):
    """The adjoint adds its scattered derivatives without atomics (the flux
    transpose in 27 colour classes, the connect transpose grouped by source
    grid), so two runs from the same state give the same gradient bit for
    bit, on a tiling where every grid both sends and receives copies."""
    case = cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0))
    prm = _prm()
    fields, f = _fields(case), _force(case)
    out = []
    for _ in range(2):
        gs = gpu_lib.Solver(case, prm)
        _load(gs, fields, f)
        J, grad = gs.energy_gradient(3, 1, 2e-2, oracle_lib.rk_scheme("williamson"))
        out.append((J, [g.copy() for g in grad], gs.get("LU")))
        gs.close()
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[0][2], out[1][2])


def test_adjoint_stage_refuses_walls(gpu_lib, oracle_lib):
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0), walls={5: abi.BC_NOS, 6: abi.BC_NOS})
    gs = gpu_lib.Solver(case, _prm())
    with pytest.raises(gpu_lib.MgletError):
        gs.adjoint_rk_stage(1, 1e-2, oracle_lib.rk_scheme("williamson"))


def test_torch_autograd_harness(gpu_lib, oracle_lib):
    """dJ/df through torch.autograd: the Function's backward hands back the
    adjoint's gradient, and a directional derivative of J taken by autograd
    matches the oracle's central difference."""
    torch = pytest.importorskip("torch")
    case = _case()
    prm = _prm()
    dt, nsteps = 2e-2, 2
    fields = _fields(case)

    class EnergyOfForce(torch.autograd.Function):
        @staticmethod
        def forward(ctx, fx, fy, fz):
            s = gpu_lib.Solver(case, prm)
            _load(s, fields, [t.detach().cpu().numpy() for t in (fx, fy, fz)])
            J, g = s.energy_gradient(nsteps, 1, dt, oracle_lib.rk_scheme("williamson"))
            ctx.save_for_backward(*[torch.from_numpy(a) for a in g])
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            return tuple(gJ * t for t in ctx.saved_tensors)

    f = [torch.tensor(a, dtype=torch.float64, requires_grad=True) for a in _force(case, seed=5)]
    J = EnergyOfForce.apply(*f)
    J.backward()
    rng = np.random.default_rng(10)
    d = [rng.standard_normal(case.idim3d) for _ in range(3)]
    ad = sum(float(torch.dot(t.grad, torch.from_numpy(b))) for t, b in zip(f, d))
    h = 1e-6
    fn = [t.detach().numpy() for t in f]
    fd = (_oracle_energy(oracle_lib, case, prm, fields, [a + h * b for a, b in zip(fn, d)], nsteps, dt)
          - _oracle_energy(oracle_lib, case, prm, fields, [a - h * b for a, b in zip(fn, d)], nsteps, dt)) / (2 * h)
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
