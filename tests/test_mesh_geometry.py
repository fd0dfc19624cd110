"""Bodies given as triangles (STL): the library's mesh signed distance
(mglet_mesh_create / mglet_mesh_distance) against a brute-force closest
triangle search written here in numpy, STL files read back as written, and
a sphere channel sample whose body comes from an STL file: blocking,
stencil lists and one RK3 step on the oracle."""
import numpy as np
import pytest

from mglet_gb300 import abi, channel, geometry


def _closest_all(p, T):
    """Distance from p to every triangle of T (n, 3, 3), by projecting onto
    the plane and clamping to the edges where the projection falls outside."""
    a, b, c = T[:, 0], T[:, 1], T[:, 2]
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    q = p - np.sum((p - a) * n, axis=1, keepdims=True) * n

    def inside(q):
        s = []
        for u, v in ((a, b), (b, c), (c, a)):
            s.append(np.sum(np.cross(v - u, q - u) * n, axis=1) >= 0)
        return s[0] & s[1] & s[2]

    def seg(u, v):
        d = v - u
        t = np.clip(np.sum((p - u) * d, axis=1) / np.sum(d * d, axis=1), 0.0, 1.0)
        return np.linalg.norm(p - (u + t[:, None] * d), axis=1)

    dp = np.linalg.norm(p - q, axis=1)
    de = np.minimum(np.minimum(seg(a, b), seg(b, c)), seg(c, a))
    return np.where(inside(q), dp, de)


@pytest.fixture(scope="module")
def sphere_mesh():
    return geometry.icosphere((0.5, 0.5, 0.5), 0.2, level=3)


def test_distance_matches_brute_force(sphere_mesh):
    m = geometry.Mesh(sphere_mesh)
    rng = np.random.default_rng(3)
    P = np.concatenate([rng.uniform(0.0, 1.0, (150, 3)), rng.uniform(0.25, 0.75, (150, 3))])
    phi = m.phi(P[:, 0], P[:, 1], P[:, 2])
    for p, f in zip(P, phi):
        d = _closest_all(p, sphere_mesh).min()
        assert abs(abs(f) - d) <= 1e-12 * max(1.0, d)
    # the sign: inside the (convex) mesh exactly when inside its inscribed test
    r = np.linalg.norm(P - 0.5, axis=1)
    assert np.all(phi[r < 0.19] < 0) and np.all(phi[r > 0.201] > 0)


def test_normals_point_out_and_planes_touch(sphere_mesh):
    m = geometry.Mesh(sphere_mesh)
    P = np.array([[0.5, 0.5, 0.9], [0.5, 0.5, 0.55], [0.1, 0.5, 0.5], [0.62, 0.61, 0.5]])
    pl = m.plane(P[:, 0], P[:, 1], P[:, 2])
    n, dpl = pl[:, :3], pl[:, 3]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0)
    radial = (P - 0.5) / np.linalg.norm(P - 0.5, axis=1, keepdims=True)
    assert np.all(np.sum(n * radial, axis=1) > 0.9)
    # the plane's signed distance at P equals the mesh distance
    phi = m.phi(P[:, 0], P[:, 1], P[:, 2])
    assert np.allclose(np.sum(n * P, axis=1) - dpl, phi, atol=1e-12)


@pytest.mark.parametrize("binary", [True, False])
def test_stl_round_trip(tmp_path, sphere_mesh, binary):
    path = tmp_path / ("s.stl" if binary else "a.stl")
    geometry.write_stl(str(path), sphere_mesh, binary=binary)
    back = geometry.read_stl(str(path))
    tol = 1e-6 if binary else 0.0     # binary STL stores single precision
    assert back.shape == sphere_mesh.shape
    assert np.max(np.abs(back - sphere_mesh)) <= tol


def test_channel_from_an_stl_body(tmp_path, oracle_lib, sphere_mesh):
    """The bounded sphere-channel sample with its body read from STL: the
    blocking agrees with the analytic sphere's away from the surface, the
    library builds the lists, and one RK3 step on the oracle stays finite."""
    sc = channel.SphereChannel(tiles=(4, 2, 2), n=8, grid_size=0.5, diameter=0.4,
                               refine_radii=(0.35,))
    tris = geometry.icosphere(sc.center, 0.2, level=3)
    path = tmp_path / "sphere.stl"
    geometry.write_stl(str(path), tris, binary=False)
    body = geometry.Mesh(geometry.read_stl(str(path)))
    geo = geometry.block(sc.case, body)
    ref = sc.geo
    frac = np.mean(geo["bp"] != ref["bp"])
    assert 0.0 <= frac < 2e-3
    assert geo["icells"].sum() > 0
    sc.geo, sc._lists = geo, None
    prm = sc.flow_params(nouter=6, ninner=5, nouter_min=6)
    o = oracle_lib.Oracle(sc.case, prm)
    sc.setup(o)
    rk = oracle_lib.rk_scheme("williamson")
    for irk in (1, 2, 3):
        st = o.timeintegrate_flow(1, 1, 0.0, sc.dt(), irk, rk)
        assert np.isfinite(st.maxrhs)
    assert not o.itinfo(sc.dt()).exploded
