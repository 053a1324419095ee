"""The synthetic workloads' geometry on the CPU: the many-body set (seeded
superellipsoids with log-uniform element counts), the superellipsoid surface
itself, orientation of particle and container normals, random rotations and the
box of quads."""
import numpy as np

from andromeda_gb300 import mesh as M


def _signed_volume(m, wall=None):
    """sum over elements of area * (centroid . n) / 3 (divergence theorem): the
    enclosed volume for outward normals, minus it for inward ones."""
    x, c = m["xyz"], m["con"]
    sel = np.ones(len(c), bool) if wall is None else (m["bcid"] == wall)
    tri = c[sel, :3]
    a, b, d = x[tri[:, 0]], x[tri[:, 1]], x[tri[:, 2]]
    return float(np.sum(np.einsum("ij,ij->i", a, np.cross(b - a, d - a))) / 6.0)


def test_batch_bodies_match_the_workload_definition():
    meshes, params = M.batch_bodies(n_bodies=64)
    assert len(meshes) == 64 and params.shape == (64, 5)
    b, c, e1, e2, n = params.T
    assert np.all((b >= 0.2) & (b <= 1.0) & (c >= 0.2) & (c <= 1.0))
    assert np.all((e1 >= 0.3) & (e1 <= 1.8) & (e2 >= 0.3) & (e2 <= 1.8))
    assert np.all((n >= 0.8 * 500) & (n <= 1.2 * 8000))
    # seeded: the same call gives the same bodies
    meshes2, params2 = M.batch_bodies(n_bodies=64)
    assert np.array_equal(params, params2)
    assert all(np.array_equal(m1["xyz"], m2["xyz"]) for m1, m2 in zip(meshes[:4], meshes2[:4]))
    for m, p in zip(meshes[:8], params[:8]):
        assert set(np.unique(m["bcid"])) == {1, 2}
        assert (m["bcid"] == 1).sum() == int(p[4])
        assert _signed_volume(m, wall=1) < 0  # particle normals point into the particle
        assert _signed_volume(m, wall=2) > 0  # container normals point out of the fluid


def test_batch_element_counts_are_log_uniform():
    _, params = M.batch_bodies(n_bodies=512)
    n = params[:, 4]
    # E[N] of log-uniform [500, 8000]: (8000 - 500) / ln 16 = 2705
    assert abs(np.mean(n) / 2705.0 - 1.0) < 0.1
    q = np.log(n / 500.0) / np.log(16.0)
    assert abs(np.mean(q) - 0.5) < 0.05 and abs(np.std(q) - np.sqrt(1 / 12)) < 0.03


def test_superellipsoid_nodes_on_the_surface():
    a, b, c, e1, e2 = 1.0, 0.5, 0.25, 0.6, 1.4
    m = M.superellipsoid(a, b, c, e1, e2, 20, 40)
    x, y, z = np.abs(m["xyz"]).T
    F = ((x / a) ** (2 / e2) + (y / b) ** (2 / e2)) ** (e2 / e1) + (z / c) ** (2 / e1)
    assert np.max(np.abs(F - 1.0)) < 1e-9
    assert _signed_volume(m) > 0  # outward by default


def test_random_rotation_is_proper_orthogonal():
    rng = np.random.default_rng(2)
    for _ in range(10):
        Q = M.random_rotation(rng)
        assert np.allclose(Q @ Q.T, np.eye(3), atol=1e-12)
        assert abs(np.linalg.det(Q) - 1.0) < 1e-12


def test_quad_box_outward_and_closed():
    m = M.quad_box(3, 2, 4, lo=(0.0, 0.0, 0.0), hi=(1.5, 1.0, 0.5))
    assert len(m["etype"]) == 2 * (3 * 2 + 2 * 4 + 3 * 4)
    x, c = m["xyz"], m["con"]
    # the two triangles (1,2,3) and (1,3,4) of each quad: the enclosed volume
    vol = 0.0
    for tri in (c[:, [0, 1, 2]], c[:, [0, 2, 3]]):
        a, b, d = x[tri[:, 0]], x[tri[:, 1]], x[tri[:, 2]]
        vol += np.sum(np.einsum("ij,ij->i", a, np.cross(b - a, d - a))) / 6.0
    assert abs(vol - 1.5 * 1.0 * 0.5) < 1e-12
