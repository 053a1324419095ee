"""GPU surface pressure and values inside the domain (agb_surface_pressure,
agb_domain_values) against the oracle's restatements of pressureStokes,
GetStokesDomainValue and GetSubDomainValue, on the same boundary fields (the
oracle's solutions), FP64 on both sides: 1e-10 relative to the largest value
(only the summation order differs: per element here, per node in the reference).
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M
from fixtures import reference_mesh

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b))


def _sphere_case(orc, level=2, R=50.0):
    m = M.particle_in_sphere(M.icosphere(level, radius=0.5, inward=True, wall=1), outer_level=2, outer_radius=R)
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    P.form_integrals()
    U = np.zeros((3, len(m["xyz"])))
    U[0, np.unique(m["con"][m["bcid"] == 2, :3])] = 1.0
    q, _, _, _ = P.stokes_solve_sequence(U[None], maxit=0, eps=1e-12, fwall=1)
    return m, P, U, q[0]


def _gpu_ctx(agb, m, kind, walls, known):
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(kind, walls, known, itri=5)
    return C


def test_surface_pressure_matches_oracle(agb, orc):
    m, P, U, q = _sphere_case(orc)
    p_ref = P.pressure(U, q)
    _, ql = P.lists()
    P.close()
    want = np.zeros(len(m["etype"]))
    want[ql] = p_ref  # row r of the oracle is subdomain element ql[r]
    C = _gpu_ctx(agb, m, agb.STOKES, [1, 2], agb.dirichlet_known(agb.STOKES, 2))
    p = C.surface_pressure(U, q)
    C.close()
    assert _rel(p, want) < 1e-10


def test_stokes_domain_values_match_oracle(agb, orc):
    m, P, U, q = _sphere_case(orc)
    rng = np.random.default_rng(3)
    pts = rng.uniform(-2.0, 2.0, (24, 3))
    pts = pts[np.linalg.norm(pts, axis=1) > 0.7]
    pts = np.vstack([pts, [[0.0, 0.0, 0.1], [0.0, 0.0, 60.0]]])  # inside the particle, beyond the container
    ref, err_ref = P.domain_values(pts, U, q)
    P.close()
    C = _gpu_ctx(agb, m, agb.STOKES, [1, 2], agb.dirichlet_known(agb.STOKES, 2))
    got, err = C.domain_values(pts, U, q)
    C.close()
    assert _rel(got, ref) < 1e-10
    assert np.allclose(err, err_ref, rtol=1e-8, atol=1e-12)
    assert np.all(err[:-2] < 1e-6) and np.all(err[-2:] > 1e-2)


def test_couette_quads_domain_and_pressure(agb, orc):
    mb = M.quad_box(4, 4, 4, face_walls=True)
    walls = [1, 2, 3, 4, 5, 6]
    P = orc.Problem(2, mb, walls=walls, known=np.ones((3, 6)), itri=5)
    P.form_integrals()
    U = np.zeros((3, len(mb["xyz"])))
    U[0] = mb["xyz"][:, 2]
    q, _, _, _ = P.stokes_solve_sequence(U[None], maxit=0, eps=1e-13, fwall=1)
    pts = np.array([[0.5, 0.5, 0.5], [0.2, 0.7, 0.4], [0.7, 0.3, 0.6]])
    ref, err_ref = P.domain_values(pts, U, q[0])
    p_ref = P.pressure(U, q[0])
    _, ql = P.lists()
    P.close()
    C = _gpu_ctx(agb, mb, agb.STOKES, walls, agb.dirichlet_known(agb.STOKES, 6))
    got, err = C.domain_values(pts, U, q[0])
    p = C.surface_pressure(U, q[0])
    C.close()
    assert _rel(got[:, :3], ref[:, :3]) < 1e-10
    assert np.max(np.abs(got[:, 3] - ref[:, 3])) < 1e-10 * max(1.0, np.max(np.abs(ref[:, 3])))
    want = np.zeros(len(mb["etype"]))
    want[ql] = p_ref
    assert np.max(np.abs(p - want)) < 1e-10 * max(1.0, np.max(np.abs(want)))


@pytest.mark.parametrize("mesh", ["sphere_01", "quad_box"])
def test_laplace_domain_values_match_oracle(agb, orc, mesh):
    m = reference_mesh("sphere_01") if mesh == "sphere_01" else M.quad_box(4, 4, 4)
    g = np.array([1.0, 2.0, 3.0])
    P = orc.Problem(1, m, walls=[1], known=[[1]], itri=5)
    P.form_integrals()
    u = m["xyz"] @ g
    _, q, _, _ = P.laplace_solve(u, np.zeros(P.nelem), maxit=0, eps=1e-12)
    c = m["xyz"].mean(axis=0)
    pts = c + np.array([[0.0, 0.0, 0.0], [0.1, 0.2, -0.1], [0.3, 0.0, 0.1], [-0.2, -0.25, 0.2]])
    ref, err_ref = P.domain_values(pts, u, q)
    P.close()
    C = _gpu_ctx(agb, m, agb.LAPLACE, [1], agb.dirichlet_known(agb.LAPLACE, 1))
    got, err = C.domain_values(pts, u[None], q[None])
    C.close()
    assert _rel(got, ref) < 1e-10
    assert np.max(np.abs(got - pts @ g)) < 1e-6
