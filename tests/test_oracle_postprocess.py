"""The oracle's post-processing of a solved field, pinned to exact solutions (CPU).

* pressureStokes (lib_Stokes.f90:4-94): the surface pressure at the element
  centroids from the pressure rows of the integral matrices;
* GetStokesDomainValue (lib_Stokes.f90:3043-3373) and GetSubDomainValue
  (lib_domain.f90:210-391): velocity / pressure and the Laplace field at points
  inside the domain, with the reference's integration check of each point.

References:
* a sphere of radius a at rest inside a concentric spherical container of radius b
  that translates with U e_x: the exact Stokes solution has the stream function
  f(r) sin^2(theta) (theta from e_x) with f = A r^4 + B r^2 + C r + D / r,
  f(a) = f'(a) = 0, f(b) = U b^2 / 2, f'(b) = U b; velocity
  u = (2 f / r^2 - f' / r) cos(theta) e_r + (f' / r) e_x, pressure
  p = mu cos(theta) (20 A r + 2 C / r^2) (the pressure level is free; the solved
  traction carries none, and p is odd in x).  Its drag -8 pi mu C is the concentric
  sphere factor the resistance tests use;
* fields the discretisation holds exactly: u = x + 2y + 3z (Laplace; linear
  elements, flux n.(1, 2, 3) on a polyhedron) and Couette flow u = (z, 0, 0)
  (Stokes, constant pressure) in the unit cube of quads.
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M
from fixtures import reference_mesh

A_PART, B_CONT = 0.5, 50.0


def _concentric_coeffs(a, b, U=1.0):
    Mx = np.array([[a ** 4, a ** 2, a, 1 / a], [4 * a ** 3, 2 * a, 1, -1 / a ** 2],
                   [b ** 4, b ** 2, b, 1 / b], [4 * b ** 3, 2 * b, 1, -1 / b ** 2]])
    return np.linalg.solve(Mx, np.array([0.0, 0.0, U * b * b / 2, U * b]))


def _concentric_field(x, a=A_PART, b=B_CONT, U=1.0, mu=1.0):
    A, B, C, D = _concentric_coeffs(a, b, U)
    r = np.linalg.norm(x)
    ct = x[0] / r
    f = A * r ** 4 + B * r ** 2 + C * r + D / r
    fp = 4 * A * r ** 3 + 2 * B * r + C - D / r ** 2
    u = (2 * f / r ** 2 - fp / r) * ct * x / r + (fp / r) * np.array([1.0, 0.0, 0.0])
    return u, mu * ct * (20 * A * r + 2 * C / r ** 2)


def test_concentric_solution_is_a_stokes_flow():
    """The reference solution itself: no slip on the particle, the container's
    velocity on the container, div u = 0, grad p = mu lap u, and the drag of the
    concentric-sphere factor."""
    a, b = A_PART, B_CONT
    assert np.allclose(_concentric_field(np.array([0.0, a, 0.0]))[0], 0.0, atol=1e-14)
    assert np.allclose(_concentric_field(np.array([0.6 * b, 0.0, 0.8 * b]))[0], [1.0, 0.0, 0.0], atol=1e-12)
    x0, h = np.array([0.8, 0.3, -0.2]), 1e-3
    lap, gp, div = np.zeros(3), np.zeros(3), 0.0
    for k in range(3):
        e = np.zeros(3)
        e[k] = h
        up, u0, um = (_concentric_field(x0 + s * e)[0] for s in (1, 0, -1))
        lap += (up - 2 * u0 + um) / h ** 2
        gp[k] = (_concentric_field(x0 + e)[1] - _concentric_field(x0 - e)[1]) / (2 * h)
        div += (up[k] - um[k]) / (2 * h)
    assert abs(div) < 1e-5 and np.allclose(lap, gp, rtol=1e-4)
    lam = a / b
    C = _concentric_coeffs(a, b)[2]
    factor = (1 - lam ** 5) / (1 - 9 * lam / 4 + 5 * lam ** 3 / 2 - 9 * lam ** 5 / 4 + lam ** 6)
    assert abs(-8 * np.pi * C / (6 * np.pi * a) - factor) < 1e-12


def _sphere_in_sphere(orc, level):
    m = M.particle_in_sphere(M.icosphere(level, radius=A_PART, inward=True, wall=1), outer_level=2,
                             outer_radius=B_CONT)
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    P.form_integrals()
    U = np.zeros((3, len(m["xyz"])))
    U[0, np.unique(m["con"][m["bcid"] == 2, :3])] = 1.0
    q, _, _, ierr = P.stokes_solve_sequence(U[None], maxit=0, eps=1e-12, fwall=1)
    assert ierr == 0
    return m, P, U, q[0]


@pytest.fixture(scope="module")
def spheres(orc):
    out = {lv: _sphere_in_sphere(orc, lv) for lv in (2, 3)}
    yield out
    for _, P, _, _ in out.values():
        P.close()


def _fluid_points(n=40, seed=1):
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < n:
        x = rng.uniform(-3.0, 3.0, 3)
        if 1.5 * A_PART < np.linalg.norm(x) < 3.0:
            pts.append(x)
    return np.array(pts)


def test_stokes_domain_values_concentric_spheres(spheres):
    """Velocity and pressure in the fluid (0.75 to 3 from the centre): second-order
    convergence to the exact solution (level 2 -> 3 halves the element size)."""
    pts = _fluid_points()
    exact = [_concentric_field(x) for x in pts]
    ue = np.array([e[0] for e in exact])
    pe = np.array([e[1] for e in exact])
    dev = {}
    for lv, (m, P, U, q) in spheres.items():
        vals, err = P.domain_values(pts, U, q)
        assert np.all(err < 1e-6)  # every point is inside the fluid
        dev[lv] = (np.max(np.abs(vals[:, :3] - ue)), np.max(np.abs(vals[:, 3] - pe)))
    assert dev[2][0] < 1.2e-2 and dev[2][1] < 1e-2
    assert dev[3][0] < 3e-3 and dev[3][1] < 2.5e-3
    assert dev[2][0] / dev[3][0] > 3.0 and dev[2][1] / dev[3][1] > 3.0


def test_stokes_domain_point_check_flags_outside(spheres):
    """getStokesDV (lib_Stokes.f90:3020-3035) rejects a point whose check exceeds
    1e-2: points inside the particle or beyond the container (the stresslet
    diagonal sums to 0 there, not 8 pi)."""
    m, P, U, q = spheres[2]
    _, err = P.domain_values(np.array([[0.0, 0.0, 0.1], [0.2, -0.1, 0.0], [0.0, 0.0, 60.0]]), U, q)
    assert np.all(err > 1e-2)


def test_stokes_surface_pressure_concentric_spheres(spheres):
    """pressureStokes on the particle against the exact surface pressure
    -(3/2) mu U cos(theta) / a x (container factor): first-order convergence (the
    self element's pressure integrals are left out, as in the reference)."""
    rms = {}
    for lv, (m, P, U, q) in spheres.items():
        p = P.pressure(U, q)
        sel = m["bcid"] == 1
        cen = m["xyz"][m["con"][sel, :3]].mean(axis=1)
        on_sphere = cen / np.linalg.norm(cen, axis=1)[:, None] * A_PART
        pe = np.array([_concentric_field(x)[1] for x in on_sphere])
        rms[lv] = np.sqrt(np.mean((p[sel] - pe) ** 2))
        assert abs(np.mean(p[sel])) < 1e-8  # no pressure level in the solved traction
    assert rms[2] < 0.2 and rms[3] < 0.1  # of a peak pressure of 3
    assert rms[2] / rms[3] > 1.7


def test_couette_quad_box_pressure_and_domain(orc):
    """Couette flow u = (z, 0, 0) on the unit cube of 4 x 4 x 4 quads per face:
    a uniform surface pressure, and the velocity and pressure inside reproduced."""
    mb = M.quad_box(4, 4, 4, face_walls=True)
    P = orc.Problem(2, mb, walls=[1, 2, 3, 4, 5, 6], known=np.ones((3, 6)), itri=5)
    P.form_integrals()
    U = np.zeros((3, len(mb["xyz"])))
    U[0] = mb["xyz"][:, 2]
    q, _, _, ierr = P.stokes_solve_sequence(U[None], maxit=0, eps=1e-13, fwall=1)
    p = P.pressure(U, q[0])
    assert np.max(p) - np.min(p) < 1e-9
    pts = np.array([[0.5, 0.5, 0.5], [0.2, 0.7, 0.4], [0.7, 0.3, 0.6], [0.5, 0.5, 0.8]])
    vals, err = P.domain_values(pts, U, q[0])
    P.close()
    assert np.all(err < 1e-5)
    want = np.zeros((len(pts), 3))
    want[:, 0] = pts[:, 2]
    assert np.max(np.abs(vals[:, :3] - want)) < 1e-5
    assert np.max(np.abs(vals[:, 3] - np.mean(p))) < 1e-5


def test_laplace_domain_values_sphere01(orc):
    """The reference's Laplace sphere (run/mesh/sphere-01.msh) with u = x + 2y + 3z:
    the field inside from the solved boundary flux."""
    m = reference_mesh("sphere_01")
    g = np.array([1.0, 2.0, 3.0])
    P = orc.Problem(1, m, walls=[1], known=[[1]], itri=5)
    P.form_integrals()
    u = m["xyz"] @ g
    _, q, _, ierr = P.laplace_solve(u, np.zeros(P.nelem), maxit=0, eps=1e-12)
    pts = np.array([[0.0, 0.0, 0.0], [0.1, 0.2, -0.1], [0.3, 0.0, 0.1], [-0.2, -0.25, 0.2]])
    v, err = P.domain_values(pts, u, q)
    P.close()
    assert ierr == 0 and np.all(err < 1e-8)
    assert np.max(np.abs(v - pts @ g)) < 1e-8


def test_laplace_domain_values_quad_box(orc):
    """Quads (the one-cell regular rule of Quad_BEMInt): u = x + 2y + 3z in the unit cube."""
    mb = M.quad_box(4, 4, 4)
    g = np.array([1.0, 2.0, 3.0])
    P = orc.Problem(1, mb, walls=[1], known=[[1]], itri=5)
    P.form_integrals()
    u = mb["xyz"] @ g
    _, q, _, ierr = P.laplace_solve(u, np.zeros(P.nelem), maxit=0, eps=1e-12)
    pts = np.array([[0.5, 0.5, 0.5], [0.2, 0.7, 0.4], [0.7, 0.3, 0.6]])
    v, err = P.domain_values(pts, u, q)
    P.close()
    assert ierr == 0 and np.all(err < 1e-6)
    assert np.max(np.abs(v - pts @ g)) < 1e-6
