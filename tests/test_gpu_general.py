"""GPU parity of the general path: integral matrices of every source row
(CoR_Integrals / CoR_Integrals_Stokes drop-in), mixed boundary conditions,
quads, against the FP64 oracle.

Tolerances: integral matrices and self-check errors 1e-12 relative to the
largest entry (FP64 on both sides, only the summation order of the row sums
differs); solutions of mixed-BC problems 1e-10 relative (both solved to eps 1e-13).
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _ctx(agb, m, kind, walls, known, itri=5, iqud=4, normMul=None):
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(kind, walls, known, normMul=normMul, itri=itri, iqud=iqud)
    return C


@pytest.mark.parametrize("triangles", [False, True])
def test_laplace_integral_matrices(agb, orc, triangles):
    m = M.quad_box(3, 2, 2, hi=(1.5, 1.0, 0.8), face_walls=True, triangles=triangles)
    walls = [1, 2, 3, 4, 5, 6]
    known = [[1, 1, 2, 2, 2, 2]]
    P = orc.Problem(1, m, walls=walls, known=known, itri=5, iqud=4)
    e_ref = P.form_integrals()
    C = _ctx(agb, m, agb.LAPLACE, walls, known)
    T, G, e = C.integral_matrices()
    assert _rel(T[0], P.integral_matrix(0)) < 1e-12
    assert _rel(G[0], P.integral_matrix(1)) < 1e-12
    assert abs(e[0] - e_ref[0]) <= 1e-12 * max(1.0, abs(e_ref[0]))
    assert abs(e[1] - e_ref[1]) <= 1e-12 * max(1.0, abs(e_ref[1]))


@pytest.mark.parametrize("case", ["sphere_tri", "box_quad"])
def test_stokes_integral_matrices(agb, orc, case):
    if case == "sphere_tri":
        m = M.particle_in_sphere(M.icosphere(1, 1.0, inward=True), outer_level=1, outer_radius=6.0)
        walls = [1, 2]
    else:
        m = M.quad_box(2, 2, 2, hi=(2.0, 1.0, 1.0), face_walls=True)
        walls = [1, 2, 3, 4, 5, 6]
    known = np.ones((3, len(walls)), np.int32)
    P = orc.Problem(2, m, walls=walls, known=known, itri=5, iqud=4)
    e_ref = P.form_integrals()
    C = _ctx(agb, m, agb.STOKES, walls, known)
    T, G, e = C.integral_matrices()
    for k in range(9):
        ref = P.integral_matrix(k)
        scale = max(np.max(np.abs(ref)), 1e-300)
        assert np.max(np.abs(T[k] - ref)) / scale < 1e-12, k
        refg = P.integral_matrix(9 + k)
        scale = max(np.max(np.abs(refg)), 1e-300)
        assert np.max(np.abs(G[k] - refg)) / scale < 1e-12, k
    assert abs(e[0] - e_ref[0]) <= 1e-10 * max(1.0, abs(e_ref[0]))
    assert abs(e[1] - e_ref[1]) <= 1e-10 * max(1.0, abs(e_ref[1]))


@pytest.mark.parametrize("triangles", [False, True])
def test_laplace_mixed_bc_solve(agb, orc, triangles):
    """Box: u known on the x-faces, flux known elsewhere, u = x + 2y + 3z."""
    m = M.quad_box(3, 3, 3, hi=(1.2, 1.0, 1.1), face_walls=True, triangles=triangles)
    walls = [1, 2, 3, 4, 5, 6]
    known = [[1, 1, 2, 2, 2, 2]]
    P = orc.Problem(1, m, walls=walls, known=known, itri=5, iqud=4)
    n, _, _ = P.geometry()
    g = np.array([1.0, 2.0, 3.0])
    u = m["xyz"] @ g
    q = -(n @ g)
    # known values (and the warm start of the unknowns): the exact fields
    u0, q0 = u.copy(), q.copy()
    u_ref, q_ref, nit_ref, ierr = P.laplace_solve(u0, q0, maxit=0, eps=1e-13)
    C = _ctx(agb, m, agb.LAPLACE, walls, known)
    C.assemble(agb.FP64)
    uo, qo, nit, istop = C.solve_fields(u0[None, None], q0[None, None], eps=1e-13)
    assert istop[0] <= 3
    assert _rel(uo[0, 0], u_ref) < 1e-10
    assert _rel(qo[0, 0], q_ref) < 1e-10
    # the discrete solution reproduces the linear field on the flux walls
    flux_nodes = np.unique(m["con"][~np.isin(m["bcid"], [1, 2])][:, :3])
    assert np.max(np.abs(uo[0, 0, flux_nodes] - u[flux_nodes])) < 5e-3 * np.max(np.abs(u))


def test_stokes_mixed_bc_solve(agb, orc):
    """Box channel: velocity known on x-, y-, y+, z-, z+ walls, traction-free x+."""
    m = M.quad_box(3, 2, 2, hi=(2.0, 1.0, 1.0), face_walls=True, triangles=True)
    walls = [1, 2, 3, 4, 5, 6]
    known = np.ones((3, 6), np.int32)
    known[:, 1] = 2  # x+ : traction known (zero)
    nn = len(m["xyz"])
    U = np.zeros((1, 3, nn))
    inlet = np.unique(m["con"][m["bcid"] == 1][:, :3])
    y, z = m["xyz"][inlet, 1], m["xyz"][inlet, 2]
    U[0, 0, inlet] = 16 * y * (1 - y) * z * (1 - z)
    P = orc.Problem(2, m, walls=walls, known=known, itri=5, iqud=4)
    P.form_integrals()
    q_ref, ft_ref, nits, ierr = P.stokes_solve_sequence(U, maxit=0, eps=1e-13, fwall=1)
    C = _ctx(agb, m, agb.STOKES, walls, known)
    C.assemble(agb.FP64)
    uo, qo, nit, istop = C.solve_fields(U, None, eps=1e-13)
    assert istop[0] <= 3
    assert _rel(qo[0], q_ref[0]) < 1e-10


def test_general_path_mixed_precision(agb):
    """A Stokes quad mesh goes through the general path; the FP32 copy of the
    routed system solves to the FP64 answer within 1e-5."""
    m = M.quad_box(2, 2, 2, hi=(2.0, 1.0, 1.0), face_walls=True)
    walls = [1, 2, 3, 4, 5, 6]
    known = np.ones((3, 6), np.int32)
    known[:, 1] = 2
    nn = len(m["xyz"])
    U = np.zeros((1, 3, nn))
    inlet = np.unique(m["con"][m["bcid"] == 1][:, :4])
    U[0, 0, inlet] = 1.0
    C = _ctx(agb, m, agb.STOKES, walls, known)
    C.assemble(agb.FP64)
    _, q64, _, _ = C.solve_fields(U, None, eps=1e-12)
    C.assemble(agb.MIXED)
    _, q32, _, _ = C.solve_fields(U, None, eps=1e-9)
    assert _rel(q32, q64) < 1e-5
