"""GPU parity tests: the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances (written here, per quantity):
* FP64 GPU path vs oracle: system matrix and right-hand sides 1e-12 relative to
  the largest entry; converged solutions / force / torque 1e-10 relative
  (both solved to eps 1e-13, so the converged least-squares solution -- not the
  iterate path -- is compared).
* CRS drop-in (agb_lsqr_precon/agb_lsqr_solve) vs the oracle's lsqr: scaling
  and matrix bit-for-bit up to 1 ulp, solution 1e-10.
* Mixed path: matrix 2e-6 relative to the largest entry of its row block,
  resistance tensor 1e-5 relative to its largest entry vs the FP64 GPU path.
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _ctx(agb, mesh, kind, walls, itri=5, iqud=4):
    C = agb.Context(0)
    C.set_mesh(mesh)
    C.set_problem(kind, walls, agb.dirichlet_known(kind, len(walls)), itri=itri, iqud=iqud)
    return C


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _sis(level_in=1, level_out=1, a=1.0, b=8.0):
    return M.particle_in_sphere(M.icosphere(level_in, a, inward=True), outer_level=level_out, outer_radius=b)


def _rigid_fields(m, outer_wall=2):
    nn = len(m["xyz"])
    on = np.zeros(nn, bool)
    for e in np.where(m["bcid"] == outer_wall)[0]:
        on[m["con"][e, :3]] = True
    U = np.zeros((6, 3, nn))
    for i in range(3):
        U[i, i, on] = 1.0
        w = np.zeros(3)
        w[i] = 1.0
        U[3 + i][:, on] = np.cross(w, m["xyz"][on]).T
    return U


def test_geometry_parity(agb, orc):
    m = _sis(1, 1)
    C = _ctx(agb, m, agb.STOKES, [1, 2])
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)))
    n1, a1, c1 = C.geometry()
    n2, a2, c2 = P.geometry()
    assert np.max(np.abs(n1 - n2)) < 1e-15
    assert np.max(np.abs(a1 - a2) / a2) < 1e-15
    assert np.max(np.abs(c1 - c2)) < 1e-15


def test_geometry_parity_quads(agb, orc):
    m = M.quad_box(3, 2, 2, hi=(2.0, 1.5, 1.0))
    C = _ctx(agb, m, agb.LAPLACE, [1])
    P = orc.Problem(1, m, walls=[1], known=[[1]])
    n1, a1, c1 = C.geometry()
    n2, a2, c2 = P.geometry()
    assert np.max(np.abs(n1 - n2)) < 1e-15
    assert np.max(np.abs(a1 - a2) / a2) < 1e-14
    assert np.max(np.abs(c1 - c2)) < 1e-15


@pytest.mark.parametrize("itri", [1, 5])
def test_laplace_c1_system_rhs_solution(agb, orc, itri):
    """Config 1: unit icosphere L3 (1280 triangles), u = x+2y+3z, FP64."""
    m = M.icosphere(3)
    u = m["xyz"] @ np.array([1.0, 2.0, 3.0])
    P = orc.Problem(1, m, walls=[1], known=[[1]], itri=itri)
    P.form_integrals()
    P.form_system()
    S = P.dense(0)
    R = P.dense(1)
    nl, _ = P.lists()
    b_ref = R @ (-u[nl])
    C = _ctx(agb, m, agb.LAPLACE, [1], itri=itri)
    C.assemble(agb.FP64)
    A, q = C.system(scaled=False)
    assert _rel(A, S) < 1e-12
    rhs = C.rhs(u[None])
    assert _rel(rhs[0], b_ref) < 1e-12
    _, q_ref, nit_ref, ierr = P.laplace_solve(u, np.zeros(P.nelem), maxit=0, eps=1e-13)
    x, nit, istop = C.solve(u[None], eps=1e-13)
    assert istop[0] <= 3
    assert _rel(x[0], q_ref) < 1e-10
    n, _, _ = C.geometry()
    qex = -(n @ np.array([1.0, 2.0, 3.0]))
    assert np.linalg.norm(x[0] - qex) / np.linalg.norm(qex) < (2e-3 if itri == 1 else 1e-7)


def test_laplace_quads_system(agb, orc):
    m = M.quad_box(3, 3, 2, hi=(2.4, 2.4, 1.3))
    u = m["xyz"] @ np.array([1.0, -0.5, 2.0])
    P = orc.Problem(1, m, walls=[1], known=[[1]], iqud=4)
    P.form_integrals()
    P.form_system()
    nl, _ = P.lists()
    C = _ctx(agb, m, agb.LAPLACE, [1], iqud=4)
    C.assemble(agb.FP64)
    A, _ = C.system(scaled=False)
    assert _rel(A, P.dense(0)) < 1e-12
    assert _rel(C.rhs(u[None])[0], P.dense(1) @ (-u[nl])) < 1e-12


def _stokes_ref(orc, m, U):
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    P.form_integrals()
    P.form_system()
    nl, _ = P.lists()
    S = P.dense(0)
    R = P.dense(1)
    B = np.stack([R @ np.concatenate([U[r, en, nl] for en in range(3)]) for r in range(U.shape[0])])
    return P, S, B


def test_stokes_fp64_system_and_rhs(agb, orc):
    m = _sis(1, 1)
    U = _rigid_fields(m)
    P, S, B = _stokes_ref(orc, m, U)
    C = _ctx(agb, m, agb.STOKES, [1, 2])
    C.assemble(agb.FP64)
    A, _ = C.system(scaled=False)
    assert A.shape == S.shape
    assert _rel(A, S) < 1e-12
    rhs = C.rhs(U)
    for r in range(6):
        assert _rel(rhs[r], B[r]) < 1e-12


def test_stokes_fp64_solve_force_torque(agb, orc):
    m = _sis(2, 1)
    U = _rigid_fields(m)
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    P.form_integrals()
    q_ref, ft_ref, nits, ierr = P.stokes_solve_sequence(U, maxit=0, eps=1e-13, fwall=1)
    C = _ctx(agb, m, agb.STOKES, [1, 2])
    C.assemble(agb.FP64)
    x, nit, istop = C.solve(U, eps=1e-13)
    assert np.all(istop <= 3)
    for r in range(6):
        assert _rel(x[r], q_ref[r].ravel()) < 1e-10
    ft = C.force_torque(x, 1)
    assert _rel(ft, ft_ref) < 1e-10
    R, nit2, times = C.resistance_tensor(agb.FP64, 1, 2, eps=1e-13)
    assert _rel(R, ft_ref) < 1e-10


def test_stokes_mixed_vs_fp64(agb):
    m = _sis(3, 1)
    C = _ctx(agb, m, agb.STOKES, [1, 2])
    C.assemble(agb.FP64)
    A64, _ = C.system(scaled=False)
    R64, _, _ = C.resistance_tensor(agb.FP64, 1, 2, eps=1e-12)
    C.assemble(agb.MIXED)
    A32, _ = C.system(scaled=False)
    # FP32 regular quadrature: entry-wise error relative to the row block scale
    assert np.max(np.abs(A32 - A64)) / np.max(np.abs(A64)) < 2e-6
    R32, nit, _ = C.resistance_tensor(agb.MIXED, 1, 2, eps=1e-7, refine=1)
    assert _rel(R32, R64) < 1e-5


def test_crs_dropin_matches_oracle(agb, orc):
    """agb_lsqr_precon / agb_lsqr_solve with the reference signature."""
    m = _sis(1, 1)
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    P.form_integrals()
    P.form_system()
    ia, ja, a = P.crs(0)
    mrow, ncol = P.neq_rows, P.nx
    a1 = a.copy()
    a2 = a.copy()
    q1 = agb.lsqr_precon(mrow, ncol, ia, ja, a1)
    q2 = orc.lsqr_precon(mrow, ncol, ia, ja, a2)
    assert np.max(np.abs(q1 - q2) / np.abs(q2)) < 1e-15
    assert np.max(np.abs(a1 - a2)) <= 2e-16 * np.max(np.abs(a2))
    # consistent right-hand side: the container translating along x
    U = _rigid_fields(m)
    nl, _ = P.lists()
    b = P.dense(1) @ np.concatenate([U[0, en, nl] for en in range(3)])
    rng = np.random.default_rng(3)
    x0 = rng.normal(size=ncol) * 1e-3
    x1 = x0.copy()
    x2 = x0.copy()
    nit1, ierr1 = agb.lsqr_solve(mrow, ncol, ia, ja, a1, q1, b, x1, maxit=0, eps=1e-13)
    nit2, ierr2, _ = orc.lsqr_solve(mrow, ncol, ia, ja, a2, q2, b, x2, maxit=0, eps=1e-13)
    assert ierr1 == ierr2
    # FP64 rounding differs between the GPU reductions and the serial loops,
    # so the iteration at which a stopping test first passes may move a little
    assert abs(nit1 - nit2) <= max(3, nit2 // 20)
    assert _rel(x1, x2) < 1e-9
    # an inconsistent right-hand side of this nearly rank-deficient operator
    # (the normal field is close to its null space) stops on the condition
    # limit (istop 4 -> ierr 4) in both implementations at the same iteration
    b = rng.normal(size=mrow)
    x1 = x0.copy()
    x2 = x0.copy()
    nit1, ierr1 = agb.lsqr_solve(mrow, ncol, ia, ja, a1, q1, b, x1, maxit=0, eps=1e-13)
    nit2, ierr2, _ = orc.lsqr_solve(mrow, ncol, ia, ja, a2, q2, b, x2, maxit=0, eps=1e-13)
    assert ierr1 == ierr2 == 4
    assert abs(nit1 - nit2) <= max(3, nit2 // 20)


def test_c2_full_size_against_frozen_fp64(agb):
    """The headline workload at full size (20 800 elements, 62 400 unknowns, the
    10.4 GB packed single layer) through the mixed path, against the FP64 GPU
    tensor frozen in tests/golden (FP64 assembly + FP64 LSQR to eps 1e-11).
    Tolerances: 1e-6 relative to the largest entry (the benchmark's accuracy
    bar), symmetry of the tensor within 1e-6 (the exact tensor is symmetric),
    drag and torque of the concentric spheres within 1e-3 of the analytic
    values (discretisation error of the level-5 sphere)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "c2_fp64_tensor.json")) as f:
        ref = json.load(f)
    R64 = np.asarray(ref["R"])
    m = M.particle_in_sphere(M.icosphere(5, 1.0, inward=True), outer_level=2, outer_radius=200.0)
    C = _ctx(agb, m, agb.STOKES, [1, 2])
    R, nit, info = C.resistance_tensor(agb.MIXED, 1, 2, eps=1e-7)
    C.close()
    assert np.all(np.isin(info["istop"], (1, 2)))
    assert _rel(R, R64) < 1e-6
    assert np.max(np.abs(R - R.T)) / np.max(np.abs(R)) < 1e-6
    lam = 1.0 / 200.0
    drag = 6 * np.pi * (1 - lam ** 5) / (1 - 9 * lam / 4 + 5 * lam ** 3 / 2 - 9 * lam ** 5 / 4 + lam ** 6)
    torque = 8 * np.pi / (1 - lam ** 3)
    assert abs(abs(R[0, 0]) / drag - 1) < 1e-3
    assert abs(abs(R[3, 3]) / torque - 1) < 1e-3
