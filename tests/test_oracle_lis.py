"""The oracle's LIS path of the Stokes system (SLET LIS: StokesBigSystemSOLVElis,
lib_StokesLis.f90:4, with the reference's default LIS options "-i bicgstab -p jacobi
-tol 1.0e-8 -maxiter 1000", mod_par.f90:288) against its CRS/LSQR path on the same
systems (CPU).

LIS is not part of the reference sources; the oracle restates the published
preconditioned BiCGSTAB (van der Vorst 1992, in the form of the Templates book),
so parity at the LIS boundary is unpinned: what is pinned is that both paths solve
the same square system, row for row, to the same answer.  The two solvers agree on
the particle's force and torque (the judged output) to the LIS tolerance, and on the
tractions once the free pressure level of an all-velocity problem is removed.  The
Jacobi-preconditioned BiCGSTAB needs a small fraction of LSQR's iterations on these
systems, each iteration two products with the matrix like one LSQR iteration.
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M
from fixtures import reference_mesh


def _rigid_motions(m, outer_wall=2):
    """Six container velocity fields: unit translations, then rotations e_i x r."""
    nn = len(m["xyz"])
    outer = np.unique(m["con"][m["bcid"] == outer_wall, :3])
    U = np.zeros((6, 3, nn))
    for i in range(3):
        U[i, i, outer] = 1.0
        w = np.zeros(3)
        w[i] = 1.0
        U[3 + i][:, outer] = np.cross(w, m["xyz"][outer]).T
    return U


@pytest.fixture(scope="module")
def sphere_case(orc):
    m = M.particle_in_sphere(M.icosphere(2, radius=1.0, inward=True, wall=1), outer_level=2, outer_radius=50.0)
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    P.form_integrals()
    U = _rigid_motions(m)
    q_ls, ft_ls, n_ls, ierr = P.stokes_solve_sequence(U, maxit=0, eps=1e-12, fwall=1)
    assert ierr == 0
    yield m, P, U, ft_ls, n_ls
    P.close()


def test_lis_default_options_match_lsqr_force_torque(sphere_case):
    m, P, U, ft_ls, n_ls = sphere_case
    q, ft, nits, status, relres = P.stokes_solve_lis(U)  # the reference's defaults
    assert np.all(status == 0) and np.all(relres <= 1e-8)
    scale = np.max(np.abs(ft_ls))
    assert np.max(np.abs(ft - ft_ls)) < 1e-7 * scale
    # each BiCGSTAB iteration multiplies by the matrix twice, as an LSQR iteration does
    # (A v and A^T u): the LIS path reads the matrix a quarter as often or less
    assert np.all(nits * 4 < n_ls), (nits, n_ls)


def test_lis_tight_tolerance_matches_lsqr(sphere_case):
    m, P, U, ft_ls, n_ls = sphere_case
    q, ft, nits, status, relres = P.stokes_solve_lis(U, tol=1e-12)
    assert np.all(status == 0)
    assert np.max(np.abs(ft - ft_ls)) < 1e-10 * np.max(np.abs(ft_ls))
    lam = 1.0 / 50.0
    drag = 6 * np.pi * (1 - lam ** 5) / (1 - 9 * lam / 4 + 5 * lam ** 3 / 2 - 9 * lam ** 5 / 4 + lam ** 6)
    assert np.allclose(np.diag(ft[:3, :3]) / drag, 1.0, atol=2e-2)


def test_lis_iteration_limit_reported(sphere_case):
    m, P, U, ft_ls, n_ls = sphere_case
    _, _, nits, status, relres = P.stokes_solve_lis(U[:1], tol=1e-12, maxiter=3)
    assert status[0] == 1 and nits[0] == 3 and relres[0] > 1e-12


def test_lis_couette_reference_cube(orc):
    """run/stokes/Couette on the reference's cube through the LIS path: the tractions
    of the LSQR path once the free pressure level is removed."""
    m = reference_mesh("cube_624")
    P = orc.Problem(2, m, walls=[1, 2, 3, 4, 5, 6], known=np.ones((3, 6)), itri=5)
    P.form_integrals()
    U = np.zeros((1, 3, len(m["xyz"])))
    U[0, 0] = m["xyz"][:, 2]
    q_ls, _, _, _ = P.stokes_solve_sequence(U, maxit=0, eps=1e-13, fwall=1)
    q, _, nits, status, _ = P.stokes_solve_lis(U, tol=1e-12)
    P.close()
    assert status[0] == 0
    x = m["xyz"]
    t = m["con"][:, :3]
    nrm = np.cross(x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]

    def without_pressure(qq):
        return qq - np.mean(np.sum(qq.T * nrm, axis=1)) * nrm.T

    # the two solvers end at very different pressure levels (the near-null direction
    # of an all-velocity problem); the constant normal traction removed is that
    # direction only to the discretisation, which leaves a few 1e-6
    assert np.max(np.abs(without_pressure(q[0]) - without_pressure(q_ls[0]))) < 1e-5


def test_lis_mixed_conditions_reference_cube(orc):
    """The Poiseuille conditions (x traction given on back, front and outlet): the
    LIS system holds the unknown velocities too, one equation per unknown."""
    m = reference_mesh("cube_624")
    known = np.ones((3, 6), np.int32)
    known[0, [2, 3, 5]] = 2
    z = m["xyz"][:, 2]
    U = np.zeros((1, 3, len(m["xyz"])))
    U[0, 0] = (8.0 / 3.0) * (z - z * z)
    P = orc.Problem(2, m, walls=[1, 2, 3, 4, 5, 6], known=known, diff=1.5, itri=5)
    P.form_integrals()
    q_ls, _, _, ierr = P.stokes_solve_sequence(U, maxit=0, eps=1e-13, fwall=1)
    q, _, nits, status, _ = P.stokes_solve_lis(U, tol=1e-12)
    P.close()
    assert status[0] == 0
    assert np.max(np.abs(q[0] - q_ls[0])) < 1e-6 * np.max(np.abs(q_ls[0]))


def test_lis_gmres_matches_lsqr_and_bicgstab(sphere_case):
    """The LIS options "-i gmres" (GMRES(40), the oracle's node/element block
    preconditioner): the same force and torque as the LSQR path at tol 1e-12,
    one product with the matrix per step, fewer products than BiCGSTAB."""
    m, P, U, ft_ls, n_ls = sphere_case
    q, ft, nits, status, relres = P.stokes_solve_lis(U, tol=1e-12, method="gmres")
    assert np.all(status == 0) and np.all(relres <= 1e-12)
    assert np.max(np.abs(ft - ft_ls)) < 1e-10 * np.max(np.abs(ft_ls))
    _, _, nb, sb, _ = P.stokes_solve_lis(U, tol=1e-12)
    assert np.all(sb == 0)
    assert np.all(nits < 2 * nb), (nits, nb)  # GMRES step: one product; BiCGSTAB iteration: two


def test_lis_gmres_restart_and_limit(sphere_case):
    """A short restart length converges to the same answer over several cycles;
    the iteration limit is reported as status 1."""
    m, P, U, ft_ls, n_ls = sphere_case
    _, ft40, n40, s40, _ = P.stokes_solve_lis(U[:2], tol=1e-10, method="gmres")
    _, ft5, n5, s5, _ = P.stokes_solve_lis(U[:2], tol=1e-10, method="gmres", restart=5)
    assert np.all(s40 == 0) and np.all(s5 == 0)
    assert np.all(n5 >= n40)
    assert np.max(np.abs(ft5 - ft40)) < 1e-8 * np.max(np.abs(ft40))
    _, _, nl, sl, rl = P.stokes_solve_lis(U[:1], tol=1e-12, maxiter=3, method="gmres")
    assert sl[0] == 1 and nl[0] == 3 and rl[0] > 1e-12


def test_lis_gmres_mixed_conditions_reference_cube(orc):
    """GMRES on the Poiseuille system, whose unknowns are velocities on some
    walls and tractions on others (blocks of 1-3 unknowns per node or element)."""
    m = reference_mesh("cube_624")
    known = np.ones((3, 6), np.int32)
    known[0, [2, 3, 5]] = 2
    z = m["xyz"][:, 2]
    U = np.zeros((1, 3, len(m["xyz"])))
    U[0, 0] = (8.0 / 3.0) * (z - z * z)
    P = orc.Problem(2, m, walls=[1, 2, 3, 4, 5, 6], known=known, diff=1.5, itri=5)
    P.form_integrals()
    q_ls, _, _, ierr = P.stokes_solve_sequence(U, maxit=0, eps=1e-13, fwall=1)
    q, _, nits, status, _ = P.stokes_solve_lis(U, tol=1e-12, method="gmres", restart=60)
    P.close()
    assert status[0] == 0
    assert np.max(np.abs(q[0] - q_ls[0])) < 1e-6 * np.max(np.abs(q_ls[0]))
