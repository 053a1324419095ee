"""GPU direct solver of the FULL path (agb_form_pre_fm / agb_solv_eqn_fm /
agb_solve_lu) against the LINPACK restatement of dgefa/dgesl in the oracle.

Pivots must be identical; U, L (converted from LINPACK to LAPACK storage) and
the solutions agree to 1e-12 relative (FP64 on both sides; the blocked GPU
elimination sums in a different order).
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _linpack_to_lapack_L(f, ipvt):
    """LINPACK stores -l and leaves later interchanges off earlier columns."""
    n = f.shape[0]
    L = -np.tril(f, -1)
    for k in range(n - 1):
        p = int(ipvt[k]) - 1
        if p != k:  # interchange of step k applies to the L columns before k
            L[[k, p], :k] = L[[p, k], :k]
    return L


@pytest.mark.parametrize("n", [7, 200, 700])
def test_lu_factor_and_solve(agb, orc, n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) + 0.1 * np.eye(n)
    b = rng.normal(size=n)
    f_ref, ipvt_ref, info_ref = orc.dgefa(A)
    f, q, ierr = agb.form_pre_fm(A)
    assert ierr == info_ref == 0
    assert np.array_equal(q, ipvt_ref)
    scale = np.max(np.abs(A))
    assert np.max(np.abs(np.triu(f) - np.triu(f_ref))) < 1e-12 * scale * n
    assert np.max(np.abs(np.tril(f, -1) - _linpack_to_lapack_L(f_ref, ipvt_ref))) < 1e-12 * n
    x, ierr = agb.solv_eqn_fm(f, q, b)
    x_ref = orc.dgesl(f_ref, ipvt_ref, b)
    assert np.max(np.abs(x - x_ref)) < 1e-10 * np.max(np.abs(x_ref))
    # prep 1: factor inside SolvEQNfm
    x2, _ = agb.solv_eqn_fm(A, np.zeros(n), b, prep=1)
    assert np.max(np.abs(x2 - x_ref)) < 1e-10 * np.max(np.abs(x_ref))
    # b = 0: x = 0
    x0, _ = agb.solv_eqn_fm(f, q, np.zeros(n))
    assert not np.any(x0)


def test_lu_zero_pivot_reported(agb, orc):
    rng = np.random.default_rng(5)
    A = rng.normal(size=(90, 90))
    A[:, 70] = 0.0
    _, _, info_ref = orc.dgefa(A)
    _, _, ierr = agb.form_pre_fm(A)
    assert ierr == info_ref == 71


def test_context_direct_solve_matches_lsqr(agb):
    """FULL path on an assembled FP64 system: LU solve = converged LSQR."""
    m = M.icosphere(2, 1.0)
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.LAPLACE, [1], [[agb.BC_FUNCTION]], itri=5)
    C.assemble(agb.FP64)
    u = (m["xyz"] @ np.array([1.0, 2.0, 3.0]))[None, :]
    x_lu, info = C.solve_lu(u)
    x_ls, _, istop = C.solve(u, eps=1e-14)
    assert info == 0
    assert np.max(np.abs(x_lu - x_ls)) < 1e-8 * np.max(np.abs(x_ls))
    C.close()
