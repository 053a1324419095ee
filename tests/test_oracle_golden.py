"""CPU tests: pin the FP64 oracle against the reference's own known answers.

The reference ships no golden output files; what it does ship are
* the analytic integrals of Triangle_TestIntegration (src/mod_trikotnik.f90:124-154),
* the rigid-body / free-term self-checks it logs as fSP/qSP errors
  (src/lib_sdBem.f90:566-581,714-718; src/lib_Stokes.f90:1781-1812,2153-2178),
* analytic resistances (src/lib_particle.f90:1910-1976).
The analytic singular integrals are pinned independently by Duffy-transformed
Gauss quadrature, and tests/golden/oracle_values.json freezes oracle outputs
(generated by tests/golden/make_golden.py) against regressions.
"""
import json
import os

import numpy as np
import pytest

from andromeda_gb300 import mesh as M

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# Triangle_TestIntegration analytic values (mod_trikotnik.f90:145-154)
ANAL = [2097152.0 / 121.0, 1.0522458619541769455, 0.98364468921563619296, 0.14027496308479503178]


def test_wx_rules_sizes_and_weights(orc):
    for itri, q in zip(range(1, 6), (7, 25, 54, 85, 126)):
        l1, l2, l3, w = orc.wx_rule(itri)
        assert len(w) == q
        assert abs(w.sum() - 1.0) < 1e-14
        assert np.all(np.abs(l1 + l2 + l3 - 1) < 1e-14)


@pytest.mark.parametrize("itri,tol", [(1, [0.46, 1e-2, 2e-3, 0.06]), (2, [1e-3, 2e-6, 1e-8, 0.006]),
                                      (3, [5e-8, 1e-10, 5e-12, 0.009]), (4, [1e-13, 1e-13, 1e-14, 0.006]),
                                      (5, [1e-13, 1e-14, 1e-14, 0.004])])
def test_triangle_test_integration(orc, itri, tol):
    """Polynomial of degree 20 is exact for the order-20/25 rules (ITRI 4, 5)."""
    r = orc.triangle_test(itri)
    for k in range(4):
        assert abs(r[k] - ANAL[k]) / ANAL[k] <= tol[k], (itri, k, r[k])


def _duffy(P0, P1, P2, f, n=120):
    x, w = np.polynomial.legendre.leggauss(n)
    u, wu = 0.5 * (x + 1), 0.5 * w
    U, V = np.meshgrid(u, u, indexing="ij")
    W = np.outer(wu, wu)
    X = P0 + U[..., None] * (P1 - P0) + (U * V)[..., None] * (P2 - P1)
    J = U * np.linalg.norm(np.cross(P1 - P0, P2 - P1))
    return np.tensordot(W * J, f(X), axes=([0, 1], [0, 1]))


def _lap(s):
    return lambda X: 1 / (4 * np.pi * np.linalg.norm(X - s, axis=-1))


def _stk(s):
    def f(X):
        r = X - s
        R = np.linalg.norm(r, axis=-1)
        G = np.eye(3)[None, None] / R[..., None, None] + r[..., :, None] * r[..., None, :] / R[..., None, None] ** 3
        return G[..., [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]]
    return f


def _numeric_self(v, isrc, f):
    if isrc < 4:
        s = v[isrc - 1]
        return _duffy(s, v[isrc % 3], v[(isrc + 1) % 3], f(s))
    s = v.mean(0)
    return sum(_duffy(s, v[k], v[(k + 1) % 3], f(s)) for k in range(3))


@pytest.mark.parametrize("isrc", [1, 2, 3, 4])
@pytest.mark.parametrize("tri", [
    [[0.1, 0.2, 0.3], [1.3, 0.1, 0.5], [0.4, 1.1, 0.2]],
    [[0.0, 0.0, 1.0], [2.0, 0.0, 1.0], [2.0, 2.0, 1.0]],
    [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.02, 0.05, 0.3]],   # skinny
])
def test_ren_chan_vs_duffy(orc, isrc, tri):
    v = np.array(tri, dtype=float)
    a = orc.si_tri_lap(v, isrc)
    b = orc.si_tri_stk(v, isrc)
    na = _numeric_self(v, isrc, _lap)
    nb = _numeric_self(v, isrc, _stk)
    assert abs(a - na) / abs(na) < 1e-12
    assert np.max(np.abs(b - nb)) / np.max(np.abs(nb)) < 1e-11


def test_quad_singular_is_triangle_fan(orc):
    q = np.array([[0, 0, 0], [1.2, 0.1, 0], [1.1, 0.9, 0.2], [-0.1, 1.0, 0.1]], dtype=float)
    # corner 1: triangles (1,2,3)+(1,3,4)
    exp = orc.si_tri_lap(q[[0, 1, 2]], 1) + orc.si_tri_lap(q[[0, 2, 3]], 1)
    assert abs(orc.si_qua_lap(q, 1) - exp) < 1e-15
    c = q.mean(0)
    exp5 = sum(orc.si_tri_lap(np.array([c, q[k], q[(k + 1) % 4]]), 1) for k in range(4))
    assert abs(orc.si_qua_lap(q, 5) - exp5) < 1e-14
    g = orc.si_qua_stk(q, 2)
    eg = orc.si_tri_stk(q[[1, 2, 3]], 1) + orc.si_tri_stk(q[[1, 3, 0]], 1)
    assert np.max(np.abs(g - eg)) < 1e-14


@pytest.mark.parametrize("isrc", [1, 2, 3, 4, 5])
def test_quad_polar_singular_scheme_against_closed_forms(orc, isrc):
    """The singular branch of Quad_BEMInt / Quad_StokesInt (lib_int.f90:408-524,
    lib_Stokes.f90:3494-3654: polar Gauss about the source in four triangles of
    the parameter square) against the Ren-Chan closed forms of the split quad
    (si_qua_lap / si_qua_stk): two independent methods, equal to 2e-14 at the
    6- and 8-point rules on a flat quad (H vanishes there); at the reference's
    default rule (IQUD 4) within 2e-7."""
    q = np.array([[0, 0, 0], [1.3, 0.1, 0], [1.1, 0.9, 0], [-0.1, 1.0, 0]], dtype=float)
    s = q[isrc - 1] if isrc < 5 else q.mean(0)
    a, b = orc.si_qua_lap(q, isrc), orc.si_qua_stk(q, isrc)
    for iqud, tol in ((4, 2e-7), (6, 2e-14), (8, 2e-14)):
        g, h = orc.quad_lap_polar(iqud, q, s, isrc)
        G = orc.quad_stk_polar(iqud, q, s, isrc)
        assert abs(g - a) <= tol * abs(a)
        assert np.max(np.abs(G - b)) <= tol * np.max(np.abs(b))
        assert np.max(np.abs(h)) == 0.0
    # a warped quad: the rule converges (6 vs 8 points) to 1e-12
    w = q.copy()
    w[2, 2] = 0.3
    s = w[isrc - 1] if isrc < 5 else w.mean(0)
    g6, h6 = orc.quad_lap_polar(6, w, s, isrc)
    g8, h8 = orc.quad_lap_polar(8, w, s, isrc)
    assert abs(g6 - g8) <= 1e-12 * abs(g8) and np.max(np.abs(h6 - h8)) <= 1e-12 * max(1e-3, np.max(np.abs(h8)))


def test_mesh_generators_counts():
    m3 = M.icosphere(3)
    assert len(m3["xyz"]) == 642 and len(m3["etype"]) == 1280
    m5 = M.icosphere(5)
    assert len(m5["xyz"]) == 10242 and len(m5["etype"]) == 20480
    se = M.superellipsoid(1.0, 0.5, 0.25, 0.6, 1.4, 160, 320)
    assert len(se["etype"]) == 102400
    # every triangle non-degenerate and outward oriented
    p = se["xyz"][se["con"][:, :3]]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    assert np.all(np.linalg.norm(n, axis=1) > 0)
    assert np.all(np.einsum("ij,ij->i", n, p.mean(1)) > 0)


def test_laplace_c1_diagnostics_and_flux(orc):
    """Config 1: unit icosphere L3, u = x+2y+3z; q = -n.(1,2,3) (q = -diff du/dn)."""
    m = M.icosphere(3)
    P = orc.Problem(1, m, walls=[1], known=[[1]], itri=5)
    errs = P.form_integrals()
    assert errs[0] < 1e-12      # u-row rigid-body residual (lib_sdBem.f90:566-581)
    assert errs[1] < 1e-7       # q-row |0.5 - c| (lib_sdBem.f90:714-718)
    n, a, c = P.geometry()
    u = m["xyz"] @ np.array([1.0, 2.0, 3.0])
    _, q, nit, ierr = P.laplace_solve(u, np.zeros(P.nelem), maxit=0, eps=1e-12)
    qex = -(n @ np.array([1.0, 2.0, 3.0]))
    assert ierr == 0
    assert np.linalg.norm(q - qex) / np.linalg.norm(qex) < 1e-7


def _sphere_in_sphere(level_in=1, level_out=1, a=1.0, b=8.0):
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


def test_stokes_concentric_spheres(orc):
    """Drag / torque of a fixed sphere inside a moving container against the
    concentric-sphere solutions (flat elements: O(h^2) discretisation error)."""
    a, b = 1.0, 8.0
    m = _sphere_in_sphere(2, 1, a, b)
    P = orc.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    errs = P.form_integrals()
    assert errs[1] < 1e-2   # q-row diagonal 4 pi / off-diagonal 0 (lib_Stokes.f90:1781-1812)
    q, ft, nits, ierr = P.stokes_solve_sequence(_rigid_fields(m), maxit=0, eps=1e-10, fwall=1)
    assert ierr == 0
    lam = a / b
    K = (1 - lam ** 5) / (1 - 9 / 4 * lam + 5 / 2 * lam ** 3 - 9 / 4 * lam ** 5 + lam ** 6)
    F = ft[:3, :3] / (6 * np.pi * a * K)
    T = ft[3:, 3:] / (8 * np.pi * a ** 3 / (1 - lam ** 3))
    assert np.allclose(np.diag(F), np.diag(F)[0], rtol=1e-6)
    assert 0.95 < F[0, 0] < 1.01
    assert 0.90 < T[0, 0] < 1.01
    R = ft.T  # rows: F,T components; columns: motions
    assert np.max(np.abs(R - R.T)) / np.max(np.abs(R)) < 1e-3  # reciprocal theorem


def test_lsqr_oracle_small_system(orc):
    rng = np.random.default_rng(7)
    A = rng.normal(size=(40, 25))
    ia = np.arange(0, 40 * 25 + 1, 25, dtype=np.int64) + 1
    ja = np.tile(np.arange(1, 26, dtype=np.int32), 40)
    a = A.ravel().copy()
    q = orc.lsqr_precon(40, 25, ia, ja, a)
    assert np.allclose(q, 1 / np.linalg.norm(A, axis=0))
    xt = rng.normal(size=25)
    b = A @ xt
    x = np.zeros(25)
    nit, ierr, st = orc.lsqr_solve(40, 25, ia, ja, a, q, b, x, maxit=0, eps=1e-14)
    assert ierr == 0
    assert np.linalg.norm(x - xt) / np.linalg.norm(xt) < 1e-10


def test_golden_values_frozen(orc):
    """Oracle outputs frozen in tests/golden/oracle_values.json."""
    with open(os.path.join(GOLDEN, "oracle_values.json")) as f:
        g = json.load(f)
    v = np.array(g["triangle"])
    for isrc in (1, 2, 3, 4):
        assert abs(orc.si_tri_lap(v, isrc) - g["si_tri_lap"][isrc - 1]) <= 1e-14 * abs(g["si_tri_lap"][isrc - 1])
        assert np.allclose(orc.si_tri_stk(v, isrc), g["si_tri_stk"][isrc - 1], rtol=1e-13, atol=0)
    for itri in range(1, 6):
        assert np.allclose(orc.triangle_test(itri), g["triangle_test"][itri - 1], rtol=1e-13, atol=0)


# ---- integration options: recursive self-element scheme, adaptive near-singular rule ----
_TRI = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.3, 0.9, 0.0]])


@pytest.mark.parametrize("isrc", [1, 2, 3, 4])
def test_recursive_singular_converges_to_analytic(orc, isrc):
    """Triangle_BEMInt's midpoint recursion toward the source (lib_sdBem.f90:775)
    converges to the Ren-Chan closed form: the error, set by the last piece
    taken with the regular rule, halves with every level."""
    v = _TRI
    s = v[isrc - 1] if isrc < 4 else v.mean(axis=0)
    n = np.array([0.0, 0.0, 1.0])
    ana = orc.si_tri_lap(v, isrc)
    errs = [abs(orc.tri_lap_opt(5, v, s, n, isrc, 1, d)[0] - ana) / ana for d in (6, 10, 14)]
    assert errs[2] < 5e-6
    assert errs[0] > 10 * errs[1] > 100 * errs[2]
    # Stokes: the six Stokeslet components against si_tri_stk
    g_ana = orc.si_tri_stk(v, isrc)
    g_rec = orc.tri_stk_opt(5, v, s, n, isrc, 1, 16)[:6]
    assert np.max(np.abs(g_rec - g_ana)) / np.max(np.abs(g_ana)) < 5e-6
    # rules with a centroid point (ITRI 1, 2, 4): the last piece of a centroid
    # recursion leaves that point out instead of dividing by r = 0
    for itri in (1, 2, 4):
        g = orc.tri_lap_opt(itri, v, s, n, isrc, 1, 14)[0]
        assert np.isfinite(g) and abs(g - ana) / ana < 5e-3


def _dblquad_tri(f, v):
    """High-order reference: adaptive Gauss-Kronrod over the triangle (scipy)."""
    from scipy import integrate
    e1, e2 = v[1] - v[0], v[2] - v[0]
    jac = np.linalg.norm(np.cross(e1, e2))
    val, _ = integrate.dblquad(lambda b, a: f(v[0] + a * e1 + b * e2, a, b), 0.0, 1.0, 0.0, lambda a: 1.0 - a,
                               epsabs=1e-14, epsrel=1e-13)
    return val * jac


@pytest.mark.parametrize("height", [0.05, 0.01])
def test_near_singular_rule_against_high_order_reference(orc, height):
    """The adaptive near-singular rule (no reference counterpart) against an
    independent adaptive Gauss-Kronrod integration of G and the nodal H."""
    pytest.importorskip("scipy")
    v = _TRI
    n = np.array([0.0, 0.0, 1.0])
    s = np.array([0.5, 0.03, height])

    def G(x, a, b):
        return 0.25 / np.pi / np.linalg.norm(s - x)

    def H(k):
        def f(x, a, b):
            r = s - x
            ra = np.linalg.norm(r)
            lam = (1.0 - a - b, a, b)[k]
            return (r @ n) / ra ** 2 * 0.25 / np.pi / ra * lam
        return f

    ref = np.array([_dblquad_tri(G, v)] + [_dblquad_tri(H(k), v) for k in range(3)])
    plain = orc.tri_lap_opt(5, v, s, n)
    near = orc.tri_lap_opt(5, v, s, n, 0, 0, 0, 1.5, 12)
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(plain - ref)) / scale > 1e-4      # the regular rule is off
    assert np.max(np.abs(near - ref)) / scale < 1e-9       # the adaptive rule is not
    # far from the element the rule changes nothing
    far = np.array([0.4, 0.3, 3.0])
    assert np.array_equal(orc.tri_lap_opt(5, v, far, n), orc.tri_lap_opt(5, v, far, n, 0, 0, 0, 1.5, 12))


def test_linpack_direct_solver(orc):
    """dgefa/dgesl restatement (lib_solveFM.f:198,318): pivots and U agree with
    an independent LU with partial pivoting (scipy/LAPACK getrf), the solves
    of A x = b and A^T x = b are exact to round-off, and a zero column is
    reported through info."""
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(3)
    n = 60
    A = rng.normal(size=(n, n))
    b = rng.normal(size=n)
    f, ipvt, info = orc.dgefa(A)
    lu, piv = sl.lu_factor(A)
    assert info == 0
    assert np.array_equal(ipvt.astype(int), piv + 1)
    assert np.max(np.abs(np.triu(f) - np.triu(lu))) < 1e-12 * np.max(np.abs(lu))
    assert np.max(np.abs(A @ orc.dgesl(f, ipvt, b) - b)) < 1e-12 * n
    assert np.max(np.abs(A.T @ orc.dgesl(f, ipvt, b, job=1) - b)) < 1e-12 * n
    A[:, 7] = 0.0
    _, _, info = orc.dgefa(A)
    assert info == 8


def test_mlp_oracle_gradient_by_finite_differences():
    """The FP64 MLP oracle's backward pass against central differences."""
    import mlp_oracle as mo
    rng = np.random.default_rng(0)
    nin, nh, nout = 5, 7, 4
    npar = nh * nin + nh + 2 * (nh * nh + nh) + nout * nh + nout
    p = rng.normal(scale=0.4, size=npar)
    X = rng.normal(size=(9, nin))
    T = rng.normal(size=(9, nout))
    args = (X, T, np.zeros(nin), np.ones(nin), np.zeros(nout), np.ones(nout), nin, nh, nout)
    _, g = mo.loss_and_grad(p, *args)
    h = 1e-6
    fd = np.zeros(npar)
    for i in range(npar):
        e = np.zeros(npar)
        e[i] = h
        fd[i] = (mo.loss_and_grad(p + e, *args)[0] - mo.loss_and_grad(p - e, *args)[0]) / (2 * h)
    assert np.max(np.abs(fd - g)) < 1e-8 * max(1.0, np.max(np.abs(g)))
