"""GPU parity of the integration options (agb_set_integration) against the
oracle run with the same options: the recursive self-element subdivision of
Triangle_BEMInt / Triangle_StokesInt (lib_sdBem.f90:775, lib_Stokes.f90:2251),
the polar singular scheme of Quad_BEMInt / Quad_StokesInt (lib_int.f90:408,
lib_Stokes.f90:3494) for a quad's own node or centre, and the adaptive
near-singular rule, through the general FP64 assembly.

Tolerance: 1e-12 relative to the largest entry of each integral matrix (FP64 on
both sides; only FMA contraction and the row-sum order differ).
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M

pytestmark = pytest.mark.gpu

OPTIONS = [(1, 6, 0.0, 0), (0, 20, 1.5, 6), (1, 4, 2.0, 8)]


def _check(T, G, P, ncomp):
    for k in range(ncomp):
        ref = P.integral_matrix(k)
        assert np.max(np.abs(T[k] - ref)) <= 1e-12 * max(np.max(np.abs(ref)), 1e-300), k
        refg = P.integral_matrix(ncomp + k) if ncomp == 9 else P.integral_matrix(1)
        assert np.max(np.abs(G[k] - refg)) <= 1e-12 * max(np.max(np.abs(refg)), 1e-300), k


@pytest.mark.parametrize("opt", OPTIONS)
def test_laplace_options_parity(agb, orc, opt):
    m = M.quad_box(2, 2, 2, hi=(1.0, 0.7, 0.5), face_walls=True, triangles=True)
    walls = [1, 2, 3, 4, 5, 6]
    known = [[1, 1, 2, 2, 2, 2]]
    P = orc.Problem(1, m, walls=walls, known=known, itri=4, iqud=4)
    P.set_integration(*opt)
    P.form_integrals()
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.LAPLACE, walls, known, itri=4, iqud=4)
    C.set_integration(*opt)
    T, G, _ = C.integral_matrices()
    _check(T, G, P, 1)


@pytest.mark.parametrize("opt", OPTIONS)
def test_stokes_options_parity(agb, orc, opt):
    m = M.particle_in_sphere(M.icosphere(1, 1.0, inward=True), outer_level=0, outer_radius=3.0)
    walls = [1, 2]
    known = np.ones((3, 2), np.int32)
    P = orc.Problem(2, m, walls=walls, known=known, itri=3, iqud=4)
    P.set_integration(*opt)
    P.form_integrals()
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, walls, known, itri=3, iqud=4)
    C.set_integration(*opt)
    T, G, _ = C.integral_matrices()
    _check(T, G, P, 9)


@pytest.mark.parametrize("kind", ["laplace", "stokes"])
def test_quad_polar_singular_parity(agb, orc, kind):
    """sing_mode 1 on a quad mesh: the own-node / centre integrals by the polar
    scheme of the singular branch of Quad_BEMInt / Quad_StokesInt, GPU against
    the oracle; a box with a warped face, so the polar H / T of the self element
    do not vanish."""
    m = M.quad_box(2, 2, 2, hi=(1.0, 0.7, 0.5), face_walls=True)
    m = dict(m)
    xyz = m["xyz"].copy()
    top = np.isclose(xyz[:, 2], 0.5) & np.isclose(xyz[:, 0], 0.5) & np.isclose(xyz[:, 1], 0.35)
    xyz[top, 2] += 0.08  # the middle node of the top face: its four quads become non-planar
    m["xyz"] = xyz
    walls = [1, 2, 3, 4, 5, 6]
    if kind == "laplace":
        known = [[1, 1, 2, 2, 2, 2]]
        P = orc.Problem(1, m, walls=walls, known=known, itri=4, iqud=4)
        k, ncomp = agb.LAPLACE, 1
    else:
        known = np.ones((3, 6), np.int32)
        P = orc.Problem(2, m, walls=walls, known=known, itri=4, iqud=4)
        k, ncomp = agb.STOKES, 9
    P.set_integration(1, 6, 0.0, 0)
    P.form_integrals()
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(k, walls, known, itri=4, iqud=4)
    C.set_integration(1, 6, 0.0, 0)
    T, G, _ = C.integral_matrices()
    C.close()
    _check(T, G, P, ncomp)
    assert np.count_nonzero(top) == 1


def test_options_route_resistance_tensor_through_general_path(agb):
    """With the near-singular rule on, the resistance workflow runs on the
    general path; the tensor stays within the discretisation error of the
    default assembly and the system differs only in the near pairs."""
    m = M.particle_in_sphere(M.icosphere(2, 1.0, inward=True), outer_level=1, outer_radius=20.0)
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, [1, 2], np.ones((3, 2), np.int32), itri=5)
    R0, _, _ = C.resistance_tensor(agb.FP64, eps=1e-12)
    C.set_integration(0, 20, 1.5, 8)
    R1, _, info = C.resistance_tensor(agb.FP64, eps=1e-12)
    assert np.all(np.asarray(info["istop"]) <= 3)
    rel = np.max(np.abs(R1 - R0)) / np.max(np.abs(R0))
    assert 0.0 < rel < 1e-2
