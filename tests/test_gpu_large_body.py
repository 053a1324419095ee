"""The single-large-body workload's superellipsoid (a = 1, b = 0.5, c = 0.25,
e1 = 0.6, e2 = 1.4, mapSphereToSuperE parametrisation, lib_particle.f90:2207-2230)
on a grid where the plain FP64 path fits: the mixed path (packed FP32 single
layer, LSQR eps 3e-8 as the large-body benchmark runs it; at 1e-7 this flat body
is 2.4e-6 off) against the FP64 path (FP64 assembly and LSQR to eps 1e-10), 1e-6
relative to the largest tensor entry -- the benchmark's accuracy bar -- and the
same with BiCGSTAB-Jacobi and its FP64 true-residual restarts at tol 1e-7."""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def test_large_body_shape_coarse_grid_within_1e6_of_fp64(agb):
    body = M.superellipsoid(1.0, 0.5, 0.25, 0.6, 1.4, 40, 80, inward=True)
    m = M.particle_in_sphere(body, outer_level=2, outer_radius=200.0)
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, [1, 2], agb.dirichlet_known(agb.STOKES, 2), itri=5)
    R, nit, info = C.resistance_tensor(agb.MIXED, 1, 2, eps=3e-8)
    C.set_solver(agb.SOLVER_BICGSTAB)
    Rb, nitb, infob = C.resistance_tensor(agb.MIXED, 1, 2, eps=1e-7)
    C.set_solver(agb.SOLVER_LSQR)
    R64, nit64, info64 = C.resistance_tensor(agb.FP64, 1, 2, eps=1e-10)
    C.close()
    err = np.max(np.abs(R - R64)) / np.max(np.abs(R64))
    errb = np.max(np.abs(Rb - R64)) / np.max(np.abs(R64))
    print("mixed vs FP64", err, "BiCGSTAB", errb, "nit", list(nit), list(nitb), list(nit64))
    assert np.all(np.asarray(info["istop"]) <= 3) and np.all(np.asarray(info64["istop"]) <= 3)
    assert np.all(np.asarray(infob["istop"]) == 0)
    assert err < 1e-6 and errb < 1e-6
