"""LSQR with the 3x3 self-block (block-Jacobi) right preconditioner
(AGB_SOLVER_LSQR_BLOCK) on the packed mixed Stokes system: the same least-
squares solution as lsqr_precon's column scaling with far fewer iterations.

* single body: the level-4 sphere in the benchmark's radius-200 container,
  tensor within 1e-6 of the FP64 path (FP64 assembly and the reference's LSQR
  to eps 1e-12) -- the benchmark's accuracy bar -- in under half of the
  column-scaled iterations;
* batched: four bodies of uneven size, every tensor within 1e-6 of the
  single-body solve with the same preconditioner and within 5e-6 of FP64 (the
  batched LSQR test's bar);
* a system it does not take (the FP64 path) is refused.
"""
import numpy as np
import pytest

from andromeda_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _ctx(agb, m):
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, [1, 2], agb.dirichlet_known(agb.STOKES, 2), itri=5)
    return C


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_block_preconditioned_lsqr_single_body(agb):
    m = M.particle_in_sphere(M.icosphere(4, 1.0, inward=True), outer_level=2, outer_radius=200.0)
    C = _ctx(agb, m)
    R64, n64, _ = C.resistance_tensor(agb.FP64, 1, 2, eps=1e-12)
    Rc, nc, _ = C.resistance_tensor(agb.MIXED, 1, 2, eps=1e-7)
    C.set_solver(agb.SOLVER_LSQR_BLOCK)
    Rb, nb, info = C.resistance_tensor(agb.MIXED, 1, 2, eps=1e-7)
    with pytest.raises(agb.AgbError):
        C.resistance_tensor(agb.FP64, 1, 2, eps=1e-8)  # the FP64 system is not packed
    C.close()
    print("iterations column scaling", list(nc), "block", list(nb), "errors", _rel(Rc, R64), _rel(Rb, R64))
    assert np.all(np.asarray(info["istop"]) <= 3)
    assert _rel(Rb, R64) < 1e-6
    assert np.max(nb) * 2 < np.max(nc)


def test_block_preconditioned_lsqr_batched(agb):
    rng = np.random.default_rng(7)
    meshes = []
    for n in (300, 520, 760, 1100):
        b, c = rng.uniform(0.4, 1.0, 2)
        e1, e2 = rng.uniform(0.6, 1.4, 2)
        body = M.superellipsoid_tri(1.0, b, c, e1, e2, n, rotation=M.random_rotation(rng), inward=True)
        meshes.append(M.particle_in_sphere(body, outer_level=2, outer_radius=200.0))
    R, nit, istop, st = agb.batch_resistance(meshes, eps=3e-8, solver=agb.SOLVER_LSQR_BLOCK)
    assert np.all(istop <= 3) and st["av_launches"] > 0
    for i, m in enumerate(meshes):
        C = _ctx(agb, m)
        R64, _, _ = C.resistance_tensor(agb.FP64, 1, 2, eps=1e-11)
        C.set_solver(agb.SOLVER_LSQR_BLOCK)
        Rs, ns, _ = C.resistance_tensor(agb.MIXED, 1, 2, eps=3e-8)
        C.close()
        assert _rel(R[i], Rs) < 1e-6, i
        assert _rel(R[i], R64) < 5e-6, i
