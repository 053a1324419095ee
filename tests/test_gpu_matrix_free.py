"""GPU tests of the matrix-free operator (AGB_MATRIX_FREE): every LSQR sweep
recomputes the single-layer entries instead of reading a stored matrix.

Against the stored mixed-precision path on the same mesh: column scales q
within 1e-6 (FP32 entries, the sums of squares grouped differently), the
resistance tensor within 1e-6 at LSQR eps 1e-9 (same FP32 entries, products
summed in a different order).
"""
import ctypes

import numpy as np
import pytest

from andromeda_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _ctx(agb, level=2):
    m = M.particle_in_sphere(M.icosphere(level, 1.0, inward=True), outer_level=1, outer_radius=20.0)
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, [1, 2], np.ones((3, 2), np.int32), itri=5)
    return C


def test_matrix_free_matches_stored(agb):
    C = _ctx(agb)
    C.assemble(agb.MIXED)
    R_st, nit_st, _ = C.resistance_tensor(agb.MIXED, eps=1e-9)
    C.assemble(agb.MIXED)
    q_st = np.zeros(C.n)
    C._ck(C._L.agb_get_system(C.h, 0, None, q_st.ctypes.data_as(ctypes.c_void_p)))
    C.assemble(agb.MATRIX_FREE)
    q_mf = np.zeros(C.n)
    C._ck(C._L.agb_get_system(C.h, 0, None, q_mf.ctypes.data_as(ctypes.c_void_p)))
    assert np.max(np.abs(q_mf - q_st)) < 1e-6 * np.max(np.abs(q_st))
    R_mf, nit_mf, info = C.resistance_tensor(agb.MATRIX_FREE, eps=1e-9)
    assert np.all(np.isin(info["istop"], (1, 2, 4)))
    assert np.max(np.abs(R_mf - R_st)) / np.max(np.abs(R_st)) < 1e-6
    assert np.all(np.abs(np.asarray(nit_mf) - np.asarray(nit_st)) <= np.maximum(3, np.asarray(nit_st) // 20))
    C.close()


def test_matrix_free_needs_zero_warm_start(agb):
    C = _ctx(agb, level=1)
    C.assemble(agb.MATRIX_FREE)
    u = np.zeros((1, 3, C.nnodes))
    with pytest.raises(agb.AgbError):
        C.solve(u, x0=np.ones((1, C.n)), eps=1e-6)
    C.close()
