"""The failure path of the bounded barrier waits, made to run out without a
fault (agb_selftest_bounded_wait): a wait on an mbarrier that nothing arrives
at, with no copy in flight and a short poll limit, gives up, raises the error
word and returns; the host reports it as AGB_ERR_CUDA ("a bounded barrier wait
gave up"), as the solvers do, and the GPU context stays usable afterwards."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_survives(agb):
    L = agb.load()
    done = C.c_int(-1)
    # control: one thread arrives, every wait completes
    assert L.agb_selftest_bounded_wait(0, 4096, 1, C.byref(done)) == agb.OK, L.agb_last_error(None)
    assert done.value == 32
    # nothing arrives: the wait gives up after its limit and the call reports it
    rc = L.agb_selftest_bounded_wait(0, 4096, 0, C.byref(done))
    assert rc == agb.ERR_CUDA
    assert b"bounded barrier wait gave up" in L.agb_last_error(None)
    assert done.value == 0
    # the context is still usable: the control again, then a small solve
    assert L.agb_selftest_bounded_wait(0, 4096, 1, C.byref(done)) == agb.OK and done.value == 32
    from andromeda_gb300 import mesh as M
    m = M.particle_in_sphere(M.icosphere(1, 1.0, inward=True), outer_level=1, outer_radius=8.0)
    ctx = agb.Context(0)
    ctx.set_mesh(m)
    ctx.set_problem(agb.STOKES, [1, 2], agb.dirichlet_known(agb.STOKES, 2), itri=5)
    R, nit, info = ctx.resistance_tensor(agb.MIXED, 1, 2, eps=1e-8)
    ctx.close()
    assert np.all(np.isfinite(R)) and np.all(np.asarray(info["istop"]) <= 3)


def test_bounded_wait_rejects_bad_limits(agb):
    L = agb.load()
    done = C.c_int(0)
    assert L.agb_selftest_bounded_wait(0, 0, 0, C.byref(done)) == agb.ERR_ARG
    assert L.agb_selftest_bounded_wait(0, (1 << 22) + 1, 0, C.byref(done)) == agb.ERR_ARG
