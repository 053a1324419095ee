"""GPU test of agb_lsqr_precon_dense_noalloc, the entry point that allocates
nothing (for callers that cannot call cudaMalloc: host programs that own all
device memory through their own pool or an OpenACC runtime, code running in an
allocation-free phase, embeddings whose device memory is fully reserved).

It must give the same column scaling as the existing entry point
agb_lsqr_precon (the lsqr_precon drop-in) on the same matrix, on two calls in a
row (the second call reuses the shared scratch array with the first call's
contents left in it).  Tolerance: 1e-14 relative -- both compute in FP64, only
the order of the column sums differs.  The device buffers here are the test's
own (torch); the entry point itself allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-14


def _dense_as_crs(A):
    m, n = A.shape
    ia = np.arange(m + 1, dtype=np.int64) * n + 1
    ja = np.tile(np.arange(1, n + 1, dtype=np.int32), m)
    return ia, ja, A.ravel().copy()


def test_noalloc_precon_matches_lsqr_precon(agb):
    torch = pytest.importorskip("torch")
    L = agb.load()
    rng = np.random.default_rng(11)
    for m, n, lda in [(300, 200, 224), (257, 129, 160)]:  # two calls in a row
        A = rng.normal(size=(m, n))
        ia, ja, a = _dense_as_crs(A)
        q_ref = agb.lsqr_precon(m, n, ia, ja, a)  # existing entry point (scales a in place)
        dA = torch.zeros((m, lda), dtype=torch.float64, device="cuda")
        dA[:, :n] = torch.from_numpy(A).cuda()
        dq = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.agb_lsqr_precon_dense_noalloc(m, n, lda, C.c_void_p(dA.data_ptr()), C.c_void_p(dq.data_ptr()))
        assert rc == 0, L.agb_last_error(None)
        q = dq.cpu().numpy()
        scaled = dA[:, :n].cpu().numpy()
        assert np.max(np.abs(q - q_ref) / q_ref) < TOL
        assert np.max(np.abs(scaled - a.reshape(m, n))) <= TOL * np.max(np.abs(a))
        assert int(torch.count_nonzero(dA[:, n:])) == 0  # padding columns untouched


def test_noalloc_precon_rejects_oversized(agb):
    L = agb.load()
    rc = L.agb_lsqr_precon_dense_noalloc(4, (1 << 20) + 1, (1 << 20) + 32, C.c_void_p(1), C.c_void_p(1))
    assert rc == 1
    assert b"AGB_NOALLOC_MAX_COLUMNS" in L.agb_last_error(None)


def test_noalloc_precon_wide_matrices(agb):
    """Widths where the scratch, not the cap of 64, sets the number of row
    groups (n > 16384), up to the largest accepted width
    AGB_NOALLOC_MAX_COLUMNS: q against 1/||A(:,j)|| computed in NumPy and the
    scaled matrix against A diag(q)."""
    torch = pytest.importorskip("torch")
    L = agb.load()
    rng = np.random.default_rng(5)
    for m, n in [(3, 40000), (70, 20000), (2, 1 << 20)]:
        lda = (n + 31) // 32 * 32
        A = rng.normal(size=(m, n))
        dA = torch.zeros((m, lda), dtype=torch.float64, device="cuda")
        dA[:, :n] = torch.from_numpy(A).cuda()
        dq = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.agb_lsqr_precon_dense_noalloc(m, n, lda, C.c_void_p(dA.data_ptr()), C.c_void_p(dq.data_ptr()))
        assert rc == 0, L.agb_last_error(None)
        q = dq.cpu().numpy()
        q_np = 1.0 / np.sqrt(np.sum(A * A, axis=0))
        assert np.max(np.abs(q - q_np) / q_np) < TOL
        scaled = dA[:, :n].cpu().numpy()
        assert np.max(np.abs(scaled - A * q_np[None, :])) <= TOL * np.max(np.abs(A * q_np[None, :]))
