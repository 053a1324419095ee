"""Host-side front end of the GB300 BEM hot path.

Mirrors the reference's operator interface for this path:

* :func:`lsqr_precon` / :func:`lsqr_solve` -- the exact argument meaning of
  ``lsqr_precon(m,n,nnz,q,ia,ja,a)`` and
  ``lsqr_solve(m,n,nnz,maxit,eps,nit,ierr,q,ia,ja,a,b,x)`` (src/lib_lsqr.f:131,33):
  1-based CRS, ``a`` scaled in place, ``x`` warm start in / solution out.
* :class:`Context` -- mesh + one subdomain + BCs (the mMesh/mEqns module state),
  assembly of the system on the GPU (CoR_Integrals + sdSetUpSysMrhsM_CRS /
  stokesFormCRSsysMrhsM + lsqr_precon), right-hand sides, block LSQR solve,
  force/torque (getForceIntegrateFluxes / getTorqueIntegrateFluxes) and the
  resistance-tensor workflow (StokesInlet3sides*CRS).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import AgbError, load

LAPLACE, STOKES = 1, 2
FP64, MIXED, MATRIX_FREE = 0, 1, 2
SOLVER_LSQR, SOLVER_BICGSTAB, SOLVER_HYBRID, SOLVER_LSQR_BLOCK, SOLVER_GMRES = 0, 1, 2, 3, 4
BC_FUNCTION, BC_FLUX, BC_CONTACT = 1, 2, 3
# return codes of the C ABI (include/andromeda_gb300.h)
OK, ERR_ARG, ERR_CUDA, ERR_STATE, ERR_UNSUPPORTED, ERR_NUMERIC = 0, 1, 2, 3, 4, 5


def _check(rc, ctx_ptr=None):
    if rc != 0:
        L = load()
        msg = L.agb_last_error(ctx_ptr).decode()
        raise AgbError(f"andromeda_gb300 error {rc}: {msg}")


def version() -> str:
    return load().agb_version().decode()


def lsqr_precon(m, n, ia, ja, a, q=None):
    """Column scaling q_j = 1/||A(:,j)|| and A <- A diag(q), on the GPU.

    ``a`` (float64) is modified in place like the reference does; returns q.
    """
    L = load()
    ia = np.ascontiguousarray(ia, dtype=np.int64)
    ja = np.ascontiguousarray(ja, dtype=np.int32)
    assert a.dtype == np.float64 and a.flags.c_contiguous
    if q is None:
        q = np.zeros(n)
    _check(L.agb_lsqr_precon(int(m), int(n), len(a), q, ia, ja, a))
    return q


def lsqr_solve(m, n, ia, ja, a, q, b, x, maxit=0, eps=1e-8):
    """LSQR with the reference's warm start and stopping rules, on the GPU.

    ``x`` (float64) holds the initial guess and receives the solution.
    Returns (nit, ierr) like the Fortran out-arguments.
    """
    L = load()
    ia = np.ascontiguousarray(ia, dtype=np.int64)
    ja = np.ascontiguousarray(ja, dtype=np.int32)
    mi, nit, ierr = C.c_int(int(maxit)), C.c_int(0), C.c_int(0)
    assert x.dtype == np.float64 and x.flags.c_contiguous
    _check(L.agb_lsqr_solve(int(m), int(n), len(a), C.byref(mi), float(eps), C.byref(nit), C.byref(ierr),
                            np.ascontiguousarray(q, dtype=np.float64), ia, ja,
                            np.ascontiguousarray(a, dtype=np.float64), np.ascontiguousarray(b, dtype=np.float64), x))
    return nit.value, ierr.value


class Context:
    """One GPU context: mesh, subdomain/BCs, resident system matrix."""

    def __init__(self, device: int = 0):
        self._L = load()
        h = C.c_void_p()
        rc = self._L.agb_create(C.byref(h), int(device))
        if rc != 0:
            raise AgbError(f"agb_create failed ({rc}): {self._L.agb_last_error(None).decode()}")
        self.h = h
        self.kind = None
        self.mesh = None

    def close(self):
        if getattr(self, "h", None):
            self._L.agb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        _check(rc, self.h)

    def set_mesh(self, mesh):
        self.mesh = mesh
        xyz = np.ascontiguousarray(mesh["xyz"], dtype=np.float64).ravel()
        et = np.ascontiguousarray(mesh["etype"], dtype=np.int32)
        con = np.ascontiguousarray(mesh["con"], dtype=np.int32).ravel()
        bc = np.ascontiguousarray(mesh["bcid"], dtype=np.int32)
        self.nnodes, self.nelem = len(mesh["xyz"]), len(et)
        self._ck(self._L.agb_set_mesh(self.h, self.nnodes, xyz, self.nelem, et, con, bc))

    def set_problem(self, kind, walls, known, normMul=None, diff=1.0, itri=5, iqud=4):
        walls = np.ascontiguousarray(walls, dtype=np.int32)
        nm = np.ones(len(walls)) if normMul is None else np.ascontiguousarray(normMul, dtype=np.float64)
        kn = np.ascontiguousarray(known, dtype=np.int32).ravel()
        self.kind = kind
        self.neq = 3 if kind == STOKES else 1
        self._ck(self._L.agb_set_problem(self.h, int(kind), len(walls), walls, nm, float(diff), kn, int(itri), int(iqud)))
        m, n = C.c_int(), C.c_int()
        self._ck(self._L.agb_system_size(self.h, C.byref(m), C.byref(n)))
        self.m, self.n = m.value, n.value

    def set_integration(self, sing_mode=0, rec_depth=20, near_eta=0.0, near_depth=0):
        """Triangle integration options: sing_mode 0 analytic / 1 recursive
        subdivision (rec_depth levels); near_eta > 0 enables the adaptive
        near-singular rule (near_depth levels).  Clears the assembled system."""
        self._ck(self._L.agb_set_integration(self.h, int(sing_mode), int(rec_depth), float(near_eta),
                                             int(near_depth)))

    def set_node_walls(self, node_wall=None):
        """Walls of the subdomain's nodes (wall id per global node, < 0 keeps the
        automatic assignment; None restores it for all): the reference's
        subdomain%BCidList after the BiC file's EDGE / CORNER directives, e.g.
        from :func:`andromeda_gb300.mesh.edge_corner_node_walls`.  Call after
        set_problem; clears the assembled system."""
        if node_wall is None:
            self._ck(self._L.agb_set_node_walls(self.h, self.nnodes, None))
            return
        w = np.ascontiguousarray(node_wall, dtype=np.int32)
        if w.shape != (self.nnodes,):
            raise ValueError("node_wall needs one entry per mesh node")
        self._ck(self._L.agb_set_node_walls(self.h, self.nnodes, w.ctypes.data_as(C.c_void_p)))

    def set_solver(self, solver, restart=None):
        """SOLVER_LSQR (default, lsqr_solve), SOLVER_LSQR_BLOCK (LSQR with the
        3x3 self-block preconditioner), SOLVER_BICGSTAB (the LIS path's BiCGSTAB
        with the Jacobi preconditioner), SOLVER_HYBRID (BiCGSTAB, LSQR where it
        does not converge) or SOLVER_GMRES (the LIS path with "-i gmres";
        restart: its restart length, default 40).  All but SOLVER_LSQR take
        packed mixed Stokes systems only."""
        self._ck(self._L.agb_set_solver(self.h, int(solver)))
        if restart is not None:
            self._ck(self._L.agb_set_gmres_restart(self.h, int(restart)))

    def set_residual_mode(self, mode):
        """0: float-float true residuals on the FP32 pipe (default); 1: FP64."""
        self._ck(self._L.agb_set_residual_mode(self.h, int(mode)))

    def surface_pressure(self, u, q):
        """Pressure at the element centroids (pressureStokes) of velocity u (3, nnodes)
        and traction q (3, nelem); elements of no subdomain wall get 0."""
        p = np.zeros(self.nelem)
        self._ck(self._L.agb_surface_pressure(self.h, np.ascontiguousarray(u, dtype=np.float64).ravel(),
                                              np.ascontiguousarray(q, dtype=np.float64).ravel(), p))
        return p

    def domain_values(self, points, u, q):
        """Field at points inside the domain: Stokes (npts, 4) velocity and pressure,
        Laplace (npts,); and the reference's check of each point."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = len(pts)
        nv = 4 if self.kind == STOKES else 1
        out = np.zeros(n * nv)
        err = np.zeros(n)
        self._ck(self._L.agb_domain_values(self.h, n, pts.ravel(), np.ascontiguousarray(u, dtype=np.float64).ravel(),
                                           np.ascontiguousarray(q, dtype=np.float64).ravel(), out, err))
        return (out.reshape(n, 4) if nv == 4 else out), err

    def geometry(self):
        nrm = np.zeros(3 * self.nelem)
        area = np.zeros(self.nelem)
        cen = np.zeros(3 * self.nelem)
        self._ck(self._L.agb_get_geometry(self.h, nrm, area, cen))
        return nrm.reshape(-1, 3), area, cen.reshape(-1, 3)

    def assemble(self, precision=FP64):
        self._ck(self._L.agb_assemble(self.h, int(precision)))

    def system(self, scaled=False):
        A = np.zeros((self.m, self.n))
        q = np.zeros(self.n)
        self._ck(self._L.agb_get_system(self.h, int(bool(scaled)), A.ctypes.data_as(C.c_void_p),
                                        q.ctypes.data_as(C.c_void_p)))
        return A, q

    def rhs(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        nrhs = u.shape[0]
        out = np.zeros((nrhs, self.m))
        self._ck(self._L.agb_rhs(self.h, nrhs, u.ravel(), out.reshape(-1)))
        return out

    def solve(self, u, x0=None, maxit=0, eps=1e-8, refine=0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        nrhs = u.shape[0]
        x = np.zeros((nrhs, self.n)) if x0 is None else np.array(x0, dtype=np.float64, copy=True).reshape(nrhs, self.n)
        nit = np.zeros(nrhs, np.int32)
        istop = np.zeros(nrhs, np.int32)
        self._ck(self._L.agb_solve(self.h, nrhs, u.ravel(), x.reshape(-1), int(maxit), float(eps), int(refine), nit, istop))
        return x, nit, istop

    def solve_lu(self, u):
        """Direct FP64 LU solve of the assembled square system (the FULL path):
        returns (x, info) with x in solve()'s layout."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        nrhs = u.shape[0]
        x = np.zeros((nrhs, self.n))
        info = C.c_int(0)
        self._ck(self._L.agb_solve_lu(self.h, nrhs, u.ravel(), x.reshape(-1), C.byref(info)))
        return x, info.value

    def force_torque(self, x, wall):
        x = np.ascontiguousarray(x, dtype=np.float64)
        nrhs = x.shape[0]
        ft = np.zeros((nrhs, 6))
        self._ck(self._L.agb_force_torque(self.h, nrhs, x.reshape(-1), int(wall), ft.reshape(-1)))
        return ft

    def layout_sizes(self):
        """(nsp, nn, nq, rows, unknowns, knowns) of the subdomain numbering."""
        out = np.zeros(6, np.int32)
        self._ck(self._L.agb_layout_sizes(self.h, out))
        return tuple(int(v) for v in out)

    def integral_matrices(self):
        """All-row integral matrices (the CoR_Integrals drop-in), FP64.

        Returns (T, G, errs): arrays of shape (ncomp, nsp, ncol) -- Laplace H/G
        (ncomp 1), Stokes T/prT and G/prG (ncomp 9) -- and the fSP/qSP errors.
        """
        nsp, nn, nq = self.layout_sizes()[:3]
        nc = 9 if self.kind == STOKES else 1
        T = np.zeros(nc * nsp * nn)
        G = np.zeros(nc * nsp * nq)
        e = np.zeros(2)
        self._ck(self._L.agb_integral_matrices(self.h, T.ctypes.data_as(C.c_void_p), G.ctypes.data_as(C.c_void_p),
                                               e.ctypes.data_as(C.c_void_p)))
        # column-major per component -> (ncomp, nsp, ncol)
        T = T.reshape(nc, nn, nsp).transpose(0, 2, 1)
        G = G.reshape(nc, nq, nsp).transpose(0, 2, 1)
        return T, G, e

    def solve_fields(self, u, q=None, maxit=0, eps=1e-8, refine=0):
        """Any-BC solve: known u (nodes) / q (elements) in, full fields out.

        ``u``: (nrhs, neq, nnodes), ``q``: (nrhs, neq, nelem) or None; both
        give the known values and the warm start of the unknowns.  Returns
        (u_out, q_out, nit, istop) with u_out/q_out in the same shapes.
        """
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, self.neq, self.nnodes)
        nrhs = u.shape[0]
        uo = np.zeros_like(u)
        qo = np.zeros((nrhs, self.neq, self.nelem))
        qp = None
        if q is not None:
            q = np.ascontiguousarray(q, dtype=np.float64).reshape(nrhs, self.neq, self.nelem)
            qp = q.ctypes.data_as(C.c_void_p)
        nit = np.zeros(nrhs, np.int32)
        istop = np.zeros(nrhs, np.int32)
        self._ck(self._L.agb_solve_fields(self.h, nrhs, u.ravel(), qp, uo.reshape(-1), qo.reshape(-1), int(maxit),
                                          float(eps), int(refine), nit, istop))
        return uo, qo, nit, istop

    def kernel_times(self, reset=False):
        """Cumulative live kernel times (ms) and launch counts since the last reset."""
        out = np.zeros(10)
        self._ck(self._L.agb_kernel_times(self.h, int(bool(reset)), out))
        return {"av_ms": out[0], "av_launches": int(out[1]), "atu_ms": out[2], "atu_launches": int(out[3]),
                "assemble_ms": out[4], "assemble_launches": int(out[5]), "rhs_ms": out[6], "rhs_calls": int(out[7]),
                "launches": int(out[8])}

    def resistance_tensor(self, precision=MIXED, particle_wall=1, outer_wall=2, maxit=0, eps=1e-8, refine=0):
        """Returns (R[6,6], nit[6], info): R[r] = (F, T) on the particle for rigid
        motion r of the container (e_x, e_y, e_z translations, then rotations)."""
        R = np.zeros((6, 6))
        nit = np.zeros(6, np.int32)
        istop = np.zeros(6, np.int32)
        t = np.zeros(6)
        self._ck(self._L.agb_resistance_tensor(self.h, int(precision), int(particle_wall), int(outer_wall), int(maxit),
                                               float(eps), int(refine), R.reshape(-1), nit, istop, t))
        return R, nit, {"assemble_ms": t[0], "rhs_ms": t[1], "solve_ms": t[2], "reduce_ms": t[3], "total_ms": t[4],
                        "device_ms": t[5], "istop": istop.tolist()}


def form_pre_fm(a, pret=2):
    """FormPREfm drop-in: returns (factors, q, ierr) for the square matrix a
    (pret 2: LU on the GPU; q = 1-based pivots; pret 1: q = 1/diag)."""
    L = load()
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    f = np.array(a.ravel(order="F"))
    q = np.zeros(n)
    cpu = C.c_float(0.0)
    ierr = C.c_int(0)
    _check(L.agb_form_pre_fm(int(pret), n, q, f, C.byref(cpu), C.byref(ierr)))
    return f.reshape((n, n), order="F"), q, ierr.value


def solv_eqn_fm(f, q, b, pret=2, prep=2):
    """SolvEQNfm drop-in (slvt 0): x = A^-1 b from form_pre_fm's output."""
    L = load()
    n = f.shape[0]
    fa = np.array(np.asarray(f, dtype=np.float64).ravel(order="F"))
    qq = np.array(q, dtype=np.float64)
    x = np.zeros(n)
    nit = C.c_int(-1)
    cpu = C.c_double(0.0)
    ierr = C.c_int(0)
    _check(L.agb_solv_eqn_fm(0, int(pret), int(prep), 0, 0, 0.0, n, qq, fa, np.ascontiguousarray(b, dtype=np.float64),
                             x, C.byref(nit), C.byref(cpu), C.byref(ierr)))
    return x, ierr.value


def batch_resistance(meshes, particle_wall=1, outer_wall=2, itri=5, maxit=0, eps=1e-7, mem_gb=0.0, autotune=True,
                     device=0, ctx=None, solver=None):
    """Mixed-precision resistance tensors of many bodies in one batched call.

    ``meshes``: list of particle-in-container triangle meshes (the dict layout
    of :mod:`andromeda_gb300.mesh`).  Returns (R[nb,6,6], nit[nb,6],
    istop[nb,6], stats) with R[i, r] = (F, T) on particle i for rigid motion r
    of its container.  ``ctx``: a :class:`Context` to run on (its per-body
    contexts are kept for later calls); a new one on ``device`` otherwise.
    ``solver``: SOLVER_LSQR / SOLVER_BICGSTAB for this call and the context's
    later ones (None: the context's setting, LSQR by default).
    """
    own = ctx is None
    C_ = Context(device) if own else ctx
    try:
        if solver is not None:
            C_.set_solver(solver)
        nb = len(meshes)
        node_off = np.zeros(nb + 1, np.int32)
        elem_off = np.zeros(nb + 1, np.int32)
        for i, m in enumerate(meshes):
            node_off[i + 1] = node_off[i] + len(m["xyz"])
            elem_off[i + 1] = elem_off[i] + len(m["etype"])
        xyz = np.ascontiguousarray(np.concatenate([m["xyz"] for m in meshes]), dtype=np.float64).ravel()
        et = np.ascontiguousarray(np.concatenate([m["etype"] for m in meshes]), dtype=np.int32)
        con = np.ascontiguousarray(np.concatenate([m["con"] for m in meshes]), dtype=np.int32).ravel()
        bc = np.ascontiguousarray(np.concatenate([m["bcid"] for m in meshes]), dtype=np.int32)
        R = np.zeros((nb, 6, 6))
        nit = np.zeros((nb, 6), np.int32)
        istop = np.zeros((nb, 6), np.int32)
        st = np.zeros(16)
        C_._ck(C_._L.agb_batch_resistance(C_.h, nb, node_off, xyz, elem_off, et, con, bc, int(particle_wall),
                                          int(outer_wall), int(itri), int(maxit), float(eps), float(mem_gb),
                                          int(bool(autotune)), R.reshape(-1), nit.reshape(-1), istop.reshape(-1), st))
        keys = ["assemble_ms", "solve_ms", "total_ms", "waves", "av_ms", "atu_ms", "av_launches", "atu_launches",
                "av_bytes", "launches", "av_rows", "atu_rs", "atu_rows", "iterations", "device_ms", "ft_ms"]
        return R, nit, istop, dict(zip(keys, st.tolist()))
    finally:
        if own:
            C_.close()


def dirichlet_known(kind, nwalls):
    neq = 3 if kind == STOKES else 1
    return np.full((neq, nwalls), BC_FUNCTION, dtype=np.int32)
