"""ctypes front end of the CPU FP64 oracle (liborc.so) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline legs import
this module.  It restates the reference algorithms; it is the checker, never
the thing measured as the GPU product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
_lib = None

dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile liborc.so with the committed Makefile (g++, OpenMP)."""
    src = os.path.join(HERE, "bem_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_wx_rule.argtypes = [C.c_int, dp, dp, dp, dp]
        L.orc_wx_rule.restype = C.c_int
        L.orc_triangle_test.argtypes = [C.c_int, dp]
        L.orc_tri_area.argtypes = [dp]
        L.orc_tri_area.restype = C.c_double
        L.orc_si_tri_lap.argtypes = [dp, C.c_int]
        L.orc_si_tri_lap.restype = C.c_double
        L.orc_si_tri_stk.argtypes = [dp, C.c_int, dp]
        L.orc_si_qua_lap.argtypes = [dp, C.c_int]
        L.orc_si_qua_lap.restype = C.c_double
        L.orc_si_qua_stk.argtypes = [dp, C.c_int, dp]
        L.orc_quad_lap_polar.argtypes = [C.c_int, dp, dp, C.c_int, C.c_double, dp]
        L.orc_quad_stk_polar.argtypes = [C.c_int, dp, dp, C.c_int, C.c_double, dp]
        L.orc_tri_lap_regular.argtypes = [C.c_int, dp, dp, dp, dp]
        L.orc_tri_stk_regular.argtypes = [C.c_int, dp, dp, dp, dp]
        L.orc_problem_create.argtypes = [C.c_int, C.c_int, dp, C.c_int, ip, ip, ip, C.c_int, ip, dp, C.c_double, ip,
                                         C.c_int, C.c_int]
        L.orc_problem_create.restype = C.c_void_p
        L.orc_problem_destroy.argtypes = [C.c_void_p]
        L.orc_problem_edge_corner.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_problem_set_node_walls.argtypes = [C.c_void_p, ip]
        L.orc_problem_node_walls.argtypes = [C.c_void_p, ip]
        L.orc_dgefa.argtypes = [dp, C.c_int, C.c_int, dp]
        L.orc_dgefa.restype = C.c_int
        L.orc_dgesl.argtypes = [dp, C.c_int, C.c_int, dp, dp, C.c_int]
        L.orc_problem_set_integration.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int]
        L.orc_tri_lap_opt.argtypes = [C.c_int, dp, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, dp]
        L.orc_tri_stk_opt.argtypes = [C.c_int, dp, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, dp]
        L.orc_problem_sizes.argtypes = [C.c_void_p, ip]
        L.orc_geometry.argtypes = [C.c_void_p, dp, dp, dp]
        L.orc_lists.argtypes = [C.c_void_p, ip, ip]
        L.orc_form_integrals.argtypes = [C.c_void_p, dp]
        L.orc_get_integral_matrix.argtypes = [C.c_void_p, C.c_int, dp]
        L.orc_integral_row.argtypes = [C.c_void_p, C.c_int, dp, dp]
        L.orc_integral_row.restype = C.c_double
        L.orc_form_system.argtypes = [C.c_void_p]
        L.orc_crs_nnz.argtypes = [C.c_void_p, C.c_int]
        L.orc_crs_nnz.restype = C.c_int64
        L.orc_get_crs.argtypes = [C.c_void_p, C.c_int, lp, ip, dp]
        L.orc_lsqr_precon.argtypes = [C.c_int, C.c_int, C.c_int64, dp, lp, ip, dp]
        L.orc_lsqr_solve.argtypes = [C.c_int, C.c_int, C.c_int64, C.POINTER(C.c_int), C.c_double,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), dp, lp, ip, dp, dp, dp, dp]
        L.orc_laplace_solve.argtypes = [C.c_void_p, dp, dp, C.c_int, C.c_double, C.POINTER(C.c_int)]
        L.orc_laplace_solve.restype = C.c_int
        L.orc_stokes_solve_sequence.argtypes = [C.c_void_p, C.c_int, dp, dp, C.c_int, C.c_double, C.c_int, dp, ip]
        L.orc_stokes_solve_sequence.restype = C.c_int
        L.orc_force_torque.argtypes = [C.c_void_p, dp, dp, dp, C.c_int, dp]
        L.orc_stokes_solve_lis.argtypes = [C.c_void_p, C.c_int, dp, dp, C.c_double, C.c_int, C.c_int, dp, ip, ip,
                                           dp]
        L.orc_stokes_solve_lis.restype = C.c_int
        L.orc_stokes_solve_lis_m.argtypes = [C.c_void_p, C.c_int, dp, dp, C.c_double, C.c_int, C.c_int, dp, ip, ip,
                                             dp, C.c_int, C.c_int]
        L.orc_stokes_solve_lis_m.restype = C.c_int
        L.orc_pressure_stokes.argtypes = [C.c_void_p, dp, dp, dp]
        L.orc_pressure_stokes.restype = C.c_int
        L.orc_domain_values.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp, dp]
        L.orc_time_rows.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.orc_time_rows.restype = C.c_double
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def wx_rule(itri: int):
    n = 130
    l1, l2, l3, w = (np.zeros(n) for _ in range(4))
    k = lib().orc_wx_rule(itri, l1, l2, l3, w)
    return l1[:k], l2[:k], l3[:k], w[:k]


def triangle_test(itri: int):
    out = np.zeros(4)
    lib().orc_triangle_test(itri, out)
    return out


def si_tri_lap(v, isrc):
    return lib().orc_si_tri_lap(np.ascontiguousarray(v, dtype=np.float64).ravel(), isrc)


def si_tri_stk(v, isrc):
    G = np.zeros(6)
    lib().orc_si_tri_stk(np.ascontiguousarray(v, dtype=np.float64).ravel(), isrc, G)
    return G


def si_qua_lap(q, isrc):
    return lib().orc_si_qua_lap(np.ascontiguousarray(q, dtype=np.float64).ravel(), isrc)


def si_qua_stk(q, isrc):
    G = np.zeros(6)
    lib().orc_si_qua_stk(np.ascontiguousarray(q, dtype=np.float64).ravel(), isrc, G)
    return G


def quad_lap_polar(iqud, q, s, isrc, multi=1.0):
    """Singular branch of Quad_BEMInt (polar Gauss about local node isrc):
    (G, H[4])."""
    out = np.zeros(5)
    lib().orc_quad_lap_polar(int(iqud), np.ascontiguousarray(q, dtype=np.float64).ravel(),
                             np.ascontiguousarray(s, dtype=np.float64).ravel(), int(isrc), float(multi), out)
    return out[0], out[1:]


def quad_stk_polar(iqud, q, s, isrc, multi=1.0):
    """Singular branch of Quad_StokesInt: the six Stokeslet integrals."""
    G = np.zeros(6)
    lib().orc_quad_stk_polar(int(iqud), np.ascontiguousarray(q, dtype=np.float64).ravel(),
                             np.ascontiguousarray(s, dtype=np.float64).ravel(), int(isrc), float(multi), G)
    return G


def tri_lap_regular(itri, v, s, n):
    out = np.zeros(4)
    lib().orc_tri_lap_regular(itri, np.ascontiguousarray(v, float).ravel(), np.ascontiguousarray(s, float),
                              np.ascontiguousarray(n, float), out)
    return out


def tri_stk_regular(itri, v, s, n):
    out = np.zeros(36)
    lib().orc_tri_stk_regular(itri, np.ascontiguousarray(v, float).ravel(), np.ascontiguousarray(s, float),
                              np.ascontiguousarray(n, float), out)
    return out


def tri_lap_opt(itri, v, s, n, isrc=0, sing=0, rdepth=20, near_eta=0.0, near_depth=0):
    """Triangle Laplace integrals {G, H1, H2, H3} under the integration options."""
    out = np.zeros(4)
    lib().orc_tri_lap_opt(itri, np.ascontiguousarray(v, float).ravel(), np.ascontiguousarray(s, float),
                          np.ascontiguousarray(n, float), isrc, sing, rdepth, near_eta, near_depth, out)
    return out


def tri_stk_opt(itri, v, s, n, isrc=0, sing=0, rdepth=20, near_eta=0.0, near_depth=0):
    """Triangle Stokes integrals G[6], prG[3], T[6][3], prT[3][3] under the integration options."""
    out = np.zeros(36)
    lib().orc_tri_stk_opt(itri, np.ascontiguousarray(v, float).ravel(), np.ascontiguousarray(s, float),
                          np.ascontiguousarray(n, float), isrc, sing, rdepth, near_eta, near_depth, out)
    return out


def dgefa(a):
    """LINPACK LU (lib_solveFM.f:198) of a square matrix: returns (factors in
    LINPACK storage, ipvt 1-based as float64, info)."""
    a = np.array(a, dtype=np.float64, order="F", copy=True)
    n = a.shape[0]
    ipvt = np.zeros(n)
    flat = a.ravel(order="F")
    info = lib().orc_dgefa(flat, n, n, ipvt)
    return flat.reshape((n, n), order="F"), ipvt, int(info)


def dgesl(f, ipvt, b, job=0):
    """LINPACK solve (lib_solveFM.f:318) with dgefa's output."""
    f = np.asarray(f, dtype=np.float64)
    n = f.shape[0]
    flat = np.ascontiguousarray(f.ravel(order="F"))
    x = np.array(b, dtype=np.float64, copy=True)
    lib().orc_dgesl(flat, n, n, np.ascontiguousarray(ipvt, dtype=np.float64), x, int(job))
    return x


class Problem:
    """Mesh + one subdomain + BCs, mirroring the reference's module state."""

    def __init__(self, kind, mesh, walls, known, normMul=None, diff=1.0, itri=5, iqud=4):
        self.kind = kind
        self.mesh = mesh
        walls = np.ascontiguousarray(walls, dtype=np.int32)
        if normMul is None:
            normMul = np.ones(len(walls))
        known = np.ascontiguousarray(known, dtype=np.int32).ravel()
        self.nnodes = len(mesh["xyz"])
        self.nelem = len(mesh["etype"])
        self._keep = (np.ascontiguousarray(mesh["xyz"], dtype=np.float64).ravel(),
                      np.ascontiguousarray(mesh["etype"], dtype=np.int32),
                      np.ascontiguousarray(mesh["con"], dtype=np.int32).ravel(),
                      np.ascontiguousarray(mesh["bcid"], dtype=np.int32), walls,
                      np.ascontiguousarray(normMul, dtype=np.float64), known)
        x, et, con, bc, w, nm, kn = self._keep
        self.h = lib().orc_problem_create(kind, self.nnodes, x, self.nelem, et, con, bc, len(w), w, nm, float(diff), kn,
                                          itri, iqud)
        s = np.zeros(6, dtype=np.int32)
        lib().orc_problem_sizes(self.h, s)
        self.nsp, self.sd_nnodes, self.sd_nqnodes, self.neq_rows, self.nx, self.nb = map(int, s)

    def close(self):
        if self.h:
            lib().orc_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def edge_rule(self, w1, w2, target):
        """EDGE directive of the BiC file (HandleCornersEdges, lib_sdBem.f90:148-215)."""
        lib().orc_problem_edge_corner(self.h, int(w1), int(w2), -1, int(target))
        self._resize()

    def corner_rule(self, w1, w2, w3, target):
        """CORNER directive of the BiC file (HandleCornersEdges, lib_sdBem.f90:217-292)."""
        lib().orc_problem_edge_corner(self.h, int(w1), int(w2), int(w3), int(target))
        self._resize()

    def set_node_walls(self, node_wall):
        """subdomain%BCidList from the caller: wall id per global node, < 0 keeps it."""
        lib().orc_problem_set_node_walls(self.h, np.ascontiguousarray(node_wall, dtype=np.int32))
        self._resize()

    def node_walls(self):
        """BCidList as wall id per global node (-1: not a node of the subdomain)."""
        out = np.zeros(self.nnodes, np.int32)
        lib().orc_problem_node_walls(self.h, out)
        return out

    def _resize(self):
        s = np.zeros(6, dtype=np.int32)
        lib().orc_problem_sizes(self.h, s)
        self.nsp, self.sd_nnodes, self.sd_nqnodes, self.neq_rows, self.nx, self.nb = map(int, s)

    def geometry(self):
        n = np.zeros(3 * self.nelem)
        a = np.zeros(self.nelem)
        c = np.zeros(3 * self.nelem)
        lib().orc_geometry(self.h, n, a, c)
        return n.reshape(-1, 3), a, c.reshape(-1, 3)

    def lists(self):
        nl = np.zeros(self.sd_nnodes, np.int32)
        ql = np.zeros(self.sd_nqnodes, np.int32)
        lib().orc_lists(self.h, nl, ql)
        return nl, ql

    def set_integration(self, sing=0, rdepth=20, near_eta=0.0, near_depth=0):
        """Integration options of the triangle integrals (IntegOpt of the oracle)."""
        lib().orc_problem_set_integration(self.h, int(sing), int(rdepth), float(near_eta), int(near_depth))

    def form_integrals(self):
        e = np.zeros(2)
        lib().orc_form_integrals(self.h, e)
        return e

    def integral_matrix(self, which):
        ncol = self.sd_nnodes if (which == 0 or (self.kind == 2 and which < 9)) else self.sd_nqnodes
        out = np.zeros(self.nsp * ncol)
        lib().orc_get_integral_matrix(self.h, which, out)
        return out.reshape(ncol, self.nsp).T  # (nsp, ncol)

    def integral_row(self, r):
        k = 9 if self.kind == 2 else 1
        rt = np.zeros(k * self.nnodes)
        rg = np.zeros(k * self.nelem)
        err = lib().orc_integral_row(self.h, r, rt, rg)
        return rt.reshape(k, self.nnodes), rg.reshape(k, self.nelem), err

    def form_system(self):
        lib().orc_form_system(self.h)

    def crs(self, which):
        nnz = lib().orc_crs_nnz(self.h, which)
        ia = np.zeros(self.neq_rows + 1, np.int64)
        ja = np.zeros(max(nnz, 1), np.int32)
        a = np.zeros(max(nnz, 1))
        lib().orc_get_crs(self.h, which, ia, ja, a)
        return ia, ja[:nnz], a[:nnz]

    def dense(self, which):
        ia, ja, a = self.crs(which)
        ncol = self.nx if which == 0 else self.nb
        M = np.zeros((self.neq_rows, ncol))
        for r in range(self.neq_rows):
            s, e = ia[r] - 1, ia[r + 1] - 1
            M[r, ja[s:e] - 1] = a[s:e]
        return M

    def laplace_solve(self, u, q, maxit=0, eps=1e-12):
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        q = np.ascontiguousarray(q, dtype=np.float64).copy()
        nit = C.c_int(0)
        ierr = lib().orc_laplace_solve(self.h, u, q, maxit, eps, C.byref(nit))
        return u, q, nit.value, ierr

    def stokes_solve_sequence(self, u_fields, maxit=0, eps=1e-12, fwall=1):
        u_fields = np.ascontiguousarray(u_fields, dtype=np.float64)
        nrhs = u_fields.shape[0]
        q = np.zeros((nrhs, 3, self.nelem))
        ft = np.zeros((nrhs, 6))
        nits = np.zeros(nrhs, np.int32)
        ierr = lib().orc_stokes_solve_sequence(self.h, nrhs, u_fields.ravel(), q.reshape(-1), maxit, eps, fwall,
                                               ft.reshape(-1), nits)
        return q, ft, nits, ierr

    def stokes_solve_lis(self, u_fields, tol=1e-8, maxiter=1000, fwall=1, method="bicgstab", restart=40):
        """The LIS path (StokesBigSystemSOLVElis, lib_StokesLis.f90:4) with the
        reference's default LIS options: BiCGSTAB, Jacobi, tol 1e-8, 1000 iterations
        (method "gmres": GMRES(restart) with the node/element block preconditioner).
        Returns (q [nrhs, 3, nelem], force/torque [nrhs, 6], iterations, status,
        relative residual); status 0 converged, 1 iteration limit, 2 breakdown,
        3 not one equation per unknown (GMRES: or stagnated)."""
        u_fields = np.ascontiguousarray(u_fields, dtype=np.float64)
        nrhs = u_fields.shape[0]
        q = np.zeros((nrhs, 3, self.nelem))
        ft = np.zeros((nrhs, 6))
        nits = np.zeros(nrhs, np.int32)
        status = np.zeros(nrhs, np.int32)
        relres = np.zeros(nrhs)
        lib().orc_stokes_solve_lis_m(self.h, nrhs, u_fields.ravel(), q.reshape(-1), float(tol), int(maxiter), fwall,
                                     ft.reshape(-1), nits, status, relres, {"bicgstab": 0, "gmres": 1}[method],
                                     int(restart))
        return q, ft, nits, status, relres

    def time_rows(self, r0, r1, nthreads):
        cs = C.c_double(0.0)
        t = lib().orc_time_rows(self.h, int(r0), int(r1), int(nthreads), C.byref(cs))
        return t, cs.value

    def force_torque(self, q3, wall):
        ft = np.zeros(6)
        q3 = np.ascontiguousarray(q3, dtype=np.float64)
        lib().orc_force_torque(self.h, q3[0].copy(), q3[1].copy(), q3[2].copy(), wall, ft)
        return ft

    def pressure(self, u3, q3):
        """Surface pressure at the q-source points (pressureStokes, lib_Stokes.f90:4-94)
        of the velocity u3 (3, nnodes) and traction q3 (3, nelem); needs form_integrals."""
        p = np.zeros(self.sd_nqnodes)
        rc = lib().orc_pressure_stokes(self.h, np.ascontiguousarray(u3, dtype=np.float64).ravel(),
                                       np.ascontiguousarray(q3, dtype=np.float64).ravel(), p)
        if rc != 0:
            raise RuntimeError("pressure needs the Stokes integral matrices (form_integrals)")
        return p

    def domain_values(self, points, u, q):
        """Field at points inside the domain (GetStokesDomainValue lib_Stokes.f90:3043,
        GetSubDomainValue lib_domain.f90:210).  Stokes: u (3, nnodes), q (3, nelem) ->
        (npts, 4) = velocity and pressure; Laplace: u (nnodes,), q (nelem,) -> (npts,).
        Also returns the reference's integration check of each point (small inside)."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = len(pts)
        out = np.zeros(n * (4 if self.kind == 2 else 1))
        err = np.zeros(n)
        lib().orc_domain_values(self.h, n, pts.ravel(), np.ascontiguousarray(u, dtype=np.float64).ravel(),
                                np.ascontiguousarray(q, dtype=np.float64).ravel(), out, err)
        return (out.reshape(n, 4) if self.kind == 2 else out), err


def lsqr_precon(m, n, ia, ja, a):
    q = np.zeros(n)
    lib().orc_lsqr_precon(m, n, len(a), q, ia, ja, a)
    return q


def lsqr_solve(m, n, ia, ja, a, q, b, x, maxit=0, eps=1e-12):
    mi = C.c_int(maxit)
    nit = C.c_int(0)
    ierr = C.c_int(0)
    st = np.zeros(7)
    lib().orc_lsqr_solve(m, n, len(a), C.byref(mi), eps, C.byref(nit), C.byref(ierr), q, ia, ja, a,
                         np.ascontiguousarray(b, dtype=np.float64), x, st)
    return nit.value, ierr.value, st


def set_threads(n):
    lib().orc_set_threads(int(n))


def num_threads():
    return lib().orc_num_threads()
