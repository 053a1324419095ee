"""The reference's file formats through the C ABI (host code, no GPU needed).

* :func:`read_mesh` -- surface meshes as ReadSurfaceMesh reads them
  (src/lib_meshRead.f90:80-160): gmsh 2.x and 4.x ASCII and the reference's
  "andromedaMesh" text format; returns the mesh dict of
  :mod:`andromeda_gb300.mesh` (0-based connectivity, element types 2/3, the
  wall id of every element) plus the named walls.
* :func:`write_vtu` -- the ParaView result file of OutputMeshParaview
  (src/lib_mesh.f90:218-392).
* :func:`write_integrals` / :func:`read_integrals` -- the integral-matrix cache
  and.integrals.bin (src/lib_int.f90:136-221, src/lib_Stokes.f90:2742-2876) in
  the matrices' layout of :meth:`andromeda_gb300.api.Context.integral_matrices`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import AgbError, load
from .api import LAPLACE, STOKES

NAME_LEN = 64


def _check(L, rc):
    if rc != 0:
        raise AgbError(f"andromeda_gb300 error {rc}: {L.agb_last_error(None).decode()}")


def read_mesh(path):
    """Mesh dict {xyz, etype, con, bcid} and walls {id: name} of a surface mesh file."""
    L = load()
    sizes = np.zeros(3, np.int32)
    _check(L, L.agb_mesh_read(str(path).encode(), sizes, None, None, None, None, None, None, 0))
    nn, ne, nw = (int(v) for v in sizes)
    xyz = np.zeros((nn, 3))
    etype = np.zeros(ne, np.int32)
    con = np.zeros((ne, 4), np.int32)
    bcid = np.zeros(ne, np.int32)
    ids = np.zeros(max(nw, 1), np.int32)
    names = C.create_string_buffer(max(nw, 1) * NAME_LEN)
    _check(L, L.agb_mesh_read(str(path).encode(), sizes, xyz.ctypes.data_as(C.c_void_p),
                              etype.ctypes.data_as(C.c_void_p), con.ctypes.data_as(C.c_void_p),
                              bcid.ctypes.data_as(C.c_void_p), ids.ctypes.data_as(C.c_void_p), names, NAME_LEN))
    walls = {int(ids[i]): names.raw[i * NAME_LEN:(i + 1) * NAME_LEN].split(b"\0")[0].decode() for i in range(nw)}
    return {"xyz": xyz, "etype": etype, "con": con, "bcid": bcid}, walls


def write_vtu(path, kind, mesh, normal, u, q, pressure=None, names=None):
    """OutputMeshParaview: u [neq][nnodes] nodal values, q [neq][nelem] fluxes
    / tractions, normal [nelem][3], the element pressure for Stokes."""
    L = load()
    u = np.ascontiguousarray(u, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    neq = u.shape[0]
    if names is None:
        names = ["x", "y", "z"] if kind == STOKES else ["1"]
    arr = (C.c_char_p * neq)(*[n.encode() for n in names])
    p = None
    if kind == STOKES:
        p = np.ascontiguousarray(pressure, dtype=np.float64)
    _check(L, L.agb_vtu_write(str(path).encode(), int(kind), len(mesh["xyz"]),
                              np.ascontiguousarray(mesh["xyz"], dtype=np.float64).ravel(), len(mesh["etype"]),
                              np.ascontiguousarray(mesh["etype"], dtype=np.int32),
                              np.ascontiguousarray(mesh["con"], dtype=np.int32).ravel(),
                              np.ascontiguousarray(mesh["bcid"], dtype=np.int32),
                              np.ascontiguousarray(normal, dtype=np.float64).ravel(), neq, arr, u.ravel(), q.ravel(),
                              None if p is None else p.ctypes.data_as(C.c_void_p)))


def write_integrals(path, kind, T, G, errs):
    """T (ncomp, nsp, nn), G (ncomp, nsp, nq) as Context.integral_matrices returns them."""
    L = load()
    T = np.asarray(T, dtype=np.float64)
    G = np.asarray(G, dtype=np.float64)
    nc, nsp, nn = T.shape
    nq = G.shape[2]
    if nc != (9 if kind == STOKES else 1):
        raise AgbError("write_integrals: wrong number of components")
    Tc = np.ascontiguousarray(T.transpose(0, 2, 1)).ravel()  # column-major per component
    Gc = np.ascontiguousarray(G.transpose(0, 2, 1)).ravel()
    _check(L, L.agb_integrals_file_write(str(path).encode(), int(kind), nsp, nn, nq,
                                         np.ascontiguousarray(errs, dtype=np.float64), Tc, Gc))


def read_integrals(path, kind):
    """(T, G, errs) of an integrals file, in the layout of write_integrals."""
    L = load()
    sizes = np.zeros(3, np.int32)
    errs = np.zeros(2)
    _check(L, L.agb_integrals_file_read(str(path).encode(), int(kind), sizes, errs, None, None))
    nsp, nn, nq = (int(v) for v in sizes)
    nc = 9 if kind == STOKES else 1
    T = np.zeros(nc * nsp * nn)
    G = np.zeros(nc * nsp * nq)
    _check(L, L.agb_integrals_file_read(str(path).encode(), int(kind), sizes, errs, T.ctypes.data_as(C.c_void_p),
                                        G.ctypes.data_as(C.c_void_p)))
    return T.reshape(nc, nn, nsp).transpose(0, 2, 1), G.reshape(nc, nq, nsp).transpose(0, 2, 1), errs


__all__ = ["read_mesh", "write_vtu", "write_integrals", "read_integrals", "LAPLACE", "STOKES"]
