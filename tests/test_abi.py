"""CPU tests of the C ABI: the library loads and exports every symbol the
header declares; argument checking needs no GPU."""
import ctypes as C
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "andromeda_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(agb_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(agb):
    L = agb.load()
    syms = declared_symbols()
    assert len(syms) >= 16
    for s in syms:
        assert hasattr(L, s), s
    from andromeda_gb300._lib import SIGNATURES
    assert sorted(SIGNATURES) == syms


def test_version_and_no_device_error(agb):
    L = agb.load()
    assert b"sm_103a" in L.agb_version()
    # a context on an absent / out-of-range device fails cleanly with a message
    h = C.c_void_p()
    rc = L.agb_create(C.byref(h), 1 << 20)
    assert rc != 0
    assert len(L.agb_last_error(None)) > 0


def test_lsqr_dropin_argument_checks(agb):
    L = agb.load()
    mi, nit, ierr = C.c_int(0), C.c_int(0), C.c_int(0)
    z = np.zeros(1)
    rc = L.agb_lsqr_solve(0, 0, 0, C.byref(mi), 1e-8, C.byref(nit), C.byref(ierr), z, np.zeros(1, np.int64),
                          np.zeros(1, np.int32), z, z, z)
    assert rc == 1  # AGB_ERR_ARG before any CUDA call


def _set_mesh_no_ctx(L, m):
    xyz = np.ascontiguousarray(m["xyz"], dtype=np.float64).ravel()
    et = np.ascontiguousarray(m["etype"], dtype=np.int32)
    con = np.ascontiguousarray(m["con"], dtype=np.int32).ravel()
    bc = np.ascontiguousarray(m["bcid"], dtype=np.int32)
    rc = L.agb_set_mesh(None, len(m["xyz"]), xyz, len(et), et, con, bc)
    return rc, L.agb_last_error(None).decode()


def test_mesh_checks_pass_every_generated_and_reference_mesh(agb):
    """The host checks of agb_set_mesh run before the context is used: every mesh
    the tests and the benchmark build gets through them (and then stops at the
    missing context)."""
    from andromeda_gb300 import mesh as M
    from fixtures import reference_mesh
    L = agb.load()
    meshes = [M.icosphere(lv, 1.0) for lv in range(4)]
    meshes += [M.quad_box(3, 2, 2, face_walls=True), M.quad_box(3, 2, 2, face_walls=True, triangles=True),
               M.particle_in_sphere(M.icosphere(2, 1.0, inward=True)),
               M.superellipsoid(1.0, 0.5, 0.25, 0.6, 1.4, 20, 40)]
    meshes += [reference_mesh(n) for n in ("sphere_01", "sphere_in_sphere_3678", "cube_624")]
    for m in meshes:
        rc, msg = _set_mesh_no_ctx(L, m)
        assert rc == 1 and msg == "agb_set_mesh: no context", msg


def test_mesh_checks_reject_defects(agb):
    """A coordinate that is not finite, connectivity out of range and degenerate
    elements (coincident or collinear nodes 1-3) are rejected with AGB_ERR_ARG
    and a message naming the node or element."""
    from andromeda_gb300 import mesh as M
    L = agb.load()
    base = M.icosphere(1, 1.0)

    def variant(**kw):
        m = {k: np.array(v, copy=True) for k, v in base.items()}
        for k, f in kw.items():
            f(m[k])
        return m

    def nan(x):
        x[7, 1] = np.nan

    def inf(x):
        x[3, 0] = np.inf

    def bad_con(c):
        c[5, 2] = 10_000

    def coincident(c):
        c[4, 1] = c[4, 0]

    def bad_type(t):
        t[2] = 7

    cases = [(variant(xyz=nan), "node 7"), (variant(xyz=inf), "node 3"),
             (variant(con=bad_con), "element 5: connectivity"), (variant(con=coincident), "element 4 is degenerate"),
             (variant(etype=bad_type), "element 2: type")]
    # collinear nodes 1-3: move node 2 of element 9 onto the line through nodes 1 and 3
    m = variant()
    c = m["con"][9]
    m["xyz"][c[1]] = 0.5 * (m["xyz"][c[0]] + m["xyz"][c[2]])
    cases.append((m, "is degenerate"))
    for m, want in cases:
        rc, msg = _set_mesh_no_ctx(L, m)
        assert rc == 1 and want in msg, msg


def test_batch_checks_run_without_context(agb):
    """agb_batch_resistance checks every body's mesh before the context: sound
    bodies stop at the missing context, a degenerate element is named with its
    body."""
    from andromeda_gb300 import mesh as M
    L = agb.load()
    bodies = [M.particle_in_sphere(M.icosphere(1, 1.0, inward=True), outer_level=1, outer_radius=20.0)
              for _ in range(3)]

    def call(bodies):
        node_off = np.cumsum([0] + [len(b["xyz"]) for b in bodies]).astype(np.int32)
        elem_off = np.cumsum([0] + [len(b["etype"]) for b in bodies]).astype(np.int32)
        xyz = np.concatenate([b["xyz"] for b in bodies]).ravel()
        et = np.concatenate([b["etype"] for b in bodies]).astype(np.int32)
        con = np.concatenate([b["con"] for b in bodies]).astype(np.int32).ravel()
        bc = np.concatenate([b["bcid"] for b in bodies]).astype(np.int32)
        R = np.zeros(36 * len(bodies))
        nit = np.zeros(6 * len(bodies), np.int32)
        ist = np.zeros(6 * len(bodies), np.int32)
        rc = L.agb_batch_resistance(None, len(bodies), node_off, xyz, elem_off, et, con, bc, 1, 2, 5, 100, 1e-6,
                                    0.0, 0, R, nit, ist, np.zeros(16))
        return rc, L.agb_last_error(None).decode()

    rc, msg = call(bodies)
    assert rc == 1 and msg == "agb_batch_resistance: no context", msg
    bad = {k: np.array(v, copy=True) for k, v in bodies[1].items()}
    bad["con"][3, 2] = bad["con"][3, 1]
    rc, msg = call([bodies[0], bad, bodies[2]])
    assert rc == 1 and msg.startswith("batched body 1: element") and "degenerate" in msg, msg
