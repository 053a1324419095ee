"""The reference's file formats through the C ABI, on the CPU (host code only).

* agb_mesh_read: the reference's own run meshes, as converted once into
  tests/golden/*.npz, written back as gmsh 2.2, gmsh 4.1 and andromedaMesh text
  and read again -- coordinates, connectivity and wall ids equal; rOneTL's
  rules (blank lines and lines holding '#' skipped); the element blocks of
  other dimensions of a gmsh 4 file skipped; the errors of the reference's
  readers (unsupported element type, a node tag out of range, not a mesh file).
* agb_vtu_write: the OutputMeshParaview file parsed back as XML.
* agb_integrals_file_write / _read: and.integrals.bin record by record
  (gfortran sequential unformatted: int32 length before and after each record;
  columns in records of 8192 values, an empty record after a column whose
  length is a multiple of 8192), Laplace and Stokes round trips.
"""
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from fixtures import reference_mesh

FIXTURES = ["sphere_01", "sphere_in_sphere_3678", "ellipsoid211_in_sphere_2117", "cube_624", "surf_tri_kocka",
            "quad_kocka_150"]


def _io():
    from andromeda_gb300 import io as IO
    return IO


def _gmsh2(m, names):
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(names))]
    out += [f'2 {k} "{v}"' for k, v in names.items()]
    out += ["$EndPhysicalNames", "$Nodes", str(len(m["xyz"]))]
    out += [f"{i + 1} {x:.17g} {y:.17g} {z:.17g}" for i, (x, y, z) in enumerate(m["xyz"])]
    out += ["$EndNodes", "$Elements", str(len(m["etype"]))]
    for e, (t, bc) in enumerate(zip(m["etype"], m["bcid"])):
        nno = 3 if t == 2 else 4
        con = " ".join(str(int(v) + 1) for v in m["con"][e, :nno])
        out.append(f"{e + 1} {t} 2 {bc} {bc + 100} {con}")
    out += ["$EndElements"]
    return "\n".join(out) + "\n"


def _gmsh4(m, names, extra_line_block=False):
    walls = sorted(set(int(b) for b in m["bcid"]))
    nn, ne = len(m["xyz"]), len(m["etype"])
    out = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(names))]
    out += [f'2 {k} "{v}"' for k, v in names.items()]
    out += ["$EndPhysicalNames", "$Entities", f"0 {1 if extra_line_block else 0} {len(walls)} 1"]
    if extra_line_block:
        out.append("1 0 0 0 1 1 1 0 2 1 2")
    for s, w in enumerate(walls):
        out.append(f"{s + 11} -1 -1 -1 1 1 1 1 {w} 0")
    out.append("1 -1 -1 -1 1 1 1 0 0")
    out += ["$EndEntities", "$Nodes", f"1 {nn} 1 {nn}", f"2 11 0 {nn}"]
    out += [str(i + 1) for i in range(nn)]
    out += [f"{x:.17g} {y:.17g} {z:.17g}" for x, y, z in m["xyz"]]
    out += ["$EndNodes"]
    blocks = []
    tag = 1
    for s, w in enumerate(walls):
        es = np.where(m["bcid"] == w)[0]
        for t in (2, 3):
            sel = [e for e in es if m["etype"][e] == t]
            if not sel:
                continue
            lines = []
            for e in sel:
                nno = 3 if t == 2 else 4
                lines.append(f"{e + 1} " + " ".join(str(int(v) + 1) for v in m["con"][e, :nno]))
            blocks.append((f"2 {s + 11} {t} {len(sel)}", lines))
    if extra_line_block:
        blocks.insert(0, ("1 1 1 2", [f"{ne + 1} 1 2", f"{ne + 2} 2 3"]))
    ntot = ne + (2 if extra_line_block else 0)
    out += ["$Elements", f"{len(blocks)} {ntot} 1 {ntot}"]
    for head, lines in blocks:
        out.append(head)
        out += lines
    out += ["$EndElements"]
    return "\n".join(out) + "\n"


def _andromeda(m, names):
    out = ["andromedaMesh", "1.0", str(len(names))] + [f"{k} {v}" for k, v in names.items()]
    out.append(str(len(m["xyz"])))
    out += [f"{i + 1} {x:.17g} {y:.17g} {z:.17g}" for i, (x, y, z) in enumerate(m["xyz"])]
    out.append(str(len(m["etype"])))
    for e, (t, bc) in enumerate(zip(m["etype"], m["bcid"])):
        nno = 3 if t == 2 else 4
        out.append(f"{e + 1} {bc} {nno} " + " ".join(str(int(v) + 1) for v in m["con"][e, :nno]))
    return "\n".join(out) + "\n"


def _same(a, b):
    nno = np.where(b["etype"] == 2, 3, 4)
    assert np.array_equal(a["xyz"], b["xyz"])
    assert np.array_equal(a["etype"], b["etype"]) and np.array_equal(a["bcid"], b["bcid"])
    for e in range(len(nno)):
        assert np.array_equal(a["con"][e, :nno[e]], b["con"][e, :nno[e]])
    assert np.all(a["con"][nno == 3, 3] == -1)


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("fmt", ["gmsh2", "gmsh4", "andromeda"])
def test_mesh_read_round_trip(tmp_path, name, fmt):
    IO = _io()
    m = reference_mesh(name)
    names = {int(w): f"wall{int(w)}" for w in sorted(set(m["bcid"]))}
    text = {"gmsh2": _gmsh2, "gmsh4": _gmsh4, "andromeda": _andromeda}[fmt](m, names)
    p = tmp_path / f"{name}.msh"
    p.write_text(text)
    got, walls = IO.read_mesh(p)
    _same(got, m)
    assert walls == names


def test_mesh_read_quads_comments_and_skipped_blocks(tmp_path):
    IO = _io()
    from andromeda_gb300 import mesh as M
    m = M.quad_box(2, 1, 1, face_walls=True)
    names = {int(w): f"face {int(w)}" for w in sorted(set(m["bcid"]))}
    # rOneTL: blank lines and every line holding '#' are skipped
    text = _gmsh2(m, names).replace("$Nodes\n", "$Nodes\n\n# a comment line\n")
    (tmp_path / "a.msh").write_text(text)
    got, walls = IO.read_mesh(tmp_path / "a.msh")
    _same(got, m)
    assert walls == names
    # gmsh 4 with a block of line elements and a volume entity: only the surface blocks are read
    (tmp_path / "b.msh").write_text(_gmsh4(m, names, extra_line_block=True))
    got, _ = IO.read_mesh(tmp_path / "b.msh")
    _same(got, m)


def test_mesh_read_errors(tmp_path):
    IO = _io()
    from andromeda_gb300 import AgbError
    m = reference_mesh("cube_624")
    names = {1: "top"}
    bad = _gmsh2(m, names).replace("\n1 2 2 ", "\n1 1 2 ", 1)  # the first element becomes a 2-node line
    (tmp_path / "line.msh").write_text(bad)
    with pytest.raises(AgbError, match="element type 1 not supported"):
        IO.read_mesh(tmp_path / "line.msh")
    text = _gmsh2(m, names)
    nn = len(m["xyz"])
    (tmp_path / "tag.msh").write_text(text.replace(f"\n{nn} ", f"\n{nn + 5} ", 1))
    with pytest.raises(AgbError, match="outside"):
        IO.read_mesh(tmp_path / "tag.msh")
    (tmp_path / "geo.geo").write_text("Point(1) = {0, 0, 0};\n")
    with pytest.raises(AgbError, match="invalid surface mesh file"):
        IO.read_mesh(tmp_path / "geo.geo")
    (tmp_path / "bin.msh").write_text("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(AgbError, match="binary"):
        IO.read_mesh(tmp_path / "bin.msh")
    with pytest.raises(AgbError, match="cannot open"):
        IO.read_mesh(tmp_path / "missing.msh")


def test_vtu_write_stokes(tmp_path):
    IO = _io()
    from andromeda_gb300 import STOKES
    m = reference_mesh("cube_624")
    nn, ne = len(m["xyz"]), len(m["etype"])
    rng = np.random.default_rng(0)
    u = rng.normal(size=(3, nn))
    q = rng.normal(size=(3, ne))
    p = rng.normal(size=ne)
    normal = rng.normal(size=(ne, 3))
    IO.write_vtu(tmp_path / "r.vtu", STOKES, m, normal, u, q, pressure=p)
    root = ET.parse(tmp_path / "r.vtu").getroot()
    assert root.tag == "VTKFile" and root.get("type") == "UnstructuredGrid"
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == nn and int(piece.get("NumberOfCells")) == ne
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=float) for a in piece.iter("DataArray") if a.get("Name")}
    assert np.allclose(arrays["u"].reshape(nn, 3), u.T, rtol=1e-8)
    assert np.allclose(arrays["ux"], u[0], rtol=1e-8) and np.allclose(arrays["qz"], q[2], rtol=1e-8)
    assert np.allclose(arrays["pressure"], p, rtol=1e-8)
    assert np.array_equal(arrays["elemBCid"], m["bcid"]) and np.array_equal(arrays["node"], np.arange(1, nn + 1))
    assert np.array_equal(arrays["connectivity"].reshape(ne, 3), m["con"][:, :3])
    assert np.array_equal(arrays["offsets"], 3 * np.arange(1, ne + 1)) and np.all(arrays["types"] == 5)
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=float).reshape(nn, 3)
    assert np.allclose(pts, m["xyz"], rtol=1e-8, atol=1e-12)
    assert piece.find("PointData").get("Scalars") == "node,ux,uy,uz"
    assert piece.find("CellData").get("Scalars") == "pressure,elemBCid,qx,qy,qz"


def _records(path):
    raw = open(path, "rb").read()
    out, i = [], 0
    while i < len(raw):
        (n,) = struct.unpack_from("<i", raw, i)
        out.append(raw[i + 4:i + 4 + n])
        (n2,) = struct.unpack_from("<i", raw, i + 4 + n)
        assert n2 == n
        i += 8 + n
    return out


@pytest.mark.parametrize("kind", ["laplace", "stokes"])
def test_integrals_file_round_trip(tmp_path, kind):
    IO = _io()
    from andromeda_gb300 import LAPLACE, STOKES
    k = LAPLACE if kind == "laplace" else STOKES
    nc = 1 if k == LAPLACE else 9
    nsp, nn, nq = 8192, 3, 2  # columns of exactly one chunk: each ends with an empty record
    rng = np.random.default_rng(1)
    T = rng.normal(size=(nc, nsp, nn))
    G = rng.normal(size=(nc, nsp, nq))
    errs = np.array([1.5e-9, 2.5e-7])
    p = tmp_path / "and.integrals.bin"
    IO.write_integrals(p, k, T, G, errs)
    T2, G2, e2 = IO.read_integrals(p, k)
    assert np.array_equal(T, T2) and np.array_equal(G, G2) and np.array_equal(errs, e2)
    rec = _records(p)
    off = 0
    if k == STOKES:
        assert struct.unpack("<i", rec[0]) == (1407,)
        off = 1
    assert struct.unpack("<3i", rec[off]) == (nsp, nn, nq)
    assert struct.unpack("<2d", rec[off + 1]) == tuple(errs)
    mats = rec[off + 2:]
    ncols = nc * (nn + nq)
    assert len(mats) == 2 * ncols  # a full record and an empty one per column
    assert all(len(r) == 8 * 8192 for r in mats[0::2]) and all(len(r) == 0 for r in mats[1::2])
    first = np.frombuffer(mats[0], dtype="<f8")
    assert np.array_equal(first, T[0][:, 0])  # Hmat / Txx, column 1
    if k == STOKES:
        # the file order Txx, Tyy, Tzz, Txy, ...: the second matrix is Tyy (component 3 here)
        second = np.frombuffer(mats[2 * nn], dtype="<f8")
        assert np.array_equal(second, T[3][:, 0])


def test_integrals_file_chunks_and_checks(tmp_path):
    IO = _io()
    from andromeda_gb300 import AgbError, LAPLACE, STOKES
    nsp, nn, nq = 10000, 2, 1
    rng = np.random.default_rng(2)
    T = rng.normal(size=(1, nsp, nn))
    G = rng.normal(size=(1, nsp, nq))
    p = tmp_path / "lap.bin"
    IO.write_integrals(p, LAPLACE, T, G, [0.0, 0.0])
    rec = _records(p)
    assert [len(r) // 8 for r in rec[2:]] == [8192, 1808] * (nn + nq)
    T2, G2, _ = IO.read_integrals(p, LAPLACE)
    assert np.array_equal(T, T2) and np.array_equal(G, G2)
    with pytest.raises(AgbError, match="not an integrals file"):
        IO.read_integrals(p, STOKES)  # no parStokes record in front
