"""Convert the reference's own test meshes into compact fixtures (run once, here).

The reference ships gmsh meshes with its run cases; four of them are the inputs of
the cases on this path:
  * run/mesh/sphere-01.msh (gmsh 2.2): the Laplace case run/laplace/sphere
    (wall "krogla", sphere of radius 0.5, 420 nodes, 836 triangles);
  * run/mesh/sphere-in-sphere-1024-1843-3678-tri.msh (gmsh 4.1): the Stokes case
    run/stokes/flow-over-sphere (walls "particle" and "outside");
  * run/mesh/ellipsoid211-in-sphere-1024-1041-2117.msh (gmsh 4.1): the Stokes case
    run/stokes/flow-over-ellipsoid (a 2:1:1 spheroid of the volume of a sphere of
    radius 0.5 in the same container);
  * run/mesh/kocka-000-111-314-624_tri.msh (gmsh 4.1): the unit cube of the Stokes
    cases run/stokes/Couette and Poiseuille (walls top, bottom, back, front, left,
    right);
  * run/mesh/surf_tri-kocka.msh (gmsh 2.2): the unit cube of the Laplace case
    run/laplace/cube-triangles (walls spredaj, zadaj, zgoraj, spodaj, levo, desno;
    50 nodes, 96 triangles), whose BiC file places its edge and corner nodes with
    EDGE / CORNER directives;
  * run/mesh/kocka-000-111-152-150_hex.msh (gmsh 4.1): the unit cube of quadrilaterals
    of the Laplace case run/laplace/cube-quadrilaterals-simple (walls bottom, front,
    right, back, left, top; 152 nodes, 150 quadrilaterals), with EDGE / CORNER
    directives too.
The node coordinates, the triangles and quadrilaterals (node order as in the file: the
reference takes the element normal from nodes 1-3) and the physical wall ids are written
to tests/golden/<name>.npz ("quads" only where the mesh has quadrilaterals).  Run from the repository root:
    python tests/golden/make_fixture_meshes.py <reference checkout>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _sections(path):
    out, name, body = {}, None, []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if line.startswith("$End"):
                out[name] = body
                name, body = None, []
            elif line.startswith("$"):
                name, body = line[1:], []
            elif name is not None:
                body.append(line)
    return out


def read_msh(path):
    """Triangles of a gmsh 2.2 or 4.1 ASCII mesh: (xyz, tris (0-based), physical id per triangle)."""
    xyz, tris, phys, _, _ = read_msh_quads(path)
    return xyz, tris, phys


def read_msh_quads(path):
    """Triangles and quadrilaterals of a gmsh 2.2 or 4.1 ASCII mesh: (xyz, tris,
    physical id per triangle, quads, physical id per quadrilateral)."""
    s = _sections(path)
    version = s["MeshFormat"][0].split()[0]
    if version.startswith("2"):
        nodes = s["Nodes"]
        n = int(nodes[0])
        ids, xyz = [], []
        for line in nodes[1:1 + n]:
            p = line.split()
            ids.append(int(p[0]))
            xyz.append([float(v) for v in p[1:4]])
        index = {t: i for i, t in enumerate(ids)}
        tris, phys, quads, qphys = [], [], [], []
        els = s["Elements"]
        for line in els[1:1 + int(els[0])]:
            p = [int(v) for v in line.split()]
            ntags = p[2]
            if p[1] == 2:
                tris.append([index[t] for t in p[3 + ntags:6 + ntags]])
                phys.append(p[3])
            elif p[1] == 3:
                quads.append([index[t] for t in p[3 + ntags:7 + ntags]])
                qphys.append(p[3])
        return (np.array(xyz), np.array(tris, np.int32).reshape(-1, 3), np.array(phys, np.int32),
                np.array(quads, np.int32).reshape(-1, 4), np.array(qphys, np.int32))
    # gmsh 4.1: physical group of every surface entity from $Entities
    ent = s["Entities"]
    npts, ncur, nsur, _ = (int(v) for v in ent[0].split())
    surf_phys = {}
    for line in ent[1 + npts + ncur:1 + npts + ncur + nsur]:
        p = line.split()
        tag, nph = int(p[0]), int(p[7])
        surf_phys[tag] = abs(int(p[8])) if nph > 0 else 0  # a negative tag: the group with reversed orientation
    nodes = s["Nodes"]
    nblocks = int(nodes[0].split()[0])
    i = 1
    ids, xyz = [], []
    for _ in range(nblocks):
        nb = int(nodes[i].split()[3])
        tags = [int(v) for v in nodes[i + 1:i + 1 + nb]]
        coords = [[float(v) for v in line.split()[:3]] for line in nodes[i + 1 + nb:i + 1 + 2 * nb]]
        ids += tags
        xyz += coords
        i += 1 + 2 * nb
    index = {t: k for k, t in enumerate(ids)}
    els = s["Elements"]
    nblocks = int(els[0].split()[0])
    i = 1
    tris, phys, quads, qphys = [], [], [], []
    for _ in range(nblocks):
        dim, etag, etype, nb = (int(v) for v in els[i].split())
        for line in els[i + 1:i + 1 + nb]:
            if etype == 2 and dim == 2:
                p = [int(v) for v in line.split()]
                tris.append([index[t] for t in p[1:4]])
                phys.append(surf_phys[etag])
            elif etype == 3 and dim == 2:
                p = [int(v) for v in line.split()]
                quads.append([index[t] for t in p[1:5]])
                qphys.append(surf_phys[etag])
        i += 1 + nb
    return (np.array(xyz), np.array(tris, np.int32).reshape(-1, 3), np.array(phys, np.int32),
            np.array(quads, np.int32).reshape(-1, 4), np.array(qphys, np.int32))


def main(ref):
    cases = {"sphere_01": "run/mesh/sphere-01.msh",
             "sphere_in_sphere_3678": "run/mesh/sphere-in-sphere-1024-1843-3678-tri.msh",
             "ellipsoid211_in_sphere_2117": "run/mesh/ellipsoid211-in-sphere-1024-1041-2117.msh",
             "cube_624": "run/mesh/kocka-000-111-314-624_tri.msh",
             "surf_tri_kocka": "run/mesh/surf_tri-kocka.msh",
             "quad_kocka_150": "run/mesh/kocka-000-111-152-150_hex.msh"}
    for name, rel in cases.items():
        xyz, tris, phys, quads, qphys = read_msh_quads(os.path.join(ref, rel))
        extra = {"quads": quads, "qphys": qphys} if len(quads) else {}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), xyz=xyz, tris=tris, phys=phys,
                            source=np.array(rel), **extra)
        print(name, xyz.shape, tris.shape, quads.shape, np.unique(np.concatenate([phys, qphys]),
                                                                 return_counts=True))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixture_meshes.py <reference checkout>")
    main(sys.argv[1])
