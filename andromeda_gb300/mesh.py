"""Synthetic boundary meshes for the BEM path (numpy, FP64).

A mesh is a plain dict of arrays in the layout the C ABI takes:

* ``xyz``   float64 (nnodes, 3)   node coordinates
* ``etype`` int32   (nelem,)      2 = 3-node triangle, 3 = 4-node quad
* ``con``   int32   (nelem, 4)    0-based connectivity, 4th entry -1 for triangles
* ``bcid``  int32   (nelem,)      wall id of each element

Element orientation fixes the normal: ``n = (x2-x1) x (x3-x1)`` normalised,
as CalElementNormal computes it (src/lib_mesh.f90:716-769).  The domain-outward
normal convention of the reference is used: for an interior problem the normals
point out of the body; for a particle in a spherical container (the reference's
flow-over-sphere cases, run/stokes/flow-over-sphere) the particle's normals
point into the particle and the container's point outwards.

Geometry generators:

* :func:`icosphere` -- icosahedron refined ``level`` times and projected on the
  sphere (level 3: 642 nodes / 1280 triangles; level 5: 10242 / 20480).
* :func:`superellipsoid` -- signed-power parametric grid of the superquadric
  surface, using the sphere-to-superellipsoid map of mapSphereToSuperE
  (src/lib_particle.f90:2207-2230).
* :func:`merge` -- several walls into one mesh (particle + container).
"""
from __future__ import annotations

import numpy as np


def _tri_mesh(xyz, tris, wall=1):
    tris = np.asarray(tris, dtype=np.int32)
    con = np.full((len(tris), 4), -1, dtype=np.int32)
    con[:, :3] = tris
    return {
        "xyz": np.ascontiguousarray(xyz, dtype=np.float64),
        "etype": np.full(len(tris), 2, dtype=np.int32),
        "con": con,
        "bcid": np.full(len(tris), wall, dtype=np.int32),
    }


def icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0), inward: bool = False, wall: int = 1):
    """Icosahedral sphere: 10*4^L+2 nodes, 20*4^L flat triangles."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = [tuple(x) for x in f]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for (a, b, c) in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    xyz = np.array(verts) * radius + np.asarray(center, dtype=np.float64)
    tris = np.array(faces, dtype=np.int32)
    # orient: outward normals unless inward requested
    p = xyz[tris]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    out = np.einsum("ij,ij->i", n, p.mean(axis=1) - np.asarray(center)) > 0
    flip = out if inward else ~out
    tris[flip] = tris[flip][:, [0, 2, 1]]
    return _tri_mesh(xyz, tris, wall)


def _spow(v, e):
    return np.sign(v) * np.abs(v) ** e


def superellipsoid(a: float, b: float, c: float, e1: float, e2: float, n_rings: int, n_sectors: int,
                   rotation=None, inward: bool = False, wall: int = 1):
    """Superellipsoid surface |x/a|^(2/e2)+|y/b|^(2/e2))^(e2/e1)+|z/c|^(2/e1)=1.

    ``n_rings`` latitude rings (poles excluded) x ``n_sectors`` longitudes plus
    two pole nodes; triangles = 2*n_sectors*n_rings, none degenerate.  The
    (eta, omega) grid is mapped by the signed-power parametrisation of
    mapSphereToSuperE.  ``rotation`` is an optional 3x3 rotation matrix.
    """
    eta = -np.pi / 2 + np.pi * (np.arange(n_rings) + 1) / (n_rings + 1)
    om = -np.pi + 2 * np.pi * np.arange(n_sectors) / n_sectors
    E, O = np.meshgrid(eta, om, indexing="ij")
    x = a * _spow(np.cos(E), e1) * _spow(np.cos(O), e2)
    y = b * _spow(np.cos(E), e1) * _spow(np.sin(O), e2)
    z = c * _spow(np.sin(E), e1)
    ring = np.stack([x, y, z], axis=-1).reshape(-1, 3)
    south = np.array([[0.0, 0.0, -c]])
    north = np.array([[0.0, 0.0, c]])
    xyz = np.concatenate([ring, south, north])
    iS, iN = len(ring), len(ring) + 1

    def nid(r, s):
        return r * n_sectors + (s % n_sectors)

    tris = []
    for s in range(n_sectors):
        tris.append((iS, nid(0, s + 1), nid(0, s)))
    for r in range(n_rings - 1):
        for s in range(n_sectors):
            a0, a1, b0, b1 = nid(r, s), nid(r, s + 1), nid(r + 1, s), nid(r + 1, s + 1)
            tris.append((a0, a1, b1))
            tris.append((a0, b1, b0))
    for s in range(n_sectors):
        tris.append((iN, nid(n_rings - 1, s), nid(n_rings - 1, s + 1)))
    tris = np.array(tris, dtype=np.int32)
    if rotation is not None:
        xyz = xyz @ np.asarray(rotation, dtype=np.float64).T
    p = xyz[tris]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    out = np.einsum("ij,ij->i", n, p.mean(axis=1)) > 0
    flip = out if inward else ~out
    tris[flip] = tris[flip][:, [0, 2, 1]]
    return _tri_mesh(xyz, tris, wall)


def merge(*meshes):
    """Concatenate meshes (node ids shifted); walls keep their bcid."""
    xyz, et, con, bc = [], [], [], []
    off = 0
    for m in meshes:
        xyz.append(m["xyz"])
        et.append(m["etype"])
        c = m["con"].copy()
        c[c >= 0] += off
        con.append(c)
        bc.append(m["bcid"])
        off += len(m["xyz"])
    return {"xyz": np.concatenate(xyz), "etype": np.concatenate(et), "con": np.concatenate(con),
            "bcid": np.concatenate(bc)}


def particle_in_sphere(particle, outer_level: int = 2, outer_radius: float = 200.0,
                       particle_wall: int = 1, outer_wall: int = 2):
    """Particle (normals into it) inside a container sphere (normals outward).

    This is the bounded geometry every particle case of the reference uses
    (run/mesh/sphere-in-sphere.geo: particle wall 'particle', container wall
    'outside').
    """
    p = dict(particle)
    p["bcid"] = np.full(len(p["bcid"]), particle_wall, dtype=np.int32)
    outer = icosphere(outer_level, outer_radius, inward=False, wall=outer_wall)
    return merge(p, outer)


def quad_box(nx: int, ny: int, nz: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), inward: bool = False, wall: int = 1,
             face_walls: bool = False, triangles: bool = False):
    """Axis-aligned box of 4-node quads (outward normals unless ``inward``).

    ``face_walls``: wall ids 1..6 for the faces x-, x+, y-, y+, z-, z+
    (otherwise every element gets ``wall``).  ``triangles``: split every quad
    into two 3-node triangles.
    """
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    nodes = {}
    xyz = []

    def node(p):
        key = tuple(np.round(p, 12))
        if key not in nodes:
            nodes[key] = len(xyz)
            xyz.append(p)
        return nodes[key]

    quads = []
    fw = []
    n = (nx, ny, nz)
    for ax in range(3):
        u, v = [a for a in range(3) if a != ax]
        for side in (0, 1):
            for i in range(n[u]):
                for j in range(n[v]):
                    corners = []
                    for (di, dj) in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        p = np.empty(3)
                        p[ax] = hi[ax] if side else lo[ax]
                        p[u] = lo[u] + (hi[u] - lo[u]) * (i + di) / n[u]
                        p[v] = lo[v] + (hi[v] - lo[v]) * (j + dj) / n[v]
                        corners.append(node(p))
                    quads.append(corners)
                    fw.append(1 + 2 * ax + side)
    xyz = np.array(xyz)
    quads = np.array(quads, dtype=np.int32)
    p = xyz[quads]
    nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    ctr = (lo + hi) / 2
    out = np.einsum("ij,ij->i", nrm, p.mean(axis=1) - ctr) > 0
    flip = out if inward else ~out
    quads[flip] = quads[flip][:, [0, 3, 2, 1]]
    bc = np.array(fw, np.int32) if face_walls else np.full(len(quads), wall, np.int32)
    if triangles:
        tris = np.concatenate([quads[:, [0, 1, 2]], quads[:, [0, 2, 3]]])
        m = _tri_mesh(xyz, tris)
        m["bcid"] = np.concatenate([bc, bc])
        return m
    return {"xyz": xyz, "etype": np.full(len(quads), 3, np.int32), "con": quads, "bcid": bc}


def superellipsoid_tri(a, b, c, e1, e2, n_target, rotation=None, inward=False, wall=1):
    """Superellipsoid with about ``n_target`` triangles: n_sectors = round(sqrt(n))
    longitudes, n_rings = round(n / (2 n_sectors)) latitude rings."""
    ns = max(4, int(round(np.sqrt(n_target))))
    nr = max(2, int(round(n_target / (2.0 * ns))))
    return superellipsoid(a, b, c, e1, e2, nr, ns, rotation=rotation, inward=inward, wall=wall)


def batch_bodies(n_bodies=512, seed=20260101, n_min=500, n_max=8000, outer_level=2, outer_radius=200.0):
    """The many-body workload: superellipsoids a = 1, b, c ~ U(0.2, 1), e1, e2 ~
    U(0.3, 1.8), uniform random orientation, element counts log-uniform in
    [n_min, n_max], each inside its own container sphere (normals into the
    particle).  Returns (meshes, params) with params rows (b, c, e1, e2, n_elem)."""
    rng = np.random.default_rng(seed)
    meshes, params = [], []
    for _ in range(n_bodies):
        b, c = rng.uniform(0.2, 1.0, 2)
        e1, e2 = rng.uniform(0.3, 1.8, 2)
        rot = random_rotation(rng)
        n = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        body = superellipsoid_tri(1.0, b, c, e1, e2, n, rotation=rot, inward=True)
        meshes.append(particle_in_sphere(body, outer_level=outer_level, outer_radius=outer_radius))
        params.append((b, c, e1, e2, len(body["etype"])))
    return meshes, np.array(params)


def random_rotation(rng: np.random.Generator):
    """Uniform random rotation matrix from a unit quaternion."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def edge_corner_node_walls(mesh, walls, rules=()):
    """Walls of the nodes of a single subdomain after the BiC file's EDGE and
    CORNER directives (HandleCornersEdges, src/lib_sdBem.f90:112-310).

    The start is the reference's own assignment (SetUpSubdomains,
    src/lib_sdBem.f90:388-394): every node takes the wall of the last element
    touching it, elements taken wall by wall in the order of `walls`.  Then
    each rule, in order: ("EDGE", w1, w2, target) puts on wall `target` every
    node shared by an element of wall w1 and an element of wall w2;
    ("CORNER", w1, w2, w3, target) every node shared by elements of the three
    walls.  Returns the wall id of every mesh node (-1 where the node is not on
    a wall of the subdomain): the argument of ``Context.set_node_walls`` (the
    reference's subdomain%BCidList)."""
    con = np.asarray(mesh["con"])
    bcid = np.asarray(mesh["bcid"])
    etype = np.asarray(mesh["etype"])
    nn = len(mesh["xyz"])
    nno = np.where(etype == 2, 3, 4)

    def touched(w):
        on = np.zeros(nn, bool)
        if w in walls:
            for e in np.where(bcid == w)[0]:
                on[con[e, :nno[e]]] = True
        return on

    node_wall = np.full(nn, -1, np.int32)
    for w in walls:
        for e in np.where(bcid == w)[0]:
            node_wall[con[e, :nno[e]]] = w
    for rule in rules:
        kind = str(rule[0]).upper()
        if kind == "EDGE" and len(rule) == 4:
            shared = touched(rule[1]) & touched(rule[2])
        elif kind == "CORNER" and len(rule) == 5:
            shared = touched(rule[1]) & touched(rule[2]) & touched(rule[3])
        else:
            raise ValueError(f"not an EDGE or CORNER rule: {rule!r}")
        node_wall[shared & (node_wall >= 0)] = int(rule[-1])
    return node_wall
