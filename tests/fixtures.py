"""The reference's own test meshes (converted by tests/golden/make_fixture_meshes.py)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference_mesh(name):
    """Mesh dict (xyz, etype, con, bcid) of tests/golden/<name>.npz; bcid = the gmsh physical id."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    tris = d["tris"]
    quads = d["quads"] if "quads" in d.files else np.zeros((0, 4), np.int32)
    con = np.full((len(tris) + len(quads), 4), -1, np.int32)
    con[:len(tris), :3] = tris
    con[len(tris):] = quads
    etype = np.concatenate([np.full(len(tris), 2, np.int32), np.full(len(quads), 3, np.int32)])
    phys = np.concatenate([d["phys"], d["qphys"] if "qphys" in d.files else np.zeros(0, np.int32)])
    return {"xyz": np.ascontiguousarray(d["xyz"], dtype=np.float64), "etype": etype, "con": con,
            "bcid": np.ascontiguousarray(phys, dtype=np.int32)}
