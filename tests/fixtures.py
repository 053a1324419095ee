"""The reference's own test meshes (converted by tests/golden/make_fixture_meshes.py)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference_mesh(name):
    """Mesh dict (xyz, etype, con, bcid) of tests/golden/<name>.npz; bcid = the gmsh physical id."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    tris = d["tris"]
    con = np.full((len(tris), 4), -1, np.int32)
    con[:, :3] = tris
    return {"xyz": np.ascontiguousarray(d["xyz"], dtype=np.float64), "etype": np.full(len(tris), 2, np.int32),
            "con": con, "bcid": np.ascontiguousarray(d["phys"], dtype=np.int32)}
