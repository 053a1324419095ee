"""Freeze the FP64 GPU resistance tensor of the config-2 workload (GPU run).

The plain FP64 path (FP64 assembly, FP64 LSQR to eps 1e-11) is the truth the
mixed path's relative error is measured against (bench.py reads the JSON).
Run on a GB300 from the repository root:  python tests/golden/make_c2_truth.py
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import andromeda_gb300 as A  # noqa: E402
from andromeda_gb300 import mesh as M  # noqa: E402

level = int(sys.argv[1]) if len(sys.argv) > 1 else 5
p = M.icosphere(level, 1.0, inward=True)
m = M.particle_in_sphere(p, outer_level=2, outer_radius=200.0)
name = (f"Stokes sphere a=1 icosphere L{level} ({len(p['etype'])} tri) in L2 container r=200 "
        f"({len(m['etype']) - len(p['etype'])} tri), 6 RHS, ITRI 5, mu=1")
C = A.Context(0)
C.set_mesh(m)
C.set_problem(A.STOKES, [1, 2], A.dirichlet_known(A.STOKES, 2), itri=5)
t = time.time()
R, nit, info = C.resistance_tensor(A.FP64, 1, 2, eps=1e-11)
out = {"workload": name, "precision": "fp64", "eps": 1e-11, "nit": nit.tolist(), "istop": info["istop"],
       "seconds": time.time() - t, "R": R.tolist()}
fn = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c2_fp64_tensor.json" if level == 5 else f"l{level}_fp64_tensor.json")
with open(fn, "w") as f:
    json.dump(out, f, indent=1)
print(json.dumps(out))
