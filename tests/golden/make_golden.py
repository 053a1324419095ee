"""Regenerate oracle_values.json (frozen oracle outputs for regression tests).

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import numpy as np  # noqa: E402
import oracle  # noqa: E402

tri = [[0.1, 0.2, 0.3], [1.3, 0.1, 0.5], [0.4, 1.1, 0.2]]
v = np.array(tri)
out = {
    "triangle": tri,
    "si_tri_lap": [oracle.si_tri_lap(v, k) for k in (1, 2, 3, 4)],
    "si_tri_stk": [oracle.si_tri_stk(v, k).tolist() for k in (1, 2, 3, 4)],
    "triangle_test": [oracle.triangle_test(k).tolist() for k in range(1, 6)],
}
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_values.json"), "w") as f:
    json.dump(out, f, indent=1)
print("written")
