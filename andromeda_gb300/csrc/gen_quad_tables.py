"""Generate quad_tables.h: the quadrature DATA used by the BEM assembly.

The two tables are published numerical data, not code:

* Wandzura & Xiao (2003), "Symmetric quadrature rules on a triangle",
  Comput. Math. Appl. 45(12):1829-1840 -- orbit data (multiplicity m, a point
  (x, y) on the reference equilateral triangle, weight w) for the five rules
  ITRI = 1..5 (7, 25, 54, 85, 126 points).  The reference stores them in
  src/mod_trikotnik.f90:320-674 (Triangle_IntegrationInit).
* Gauss-Legendre abscissae/weights for N = 2, 4, 6, 8, 16, 32, 40, 48 packed
  in one 156-entry array with 1-based index ranges ng1/ng2, as in
  src/mod_gauss.f90:33-393 (GaussPosWeights).

The header keeps the reference's digits exactly (so quadrature sums agree with
the reference to the last bit of the inputs).  Expansion of the orbits into
barycentric points (WandzuratXiaoBary) is done by the consumers.

Usage:  python gen_quad_tables.py <reference checkout>/src  > quad_tables.h
"""
import re
import sys


def fnum(tok: str) -> str:
    """Fortran literal -> C double literal (keeps all digits)."""
    t = tok.strip().replace("_rk", "").replace("D", "e").replace("d", "e")
    float(t)  # validate
    if "e" not in t and "." not in t:
        t += ".0"
    return t


def parse_wx(path):
    src = open(path).read().splitlines()
    rules = {}
    cur = None
    pat_n = re.compile(r"waxi%n\.EQ\.(\d+)")
    pat_v = re.compile(r"waxi%(m|x|y|w)\((\d+)\)\s*=\s*([-+0-9.eEdD_rk]+)")
    for line in src[300:700]:
        s = line.split("!")[0]
        mn = pat_n.search(s)
        if mn and "IF" in s:
            cur = int(mn.group(1))
            rules[cur] = {}
            continue
        mv = pat_v.search(s)
        if mv and cur is not None:
            key, idx, val = mv.group(1), int(mv.group(2)), mv.group(3)
            rules[cur].setdefault(idx, {})[key] = val
    out = []
    for norb, ent in sorted(rules.items()):
        orbs = []
        for i in range(1, norb + 1):
            e = ent[i]
            orbs.append((int(e["m"]), fnum(e["x"]), fnum(e["y"]), fnum(e["w"])))
        out.append(orbs)
    return out


def parse_gauss(path):
    src = open(path).read()
    gi, ome, ng1, ng2 = {}, {}, {}, {}
    for m in re.finditer(r"gaus%(gi|ome|ng1|ng2)\((\d+)\)\s*=\s*([-+0-9.eEdD_rk]+)", src, re.I):
        k, i, v = m.group(1).lower(), int(m.group(2)), m.group(3)
        {"gi": gi, "ome": ome, "ng1": ng1, "ng2": ng2}[k][i] = v
    assert len(gi) == 156 and len(ome) == 156
    return ([fnum(gi[i]) for i in range(1, 157)], [fnum(ome[i]) for i in range(1, 157)],
            [int(ng1[i]) for i in range(1, 9)], [int(ng2[i]) for i in range(1, 9)])


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python gen_quad_tables.py <reference checkout>/src > quad_tables.h")
    srcdir = sys.argv[1]
    wx = parse_wx(srcdir + "/mod_trikotnik.f90")
    gi, ome, ng1, ng2 = parse_gauss(srcdir + "/mod_gauss.f90")
    assert [len(r) for r in wx] == [3, 7, 12, 19, 26], [len(r) for r in wx]
    p = print
    p("// Generated by gen_quad_tables.py -- quadrature data only (see that script).")
    p("// Wandzura-Xiao (2003) symmetric triangle rules, orbit form, and the")
    p("// Gauss-Legendre table packed as in the reference's GaussPosWeights.")
    p("#pragma once")
    p("namespace agb_tables {")
    p("struct WxOrbit { int m; double x, y, w; };")
    offs, n = [], 0
    for r in wx:
        offs.append(n)
        n += len(r)
    p(f"static const int kWxNumRules = 5;")
    p(f"static const int kWxOrbitOffset[6] = {{{', '.join(map(str, offs + [n]))}}};")
    npts = [sum(o[0] for o in r) for r in wx]
    p(f"static const int kWxPoints[5] = {{{', '.join(map(str, npts))}}};")
    p("static const WxOrbit kWxOrbits[] = {")
    for ri, r in enumerate(wx):
        p(f"  // ITRI {ri + 1}: {len(r)} orbits, {npts[ri]} points")
        for (m, x, y, w) in r:
            p(f"  {{{m}, {x}, {y}, {w}}},")
    p("};")
    p("static const double kGaussGi[156] = {")
    for i in range(0, 156, 4):
        p("  " + ", ".join(gi[i:i + 4]) + ",")
    p("};")
    p("static const double kGaussOme[156] = {")
    for i in range(0, 156, 4):
        p("  " + ", ".join(ome[i:i + 4]) + ",")
    p("};")
    p(f"static const int kGaussNg1[8] = {{{', '.join(map(str, ng1))}}};  // 1-based")
    p(f"static const int kGaussNg2[8] = {{{', '.join(map(str, ng2))}}};  // 1-based, inclusive")
    p("}  // namespace agb_tables")


if __name__ == "__main__":
    main()
