"""Cases on the reference's own meshes (run/mesh/sphere-01.msh of run/laplace/sphere,
run/mesh/sphere-in-sphere-1024-1843-3678-tri.msh of run/stokes/flow-over-sphere,
run/mesh/ellipsoid211-in-sphere-1024-1041-2117.msh of run/stokes/flow-over-ellipsoid,
run/mesh/kocka-000-111-314-624_tri.msh of run/stokes/Couette and Poiseuille),
converted once into tests/golden/*.npz with the node order of the files (the element
normal comes from nodes 1-3, as in the reference).

CPU (oracle): the Laplace case as the reference runs it (ITRI 5, u = 1 on the sphere:
the flux vanishes) and u = x + 2y + 3z, whose flux n.(1,2,3) is exact on the
polyhedral surface, so only quadrature and solver errors remain.
GPU: the same cases through the C ABI against the oracle (1e-10), and the
flow-over-sphere mesh through the resistance workflow: the mixed tensor within 1e-5
of the FP64 one (this container is 1024 particle radii across: the FP32 matrix's
rounding shows at a few 1e-6), symmetric, and the drag and torque within the
discretisation error of the analytic concentric-sphere values (particle a = 0.5,
container b = 512); the flow-over-ellipsoid mesh: the drag along and across the
spheroid's axis against the reference's own analytic resistances
(CalResTensorPrime, lib_particle.f90:1906-1927, with the semi-minor axis of
calForceOnEllipsoid, lib_particle.f90:1979-1996) within 1.5 % (discretisation and
the container, 645 semi-minor axes away); the Couette case on the cube (velocity on
all six walls): the piecewise-constant traction of u = (z, 0, 0), oracle and GPU;
the Poiseuille case (mixed boundary conditions) on the oracle; the Laplace case
run/laplace/cube-triangles on run/mesh/surf_tri-kocka.msh with its BiC file's EDGE /
CORNER directives (the walls of the nodes on the cube's edges and corners): the
package's restatement of the directives against the oracle's, the oracle's fields
against the exact linear fields, and the GPU (agb_set_node_walls) against the oracle;
the same directives on the quadrilateral cube of run/laplace/cube-quadrilaterals-simple
(run/mesh/kocka-000-111-152-150_hex.msh) on the oracle.
"""
import numpy as np
import pytest

from fixtures import reference_mesh


def _laplace_oracle(orc, m, u):
    P = orc.Problem(1, m, walls=[1], known=[[1]], itri=5)
    errs = P.form_integrals()
    n, _, _ = P.geometry()
    _, q, nit, ierr = P.laplace_solve(u, np.zeros(P.nelem), maxit=0, eps=1e-13)
    P.close()
    return q, n, errs, ierr


def test_fixture_meshes_shapes():
    s = reference_mesh("sphere_01")
    assert s["xyz"].shape == (420, 3) and len(s["etype"]) == 836 and set(s["bcid"]) == {1}
    assert np.allclose(np.linalg.norm(s["xyz"], axis=1), 0.5)
    f = reference_mesh("sphere_in_sphere_3678")
    assert f["xyz"].shape == (1843, 3) and len(f["etype"]) == 3678
    assert (f["bcid"] == 1).sum() == 3202 and (f["bcid"] == 2).sum() == 476


def test_laplace_sphere01_reference_case(orc):
    """run/laplace/sphere: u = 1 on the whole sphere -> q = 0."""
    m = reference_mesh("sphere_01")
    q, n, errs, ierr = _laplace_oracle(orc, m, np.ones(len(m["xyz"])))
    assert ierr == 0 and errs[0] < 1e-12
    assert np.max(np.abs(q)) < 1e-9


def test_laplace_sphere01_linear_field(orc):
    m = reference_mesh("sphere_01")
    u = m["xyz"] @ np.array([1.0, 2.0, 3.0])
    q, n, errs, ierr = _laplace_oracle(orc, m, u)
    qex = -(n @ np.array([1.0, 2.0, 3.0]))
    assert ierr == 0
    assert np.linalg.norm(q - qex) / np.linalg.norm(qex) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("field", ["one", "linear"])
def test_gpu_laplace_sphere01_vs_oracle(agb, orc, field):
    m = reference_mesh("sphere_01")
    u = np.ones(len(m["xyz"])) if field == "one" else m["xyz"] @ np.array([1.0, 2.0, 3.0])
    q_ref, _, _, _ = _laplace_oracle(orc, m, u)
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.LAPLACE, [1], agb.dirichlet_known(agb.LAPLACE, 1), itri=5)
    C.assemble(agb.FP64)
    x, nit, istop = C.solve(u[None], eps=1e-13)
    C.close()
    scale = max(np.max(np.abs(q_ref)), 1.0)
    assert istop[0] <= 3
    assert np.max(np.abs(x[0] - q_ref)) < 1e-10 * scale


@pytest.mark.gpu
def test_gpu_flow_over_sphere_reference_mesh(agb):
    m = reference_mesh("sphere_in_sphere_3678")
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, [1, 2], agb.dirichlet_known(agb.STOKES, 2), itri=5)
    R64, _, info64 = C.resistance_tensor(agb.FP64, 1, 2, eps=1e-11)
    R32, _, info32 = C.resistance_tensor(agb.MIXED, 1, 2, eps=1e-8)
    C.close()
    # 1/2: converged; 4: the reference's condition limit (conlim 1e8), a legitimate stop of lsqr_solve
    assert np.all(np.isin(info64["istop"], (1, 2, 4))) and np.all(np.isin(info32["istop"], (1, 2, 4)))
    scale = np.max(np.abs(R64))
    # the container is 1024 particle radii across (the benchmark's 200): the FP32
    # matrix's rounding reaches the rotation couplings at a few 1e-6 here
    print("mixed vs FP64", np.max(np.abs(R32 - R64)) / scale, "asymmetry", np.max(np.abs(R64 - R64.T)) / scale,
          "drag", np.diag(R64)[:3] / (6 * np.pi * 0.5), "torque", np.diag(R64)[3:] / (np.pi))
    assert np.max(np.abs(R32 - R64)) < 1e-5 * scale
    assert np.max(np.abs(R64 - R64.T)) < 1e-4 * scale
    lam = 0.5 / 512.0
    drag = 6 * np.pi * 0.5 * (1 - lam ** 5) / (1 - 9 * lam / 4 + 5 * lam ** 3 / 2 - 9 * lam ** 5 / 4 + lam ** 6)
    torque = 8 * np.pi * 0.5 ** 3 / (1 - lam ** 3)
    assert np.allclose(np.diag(R64)[:3] / drag, 1.0, atol=5e-3)
    assert np.allclose(np.diag(R64)[3:] / torque, 1.0, atol=1e-2)


def _spheroid_resistance(lam):
    """Translational resistances of a prolate spheroid of aspect ratio lam, in units of
    pi mu b U (b = semi-minor axis): (along the axis, across it) -- the closed forms
    the reference evaluates in CalResTensorPrime (Oberbeck's solution)."""
    l2 = lam * lam - 1.0
    s = np.sqrt(l2)
    lg = np.log(lam + s)
    along = 8.0 * l2 ** 1.5 / ((2.0 * l2 + 1.0) * lg - lam * s)
    across = 16.0 * l2 ** 1.5 / ((2.0 * l2 - 1.0) * lg + lam * s)
    return along, across


def test_spheroid_resistance_limits():
    along, across = _spheroid_resistance(1.0 + 1e-6)
    assert abs(along - 6.0) < 1e-4 and abs(across - 6.0) < 1e-4  # the sphere: 6 pi mu a U
    along, across = _spheroid_resistance(2.0)
    assert 6.0 < along < across


@pytest.mark.gpu
def test_gpu_flow_over_ellipsoid_reference_mesh(agb):
    m = reference_mesh("ellipsoid211_in_sphere_2117")
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, [1, 2], agb.dirichlet_known(agb.STOKES, 2), itri=5)
    R64, _, info64 = C.resistance_tensor(agb.FP64, 1, 2, eps=1e-11)
    R32, _, _ = C.resistance_tensor(agb.MIXED, 1, 2, eps=1e-8)
    C.close()
    scale = np.max(np.abs(R64))
    assert np.max(np.abs(R32 - R64)) < 1e-5 * scale
    b = (3.0 * (np.pi / 6.0) / (4.0 * np.pi * 2.0)) ** (1.0 / 3.0)  # volume of the sphere of radius 0.5
    along, across = _spheroid_resistance(2.0)
    ratio = np.diag(R64)[:3] / (np.array([along, across, across]) * b * np.pi)  # axis along x
    print("spheroid drag / analytic", ratio)
    assert np.allclose(ratio, 1.0, atol=1.5e-2)


def _couette_checks(q, m):
    """Couette flow u = (z, 0, 0) in the reference's unit cube (mu = 1): traction
    q = -(sigma . n) with n the mesh normal (out of the fluid): q_x = -1 on top, +1 on
    bottom, q_z = +1 on left, -1 on right, the other tangential components 0, and the
    normal component the same constant (the pressure level, free in an all-Dirichlet
    problem) on every face.  Returns the largest deviation."""
    x = m["xyz"]
    t = m["con"][:, :3]
    nrm = np.cross(x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    want = {1: (0, -1.0), 2: (0, 1.0), 5: (2, 1.0), 6: (2, -1.0), 3: None, 4: None}  # wall: (component, value)
    qn = np.sum(q.T * nrm, axis=1)
    dev = np.max(np.abs(qn - np.mean(qn)))
    for wall, w in want.items():
        sel = m["bcid"] == wall
        normal = int(np.argmax(np.abs(nrm[sel].mean(0))))
        for comp in range(3):
            if comp == normal:
                continue
            target = w[1] if (w is not None and comp == w[0]) else 0.0
            dev = max(dev, np.max(np.abs(q[comp, sel] - target)))
    return dev


def _couette_fields(m):
    U = np.zeros((1, 3, len(m["xyz"])))
    U[0, 0] = m["xyz"][:, 2]
    return U


def test_couette_reference_cube(orc):
    """run/stokes/Couette on run/mesh/kocka-000-111-314-624_tri.msh (velocity given on
    all six walls)."""
    m = reference_mesh("cube_624")
    P = orc.Problem(2, m, walls=[1, 2, 3, 4, 5, 6], known=np.ones((3, 6)), itri=5)
    P.form_integrals()
    q, _, nits, ierr = P.stokes_solve_sequence(_couette_fields(m), maxit=0, eps=1e-13, fwall=1)
    P.close()
    assert _couette_checks(q[0], m) < 2e-3


@pytest.mark.gpu
def test_gpu_couette_reference_cube(agb, orc):
    m = reference_mesh("cube_624")
    U = _couette_fields(m)
    P = orc.Problem(2, m, walls=[1, 2, 3, 4, 5, 6], known=np.ones((3, 6)), itri=5)
    P.form_integrals()
    q_ref, _, _, _ = P.stokes_solve_sequence(U, maxit=0, eps=1e-13, fwall=1)
    P.close()
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, [1, 2, 3, 4, 5, 6], agb.dirichlet_known(agb.STOKES, 6), itri=5)
    C.assemble(agb.FP64)
    x, nit, istop = C.solve(U, eps=1e-13)
    C.close()
    # the solution comes in the subdomain's element order: wall by wall in the order
    # of the wall list (SetUpSubdomains), mesh order within a wall
    order = np.concatenate([np.where(m["bcid"] == w)[0] for w in (1, 2, 3, 4, 5, 6)])
    q = np.zeros((3, len(order)))
    q[:, order] = x[0].reshape(3, -1)
    assert _couette_checks(q, m) < 2e-3
    # the pressure level (a constant normal traction) is the null direction of the
    # all-Dirichlet system, where both LSQR runs stop on the condition limit at
    # different levels: compare the solutions with it removed
    x_ = m["xyz"]
    t = m["con"][:, :3]
    nrm = np.cross(x_[t[:, 1]] - x_[t[:, 0]], x_[t[:, 2]] - x_[t[:, 0]])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]

    def without_pressure(qq):
        return qq - np.mean(np.sum(qq.T * nrm, axis=1)) * nrm.T

    assert np.max(np.abs(without_pressure(q) - without_pressure(q_ref[0]))) < 1e-5


@pytest.mark.gpu
def test_gpu_couette_flux_bc_reference_cube(agb):
    """run/stokes/Couette with stokesCouette-X-fluxBC.bic: the x traction given on the
    four side walls (0 on front and back, -3 on left, +3 on right: pressure 3), the
    velocity elsewhere.  Mixed boundary conditions through the general path: the side
    walls' x velocity comes out as z, the tractions as in the Dirichlet case with the
    normal component equal to the pressure."""
    m = reference_mesh("cube_624")
    walls = [1, 2, 3, 4, 5, 6]  # top, bottom, back, front, left, right
    known = np.ones((3, 6), np.int32)
    known[0, 2:] = 2  # x traction known on back, front, left, right
    nn, ne = len(m["xyz"]), len(m["etype"])
    U = _couette_fields(m)
    Q = np.zeros((1, 3, ne))
    Q[0, 0, m["bcid"] == 5] = -3.0
    Q[0, 0, m["bcid"] == 6] = 3.0
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.STOKES, walls, known, itri=5)
    C.assemble(agb.FP64)
    uo, qo, nit, istop = C.solve_fields(U, Q, eps=1e-13)
    C.close()
    assert istop[0] <= 4
    assert np.max(np.abs(uo[0, 0] - m["xyz"][:, 2])) < 2e-3 and np.max(np.abs(uo[0, 1:])) < 2e-3
    x = m["xyz"]
    t = m["con"][:, :3]
    nrm = np.cross(x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    q = qo[0]
    assert np.max(np.abs(np.sum(q.T * nrm, axis=1) - 3.0)) < 5e-3  # normal traction = pressure
    tang = q - np.sum(q.T * nrm, axis=1) * nrm.T
    want = np.zeros_like(q)
    want[0, m["bcid"] == 1] = -1.0
    want[0, m["bcid"] == 2] = 1.0
    want[2, m["bcid"] == 5] = 1.0
    want[2, m["bcid"] == 6] = -1.0
    assert np.max(np.abs(tang - want)) < 5e-3


def test_poiseuille_reference_cube(orc):
    """run/stokes/Poiseuille (stokesPoiseuille-X.bic) on the reference's cube, on the
    oracle: viscosity 1.5, inlet (left) u_x = (8/3) z (1 - z), x traction given on the
    outlet (right; taken as 0 here, which only shifts the free pressure level) and on
    front and back (0), no slip on top and bottom.  Plane Poiseuille flow: pressure
    p = 8 (1 - x), wall shear mu du/dz = -+4.  With the traction convention
    q = -(sigma . n): q_x = 4 on both plates, q_z = +-p on top/bottom, q_y = +-p on
    back/front, q_x = -8 on the inlet.  The linear velocity elements carry the
    quadratic profile only approximately (624 triangles): wall means within 5 %."""
    m = reference_mesh("cube_624")
    known = np.ones((3, 6), np.int32)
    known[0, [2, 3, 5]] = 2  # x traction known on back, front, right
    U = np.zeros((1, 3, len(m["xyz"])))
    z = m["xyz"][:, 2]
    U[0, 0] = (8.0 / 3.0) * (z - z * z)
    P = orc.Problem(2, m, walls=[1, 2, 3, 4, 5, 6], known=known, diff=1.5, itri=5)
    P.form_integrals()
    q, _, nits, ierr = P.stokes_solve_sequence(U, maxit=0, eps=1e-13, fwall=1)
    P.close()
    assert ierr == 0
    q = q[0]
    cx = m["xyz"][m["con"][:, :3]].mean(axis=1)[:, 0]
    top, bottom, back, front, left = (m["bcid"] == w for w in (1, 2, 3, 4, 5))
    for sel in (top, bottom):
        assert abs(np.mean(q[0, sel]) - 4.0) < 0.2
    slope, icpt = np.polyfit(cx[top], q[2, top], 1)
    assert abs(slope + 8.0) < 0.4 and abs(icpt - 8.0) < 0.4
    slope, icpt = np.polyfit(cx[bottom], q[2, bottom], 1)
    assert abs(slope - 8.0) < 0.4 and abs(icpt + 8.0) < 0.4
    p_mean = 8.0 * (1.0 - np.mean(cx[back]))
    assert abs(np.mean(q[1, back]) - p_mean) < 0.05 * p_mean
    assert abs(np.mean(q[1, front]) + p_mean) < 0.05 * p_mean
    assert abs(np.mean(q[0, left]) + 8.0) < 0.4


# run/laplace/cube-triangles: the unit cube of run/mesh/surf_tri-kocka.msh (walls 1
# spredaj z=1, 2 zadaj z=0, 3 zgoraj y=1, 4 spodaj y=0, 5 levo x=0, 6 desno x=1), the
# subdomain's walls in the order of its BiC file, and the file's EDGE / CORNER
# directives (tri-kocka-prevod.bic) as wall ids
CUBE_WALLS = [1, 2, 5, 6, 4, 3]
CUBE_RULES = [("EDGE", 3, 2, 2), ("EDGE", 3, 1, 1), ("EDGE", 3, 6, 6), ("EDGE", 3, 5, 5),
              ("EDGE", 4, 2, 2), ("EDGE", 4, 1, 1), ("EDGE", 4, 6, 6), ("EDGE", 4, 5, 5),
              ("EDGE", 1, 5, 5), ("EDGE", 1, 6, 6), ("EDGE", 2, 5, 5), ("EDGE", 2, 6, 6),
              ("CORNER", 3, 1, 5, 5), ("CORNER", 3, 1, 6, 6), ("CORNER", 3, 2, 5, 5), ("CORNER", 3, 2, 5, 5),
              ("CORNER", 4, 1, 5, 5), ("CORNER", 4, 1, 6, 6), ("CORNER", 4, 2, 5, 5), ("CORNER", 4, 2, 5, 5)]
# the two equations of the case: temperature u = -0.5 on levo, 0.5 on desno, no flux
# elsewhere (u = x - 0.5); concentration u = 1 on spredaj, 3 on zadaj (u = 3 - 2z)
CUBE_CASES = {"temperatura": ({5: -0.5, 6: 0.5}, lambda p: p[:, 0] - 0.5),
              "koncentracija": ({1: 1.0, 2: 3.0}, lambda p: 3.0 - 2.0 * p[:, 2])}


# run/laplace/cube-quadrilaterals-simple: run/mesh/kocka-000-111-152-150_hex.msh (walls 1
# bottom z=0, 2 front y=0, 3 right x=1, 4 back y=1, 5 left x=0, 6 top z=1), its
# subdomain's wall order and its EDGE / CORNER directives (kocka-1sd-prevod.bic); one
# equation: u = -0.5 on right, 0.5 on left, no flux elsewhere (u = 0.5 - x)
QUAD_WALLS = [2, 4, 3, 5, 1, 6]
QUAD_RULES = [("EDGE", 6, 4, 4), ("EDGE", 6, 2, 2), ("EDGE", 6, 5, 5), ("EDGE", 6, 3, 3),
              ("EDGE", 1, 4, 4), ("EDGE", 1, 2, 2), ("EDGE", 1, 5, 5), ("EDGE", 1, 3, 3),
              ("EDGE", 2, 3, 3), ("EDGE", 2, 5, 5), ("EDGE", 4, 3, 3), ("EDGE", 4, 5, 5),
              ("CORNER", 6, 2, 3, 3), ("CORNER", 6, 2, 5, 5), ("CORNER", 6, 4, 3, 3), ("CORNER", 6, 4, 3, 3),
              ("CORNER", 1, 2, 3, 3), ("CORNER", 1, 2, 5, 5), ("CORNER", 1, 4, 3, 3), ("CORNER", 1, 4, 3, 3)]
QUAD_CASE = ({3: -0.5, 5: 0.5}, lambda p: 0.5 - p[:, 0])


def _cube_oracle(orc, m, case, rules=True, walls_order=None, rule_list=None):
    """Oracle solve of one equation of a cube case; returns (u, q, node walls, problem sizes, known u)."""
    dirichlet, exact = CUBE_CASES[case] if isinstance(case, str) else case
    walls_order = CUBE_WALLS if walls_order is None else walls_order
    rule_list = CUBE_RULES if rule_list is None else rule_list
    known = [[1 if w in dirichlet else 2 for w in walls_order]]
    P = orc.Problem(1, m, walls=walls_order, known=known, itri=5, iqud=4)
    if rules:
        for r in rule_list:
            if r[0] == "EDGE":
                P.edge_rule(*r[1:])
            else:
                P.corner_rule(*r[1:])
    P.form_integrals()
    walls = P.node_walls()
    # known values: u on the Dirichlet walls' nodes (by the node's wall), q = 0 elsewhere
    u0 = np.array([dirichlet.get(int(w), 0.0) for w in walls])
    u, q, nit, ierr = P.laplace_solve(u0, np.zeros(P.nelem), maxit=0, eps=1e-13)
    sizes = (P.nx, P.nb)
    P.close()
    assert ierr == 0
    return u, q, walls, sizes, u0


def test_edge_corner_rules_match_the_oracle(orc):
    """The package's restatement of HandleCornersEdges (mesh.edge_corner_node_walls)
    against the oracle's on the reference's cube with its BiC file's directives:
    the same wall for every node; every node on an edge or corner of a Dirichlet
    face (levo, desno) ends on that face."""
    from andromeda_gb300 import mesh as M
    m = reference_mesh("surf_tri_kocka")
    P = orc.Problem(1, m, walls=CUBE_WALLS, known=[[2, 2, 1, 1, 2, 2]], itri=5)
    auto = P.node_walls()
    assert np.array_equal(auto, M.edge_corner_node_walls(m, CUBE_WALLS))  # the automatic rule
    for r in CUBE_RULES:
        (P.edge_rule if r[0] == "EDGE" else P.corner_rule)(*r[1:])
    walls = P.node_walls()
    P.close()
    assert np.array_equal(walls, M.edge_corner_node_walls(m, CUBE_WALLS, CUBE_RULES))
    x = m["xyz"][:, 0]
    assert np.all(walls[np.isclose(x, 0.0)] == 5) and np.all(walls[np.isclose(x, 1.0)] == 6)
    assert np.sum(walls != auto) > 0
    with pytest.raises(ValueError):
        M.edge_corner_node_walls(m, CUBE_WALLS, [("EDGE", 1, 2)])


def test_edge_corner_rules_quadrilaterals(orc):
    """The same on the reference's cube of quadrilaterals (cube-quadrilaterals-simple),
    and its equation on the oracle: the Dirichlet faces' edges and corners on those
    faces, the linear field u = 0.5 - x at every node."""
    from andromeda_gb300 import mesh as M
    m = reference_mesh("quad_kocka_150")
    assert np.all(m["etype"] == 3) and len(m["etype"]) == 150
    P = orc.Problem(1, m, walls=QUAD_WALLS, known=[[2, 2, 1, 1, 2, 2]], itri=5, iqud=4)
    for r in QUAD_RULES:
        (P.edge_rule if r[0] == "EDGE" else P.corner_rule)(*r[1:])
    walls = P.node_walls()
    P.close()
    assert np.array_equal(walls, M.edge_corner_node_walls(m, QUAD_WALLS, QUAD_RULES))
    x = m["xyz"][:, 0]
    assert np.all(walls[np.isclose(x, 1.0)] == 3) and np.all(walls[np.isclose(x, 0.0)] == 5)
    u, q, walls, sizes, u0 = _cube_oracle(orc, m, QUAD_CASE, walls_order=QUAD_WALLS, rule_list=QUAD_RULES)
    ue = QUAD_CASE[1](m["xyz"])
    known = np.isin(walls, [3, 5])
    assert np.max(np.abs(u[known] - ue[known])) < 1e-14
    assert np.max(np.abs(u - ue)) < 1e-10  # 8e-13 (5e-12 with the automatic assignment)


@pytest.mark.parametrize("case", ["temperatura", "koncentracija"])
def test_laplace_cube_edge_corner_case(orc, case):
    """run/laplace/cube-triangles on the oracle with the BiC file's EDGE / CORNER
    directives: the linear field of each equation at every node (the Dirichlet
    ones exactly) and its flux on the elements."""
    m = reference_mesh("surf_tri_kocka")
    u, q, walls, sizes, u0 = _cube_oracle(orc, m, case)
    dirichlet, exact = CUBE_CASES[case]
    ue = exact(m["xyz"])
    known = np.isin(walls, list(dirichlet))
    assert np.max(np.abs(u[known] - ue[known])) < 1e-14
    assert np.max(np.abs(u - ue)) < 1e-6  # 2.7e-8 / 6.7e-7 (3.3e-7 / 7.2e-7 without the directives)
    u_auto, _, _, sizes_auto, _ = _cube_oracle(orc, m, case, rules=False)
    assert sizes != sizes_auto  # the directives change which nodes are unknowns


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["temperatura", "koncentracija"])
def test_gpu_laplace_cube_edge_corner_case(agb, orc, case):
    """The same case through the C ABI, the node walls set by agb_set_node_walls from
    the package's restatement of the directives: the oracle's fields to 1e-10."""
    from andromeda_gb300 import mesh as M
    m = reference_mesh("surf_tri_kocka")
    u_ref, q_ref, walls, sizes, u0 = _cube_oracle(orc, m, case)
    dirichlet, _ = CUBE_CASES[case]
    known = [[1 if w in dirichlet else 2 for w in CUBE_WALLS]]
    C = agb.Context(0)
    C.set_mesh(m)
    C.set_problem(agb.LAPLACE, CUBE_WALLS, known, itri=5)
    C.set_node_walls(M.edge_corner_node_walls(m, CUBE_WALLS, CUBE_RULES))
    C.assemble(agb.FP64)
    uo, qo, nit, istop = C.solve_fields(u0[None, None], np.zeros((1, 1, len(m["etype"]))), eps=1e-13)
    C.close()
    assert istop[0] <= 3
    assert np.max(np.abs(uo[0, 0] - u_ref)) < 1e-10 * np.max(np.abs(u_ref))
    assert np.max(np.abs(qo[0, 0] - q_ref)) < 1e-10 * max(np.max(np.abs(q_ref)), 1.0)
