#!/usr/bin/env python3
"""Stokes resistance-tensor solves/s on GB300 (one JSON line on stdout).

Workload (configuration 2 of the benchmark plan): a rigid sphere of radius
a = 1 meshed as an icosahedral sphere of level 5 (20480 flat triangles,
10242 nodes), inside a spherical container of radius 200 (level 2, 320
triangles) -- the bounded geometry every particle case of the reference
uses.  Viscosity 1, ITRI 5 (126-point Wandzura-Xiao rule), all walls with
known velocity, six right-hand sides = the container's unit translations and
rotations.  One solve = assembly of the 62400 x 62400 single-layer system,
its right-hand sides, block LSQR of the six fields to eps, force and torque
on the sphere (the 6x6 resistance tensor).  Inputs: synthetic meshes built
in-process (no dataset); the 10.4 GB packed system matrix is far larger than L2, so
no L2 flush is needed between timed steps.

--impl ours (default): the mixed-precision GPU path through the C ABI.
--impl reference: the reference's algorithm on the host cores (the FP64 C++
restatement in oracle/, since the Fortran reference cannot be compiled on
this image or the GPU machine), timed on a bounded sample and scaled to one solve.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Stokes resistance-tensor solves/s at <=1e-6 rel err: mixed/batched vs FP64 GPU"
GOLDEN_TRUTH = os.path.join(ROOT, "tests", "golden", "c2_fp64_tensor.json")
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "k_avp_k_atup_l4.md")
PROFILE_BATCH = os.path.join(ROOT, "profiles", "batch_sweeps_b16.md")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=5)
    ap.add_argument("--outer-level", type=int, default=2)
    ap.add_argument("--outer-radius", type=float, default=200.0)
    ap.add_argument("--eps", type=float, default=1e-7)
    ap.add_argument("--solver", default=None, choices=["lsqr", "lsqr_block", "bicgstab", "hybrid", "gmres"],
                    help="sphere, batch, large: gmres (the default of sphere and large; the LIS path with -i gmres, "
                         "3x3 self-block right preconditioner, FP64 true-residual restarts), lsqr_block (LSQR with "
                         "the 3x3 self-block right preconditioner, the default of batch), lsqr (lsqr_solve with "
                         "lsqr_precon's column scaling, the reference's), bicgstab "
                         "(BiCGSTAB-Jacobi, the LIS path's default solver) or hybrid (BiCGSTAB, LSQR for the "
                         "systems where it does not converge)")
    ap.add_argument("--restart", type=int, default=40, help="gmres: restart length (40: the LIS default)")
    ap.add_argument("--fp64", default="full", choices=["full", "off"],
                    help="sphere: the plain FP64 GPU comparator solved to convergence at the same eps (full)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="budget of the full-size CPU estimate's sample")
    ap.add_argument("--cpu-level", type=int, default=2,
                    help="icosphere level of the body the CPU solves completely (the full-size body takes hours)")
    ap.add_argument("--cpu-solves", type=int, default=3, help="sphere: complete CPU solves of the small body")
    ap.add_argument("--c2-estimate", type=int, default=1, help="also estimate the full-size CPU solve (labelled)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lis-compare", type=int, default=3,
                    help="sphere: timed solves of each other solver (column-scaled LSQR, block LSQR, BiCGSTAB hybrid)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--workload", default="sphere", choices=["sphere", "batch", "surrogate", "large", "laplace", "mlp"],
                    help="sphere: one level-5 sphere (default); batch: the many-body superellipsoid set")
    ap.add_argument("--bodies", type=int, default=512, help="batch workload: number of bodies")
    ap.add_argument("--fp64-sample", type=int, default=6, help="batch workload: bodies solved on the FP64 path")
    ap.add_argument("--batch-eps", type=float, default=None,
                    help="batch and surrogate: solver tolerance (default 1e-7 for GMRES, 3e-8 for LSQR, which "
                         "keeps every sampled body within 1e-6 of FP64)")
    ap.add_argument("--no-autotune", action="store_true", help="batch workload: default tile shapes")
    ap.add_argument("--train-bodies", type=int, default=20000, help="surrogate: BEM tensors to train on")
    ap.add_argument("--sur-elements", type=int, default=500, help="surrogate: triangles per training body")
    ap.add_argument("--members", type=int, default=4, help="surrogate: networks in the ensemble")
    ap.add_argument("--sur-margin", type=float, default=0.7,
                    help="surrogate: calibrated held-out answers must be within margin x 1e-3")
    ap.add_argument("--queries", type=int, default=1000000, help="surrogate: inference batch")
    ap.add_argument("--audit", type=float, default=0.01, help="surrogate: fraction of queries re-solved by the BEM")
    ap.add_argument("--predict-queries", type=int, default=100000,
                    help="surrogate: queries answered end to end (ensemble, BEM where it refuses)")
    ap.add_argument("--epochs", type=int, default=800, help="surrogate: training epochs")
    ap.add_argument("--mf-iters", type=int, default=6, help="large: LSQR iterations timed (matrix-free sweeps)")
    ap.add_argument("--large-mode", default="resident", choices=["resident", "mf"],
                    help="large: packed FP32 matrix resident in HBM and solved to convergence, or matrix-free sweeps")
    ap.add_argument("--large-maxit", type=int, default=0, help="large/resident: LSQR iteration limit (0: reference default)")
    ap.add_argument("--grid", default="160x320", help="large: superellipsoid rings x sectors")
    ap.add_argument("--large-eps", type=float, default=3e-8,
                    help="large: solver tolerance (LSQR at 1e-7 leaves 2.4e-6 on the 40x80 grid of this shape; "
                         "3e-8 meets 1e-6)")
    ap.add_argument("--large-fp64-eps", type=float, default=1e-10,
                    help="large/resident: also solve the FP64 path to this eps where its matrix fits (0: off)")
    ap.add_argument("--itri", type=int, default=1, help="laplace: triangle rule (1 = 7 points)")
    ap.add_argument("--laplace-eps", type=float, default=1e-12, help="laplace: LSQR eps")
    args = ap.parse_args()
    if args.solver is None:
        args.solver = "gmres"
    if args.batch_eps is None:
        # GMRES stops on the true residual (1e-7 leaves 2-3e-7 on the sampled
        # bodies); LSQR's stopping test needs 3e-8 for every body within 1e-6
        args.batch_eps = 1e-7 if args.solver == "gmres" else 3e-8
    return args


def solver_id(A, name):
    return {"lsqr": A.SOLVER_LSQR, "bicgstab": A.SOLVER_BICGSTAB, "hybrid": A.SOLVER_HYBRID,
            "lsqr_block": A.SOLVER_LSQR_BLOCK, "gmres": A.SOLVER_GMRES}[name]


def solver_text(name, eps):
    return {"lsqr": f"LSQR eps {eps:g}", "lsqr_block": f"LSQR (3x3 self-block preconditioner) eps {eps:g}",
            "bicgstab": f"BiCGSTAB-Jacobi tol {eps:g}",
            "hybrid": f"BiCGSTAB-Jacobi tol {eps:g}, LSQR eps {eps:g} where it does not converge",
            "gmres": f"GMRES (3x3 self-block preconditioner) tol {eps:g}"}[name]


def mesh_part(name):
    """The mesh and boundary conditions of a workload name (without the solver)."""
    for key in (", LSQR", ", BiCGSTAB", ", GMRES"):
        name = name.split(key)[0]
    return name


def set_solver(A, C, name, args):
    C.set_solver(solver_id(A, name), restart=args.restart if name == "gmres" else None)


def workload(args):
    from andromeda_gb300 import mesh as M
    p = M.icosphere(args.level, 1.0, inward=True)
    m = M.particle_in_sphere(p, outer_level=args.outer_level, outer_radius=args.outer_radius)
    name = (f"Stokes sphere a=1 icosphere L{args.level} ({len(p['etype'])} tri) in L{args.outer_level} container "
            f"r={args.outer_radius:g} ({len(m['etype']) - len(p['etype'])} tri), 6 RHS, ITRI 5, mu=1, "
            f"{solver_text(getattr(args, 'solver', 'lsqr'), args.eps)}")
    return m, name


def rigid_fields(m, outer_wall=2):
    import numpy as np
    nn = len(m["xyz"])
    on = np.zeros(nn, bool)
    for e in np.where(m["bcid"] == outer_wall)[0]:
        on[m["con"][e, :3]] = True
    U = np.zeros((6, 3, nn))
    for i in range(3):
        U[i, i, on] = 1.0
        w = np.zeros(3)
        w[i] = 1.0
        U[3 + i][:, on] = np.cross(w, m["xyz"][on]).T
    return U


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    def __init__(self, index=0):
        self.cmd = ["nvidia-smi", "-i", str(index),
                    "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                    "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                    "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                    "--format=csv,noheader,nounits", "-lms", "200"]
        self.p = None
        self.out = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(self.cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out, _ = self.p.communicate()

    def summary(self):
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks(key="hbm_gbs"):
    """The measured peak (HBM copy GB/s, or "bf16_tflops") and its source."""
    fallback = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}[key]
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if key in d:
            return float(d[key]), "measured"
    return fallback, "fallback"


# FLOPs of k_stokes_G per (collocation point, element, quadrature point)
STOKES_G_FLOPS_PER_POINT = 28


def fp32_peak_tflops():
    """Nominal FP32 peak of the GPU: SMs x 128 FP32 lanes x 2 (FMA) x the
    maximum SM clock (measured clock from MEASURED_PEAKS.json when present).
    No measured FP32 figure exists, so this is the nominal one."""
    sms = 152
    try:
        import torch
        if torch.cuda.is_available():
            sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    mhz, src = 2070.0, "nominal (152 SMs x 128 lanes x 2 x 2070 MHz)"
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    src = f"nominal: {sms} SMs x 128 FP32 lanes x 2 (FMA) x {mhz:g} MHz"
    return sms * 128 * 2 * mhz * 1e6 / 1e12, src


def dist_env():
    from andromeda_gb300.ranks import dist_env as env
    return env()


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 restatement of the reference on the host cores
# ---------------------------------------------------------------------------
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle


def small_body(level, outer_level, outer_radius):
    from andromeda_gb300 import mesh as M
    p = M.icosphere(level, 1.0, inward=True)
    m = M.particle_in_sphere(p, outer_level=outer_level, outer_radius=outer_radius)
    name = (f"Stokes sphere a=1 icosphere L{level} ({len(p['etype'])} tri) in L{outer_level} container "
            f"r={outer_radius:g} ({len(m['etype']) - len(p['etype'])} tri), 6 RHS, ITRI 5, mu=1")
    return m, name


def cpu_complete_solve(m, eps, threads=None):
    """One complete resistance-tensor solve by the reference algorithm (the
    oracle's FP64 restatement), timed in full: CoR_Integrals_Stokes over all
    nsp = nnodes + nelem source rows on every host thread (the reference
    splits rows over MPI ranks), then per right-hand side the reference's
    serial CRS system, lsqr_precon + lsqr_solve to eps and the force/torque
    integrals (StokesInlet3sidesForceCRS / ...TorqueOmegaCRS, one field after
    another).  Nothing is scaled.  threads: the integration's host threads
    (default: all of them; 1 is the reference's serial path)."""
    import numpy as np
    oracle = _oracle()
    U = rigid_fields(m)
    prev = oracle.num_threads()
    if threads:
        oracle.set_threads(threads)
    try:
        t0 = time.perf_counter()
        P = oracle.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
        P.form_integrals()
        t1 = time.perf_counter()
        _, ft, nits, ierr = P.stokes_solve_sequence(U, maxit=0, eps=eps, fwall=1)
        t2 = time.perf_counter()
        P.close()
    finally:
        oracle.set_threads(prev)
    return {"seconds": t2 - t0, "integration_s": t1 - t0, "solve_s": t2 - t1, "nit": [int(v) for v in nits],
            "ierr": int(ierr), "R": ft}


def single_thread_leg(m, eps):
    """The same complete solve with the integration on one host thread (the
    reference's serial path: the whole solve on one core)."""
    r = cpu_complete_solve(m, eps, threads=1)
    return {"solves_per_s": 1.0 / r["seconds"], "seconds": r["seconds"], "integration_s": r["integration_s"],
            "cores": 1}


def cpu_c2_estimate(m, nit_fp64, budget_s):
    """Estimate (not a measurement) of one solve of the full-size workload by
    the reference algorithm on these cores, which would take hours:
      * integration: a slice of the source rows of this very mesh at ITRI 5 on
        every host thread, scaled by nsp (every row integrates over all
        elements, so the cost per row is uniform);
      * LSQR: serial CRS iterations on the ITRI-5 system of a smaller body of
        the same kind, per nonzero, scaled to the full system's nonzeros and to
        the FP64 LSQR iteration counts of this workload (nit_fp64, summed over
        the six right-hand sides the reference solves one after another)."""
    import numpy as np
    oracle = _oracle()
    threads = os.cpu_count() or 1
    P = oracle.Problem(2, m, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    nsp = P.nsp
    t_row, rows = 0.0, 0
    r0 = P.sd_nnodes
    t_start = time.perf_counter()
    while time.perf_counter() - t_start < 0.5 * budget_s and rows < 4 * threads * 8:
        t, _ = P.time_rows(r0 + rows, r0 + rows + threads, threads)
        t_row += t
        rows += threads
    P.close()
    t_integration = t_row / rows * nsp
    ms, _ = small_body(3, 2, 200.0)
    Ps = oracle.Problem(2, ms, walls=[1, 2], known=np.ones((3, 2)), itri=5)
    Ps.form_integrals()
    Ps.form_system()
    ia, ja, a = Ps.crs(0)
    q = oracle.lsqr_precon(Ps.neq_rows, Ps.nx, ia, ja, a)
    b = np.random.default_rng(0).normal(size=Ps.neq_rows)
    it = 8
    while True:
        x = np.zeros(Ps.nx)
        t0 = time.perf_counter()
        oracle.lsqr_solve(Ps.neq_rows, Ps.nx, ia, ja, a, q, b, x, maxit=it, eps=1e-30)
        dt = time.perf_counter() - t0
        if dt > 0.25 * budget_s or it >= 4096:
            break
        it *= 2
    per_nnz_iter = dt / (it * len(a))
    n_full = 3 * len(m["etype"])
    nit_total = int(sum(nit_fp64))
    t_lsqr = per_nnz_iter * float(n_full) ** 2 * nit_total
    total = t_integration + t_lsqr
    return {"kind": "extrapolated", "seconds_per_solve": total, "solves_per_s": 1.0 / total,
            "integration_s": t_integration, "lsqr_s": t_lsqr, "cores": threads, "lsqr_threads": 1,
            "sample": (f"{rows} of {nsp} integration rows (ITRI 5) on {threads} threads, scaled by nsp; {it} serial "
                       f"CRS LSQR iterations on the ITRI-5 {Ps.neq_rows}^2 system of the L3 sphere, scaled by nnz "
                       f"to {n_full}^2 and to {nit_total} iterations (FP64 LSQR counts {list(nit_fp64)} of this "
                       f"workload, summed over the six sequential right-hand sides)")}


# FP64 LSQR iteration counts of the full-size workload at eps 1e-7 (the six
# rigid motions), measured by the converged FP64 GPU solve of this benchmark,
# whose LSQR recurrence is the reference's (iteration counts equal to the
# oracle's on every tested system); used only by the estimate above when the
# reference arm runs alone.
C2_NIT_FP64_EPS1E7 = [603, 605, 606, 194, 195, 196]


def run_reference(args, rank):
    """Reference arm: complete solves by the reference algorithm (the FP64
    oracle port) on the host cores, each step one full resistance-tensor solve
    of a body small enough to finish in seconds (the L2 sphere in the same
    container); the full-size workload's time is given as an estimate beside
    it, labelled as such."""
    if rank != 0:
        return
    import numpy as np
    m, name = small_body(args.cpu_level, args.outer_level, args.outer_radius)
    for _ in range(args.warmup):
        cpu_complete_solve(m, args.eps)
    secs, last = [], None
    t0 = time.perf_counter()
    for _ in range(args.steps):
        last = cpu_complete_solve(m, args.eps)
        secs.append(last["seconds"])
    wall = time.perf_counter() - t0
    v = args.steps / sum(secs)
    threads = os.cpu_count() or 1
    single = single_thread_leg(m, args.eps)
    est = None
    if args.c2_estimate:
        mf, _ = workload(args)
        nit64 = C2_NIT_FP64_EPS1E7 if (args.level == 5 and abs(args.eps - 1e-7) < 1e-12 and C2_NIT_FP64_EPS1E7) \
            else None
        if nit64:
            est = cpu_c2_estimate(mf, nit64, args.cpu_seconds)
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * sum(secs) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (meshes generated in-process)",
            "config": {"workload": f"{name}, LSQR eps {args.eps:g} (complete solves; the full-size L{args.level} "
                                   f"workload takes hours on the host cores, see c2_estimate)",
                       "same_body_as_gpu_line": False, "nit": last["nit"]},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} complete solves of the L{args.cpu_level} body, nothing scaled "
                                       f"(integration on {threads} threads, serial CRS LSQR per right-hand side)"},
            "host_s": wall, "c2_estimate": est, "single_thread": single,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_batch(args, rank, world, local):
    """Many-body workload: superellipsoids a=1, b,c ~ U(0.2,1), e1,e2 ~ U(0.3,1.8),
    random orientation, 500..8000 triangles (log-uniform), seed 20260101, each
    in a level-2 container of radius 200; 6 RHS each; one agb_batch_resistance
    call per step.  Under torchrun every rank solves its own share of the
    bodies (bodies i with i % world == rank): no collective on the data path."""
    import numpy as np
    import andromeda_gb300 as A
    from andromeda_gb300 import mesh as M
    meshes, params = M.batch_bodies(n_bodies=args.bodies)
    from andromeda_gb300.ranks import shard, max_over_ranks, barrier
    mine = [meshes[i] for i in shard(len(meshes), world, rank)]
    ctx = A.Context(local if world > 1 else 0)
    eps = args.batch_eps
    tune = not args.no_autotune
    warm = mine[:32]
    solver = solver_id(A, args.solver)
    for _ in range(args.warmup):
        A.batch_resistance(warm, eps=eps, ctx=ctx, autotune=tune, solver=solver)
    barrier()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        Rs, nits, istops, sts = [], [], [], []
        for _ in range(args.steps):
            R, nit, istop, st = A.batch_resistance(mine, eps=eps, ctx=ctx, autotune=tune, solver=solver)
            Rs.append(R); nits.append(nit); istops.append(istop); sts.append(st)
        t1 = time.perf_counter()
    dev_s = sum(st["device_ms"] for st in sts) / 1000.0
    wall_s = t1 - t0
    dev_s, wall_s = max_over_ranks([dev_s, wall_s], device="cuda" if world > 1 else "cpu")
    value = args.bodies * args.steps / dev_s
    R, nit, istop, st = Rs[-1], nits[-1], istops[-1], sts[-1]
    # FP64 GPU path on a seeded random sample of the bodies: its rate at the same
    # eps, and a tighter FP64 solve as the truth for the mixed tensors' error
    fp64 = None
    if rank == 0 and world == 1 and args.fp64_sample > 0:
        rng = np.random.default_rng(1)
        pick = sorted(rng.choice(len(mine), size=min(args.fp64_sample, len(mine)), replace=False).tolist())
        t64, errs = [], []
        for i in pick:
            C = A.Context(0)
            C.set_mesh(mine[i])
            C.set_problem(A.STOKES, [1, 2], A.dirichlet_known(A.STOKES, 2), itri=5)
            _, _, info = C.resistance_tensor(A.FP64, 1, 2, eps=eps)
            t64.append(info["device_ms"])
            Rt, _, _ = C.resistance_tensor(A.FP64, 1, 2, eps=eps * 1e-3)
            errs.append(float(np.max(np.abs(R[i] - Rt)) / np.max(np.abs(Rt))))
            C.close()
        rate64 = len(pick) / (sum(t64) / 1000.0)
        fp64 = {"solves_per_s": rate64, "sample_bodies": pick,
                "sample_elements": [int(params[i][4]) for i in pick], "ms_per_body": t64,
                "ratio_mixed_batched_over_fp64": value / world / rate64,
                "truth": f"FP64 assembly + FP64 LSQR to eps {eps * 1e-3:g}"}
        rel_err = max(errs)
    else:
        errs, rel_err = None, None
    peak, peak_kind = measured_peaks()
    av_gbs = st["av_bytes"] / (st["av_ms"] * 1e-3) / 1e9 if st["av_ms"] > 0 else None
    # DRAM traffic of one sweep launch: its algorithmic bytes times the
    # traffic/algorithmic ratio of the 16-body ncu capture of the same kernel
    av_bytes_launch = st["av_bytes"] / max(st["av_launches"], 1.0)
    traffic = None
    if os.path.exists(PROFILE_BATCH) and args.solver == "gmres":
        with open(PROFILE_BATCH) as f:
            for ln in f:
                if ln.startswith("traffic_ratio_gb_avp_b16:"):
                    traffic = float(ln.split(":")[1]) * av_bytes_launch
    atu_gbs = st["av_bytes"] / (st["atu_ms"] * 1e-3) / 1e9 if st["atu_ms"] > 0 else None
    ne = params[:, 4]
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
                "scaling": "weak" if world > 1 else "weak", "vs_baseline": None,
                "dtype": "fp32 (fp64 singular/free-term/reductions)",
                "data": "synthetic (meshes generated in-process, seed 20260101)",
                "config": {"workload": f"{args.bodies} superellipsoids a=1, b,c~U(0.2,1), e1,e2~U(0.3,1.8), "
                                       f"random orientation, {int(ne.min())}..{int(ne.max())} tri (mean "
                                       f"{ne.mean():.0f}), each in an L2 container r=200, 6 RHS, ITRI 5, "
                                       + solver_text(args.solver, eps),
                           "precision": "mixed", "parallelism": "bodies split over ranks" if world > 1 else
                           "single GPU", "l2": "inputs larger than L2 (waves of tens of GB), no flush",
                           "warmup": f"{args.warmup} x the first {len(warm)} bodies"},
                "rel_err_vs_fp64": rel_err, "rel_err_sample": errs,
                "istop_counts": {str(k): int(v) for k, v in zip(*np.unique(istop, return_counts=True))},
                "nit_mean": float(np.mean(nit)), "nit_max": int(np.max(nit)),
                "e2e": {"value": args.bodies * args.steps / wall_s, "unit": "solves/s",
                        "h2d_bytes_per_step": int(sum(m["xyz"].nbytes + m["etype"].nbytes + m["con"].nbytes +
                                                      m["bcid"].nbytes for m in meshes)),
                        "d2h_bytes_per_step": int(args.bodies * (36 * 8 + 12 * 4))},
                "roofline": {"bound": "hbm", "kernel": ("gb_avp (batched GMRES A M^-1 v sweep" if args.solver == "gmres"
                                                        else "g_avp (batched LSQR A*V sweep") +
                                                       " over the packed symmetric 3x3 blocks, FP32 by TMA, all bodies "
                                                       "in one launch)",
                             "achieved": av_gbs, "peak": peak, "unit": "GB/s",
                             "frac": av_gbs / peak if av_gbs else None, "traffic": traffic, "peak_source": peak_kind,
                             "algorithmic_bytes_per_launch": av_bytes_launch,
                             "other_sweep": {"kernel": "g_atup (batched A^T*U, packed)", "achieved": atu_gbs,
                                             "frac": atu_gbs / peak if atu_gbs else None}},
                "batch": {k: st[k] for k in ("assemble_ms", "solve_ms", "total_ms", "waves", "av_rows", "atu_rs",
                                              "atu_rows", "iterations", "device_ms", "ft_ms")},
                "cpu_baseline": None, "clocks": clk.summary(), "gpu_launches": int(sum(s_["launches"] for s_ in sts)),
                "host_s": wall_s, "fp64_gpu": fp64}
        print(json.dumps(line), flush=True)
    ctx.close()


def run_large(args):
    """Single large body: superellipsoid a=1, b=0.5, c=0.25, e1=0.6, e2=1.4 on
    a rings x sectors signed-power grid (160 x 320 = 102400 triangles) in a
    level-2 container of radius 200 (102 720 elements, 308 160 unknowns).

    resident (default): the single layer is assembled once in the packed
    symmetric-block FP32 layout (6 x 102 720^2 x 4 B = 253 GB, resident in HBM)
    and the resistance tensor is solved to convergence (LSQR eps --eps); the
    line reports solves/s.  mf: the matrix (377 GB as a full FP32 matrix) is
    recomputed in every LSQR sweep; a bounded number of iterations is timed and
    the line reports iterations/s."""
    import numpy as np
    import andromeda_gb300 as A
    from andromeda_gb300 import mesh as M
    nr, ns = (int(v) for v in args.grid.split("x"))
    body = M.superellipsoid(1.0, 0.5, 0.25, 0.6, 1.4, nr, ns, inward=True)
    m = M.particle_in_sphere(body, outer_level=2, outer_radius=200.0)
    C = A.Context(0)
    C.set_mesh(m)
    C.set_problem(A.STOKES, [1, 2], A.dirichlet_known(A.STOKES, 2), itri=5)
    set_solver(A, C, args.solver, args)
    ne = len(m["etype"])
    workload = (f"superellipsoid a=1 b=0.5 c=0.25 e1=0.6 e2=1.4, {nr}x{ns} grid ({len(body['etype'])} tri) "
                f"in an L2 container r=200, 6 RHS, ITRI 5")
    if args.large_mode == "resident":
        # the packed FP32 single layer must fit in device memory (6 ne^2 x 4 B + ~2 %
        # for the vectors); otherwise the matrix-free sweeps below
        free_b = None
        try:
            import torch
            free_b = torch.cuda.mem_get_info(0)[0]
        except Exception:
            pass
        if free_b is not None and 24.0 * ne * ne * 1.02 > free_b:
            print(f"# packed matrix ({24.0 * ne * ne / 1e9:.0f} GB) exceeds the free device memory "
                  f"({free_b / 1e9:.0f} GB): matrix-free sweeps", file=sys.stderr)
            args.large_mode = "mf"
    if args.large_mode == "resident":
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            C.kernel_times(reset=True)
            R, nit, info = C.resistance_tensor(A.MIXED, 1, 2, maxit=args.large_maxit, eps=args.large_eps)
            t1 = time.perf_counter()
        kt = C.kernel_times(reset=True)
        av_ms = kt["av_ms"] / max(kt["av_launches"], 1)
        atu_ms = kt["atu_ms"] / max(kt["atu_launches"], 1)
        peak, peak_kind = measured_peaks()
        alg = 24.0 * ne * ne
        sym = float(np.max(np.abs(R - R.T)) / np.max(np.abs(R)))
        # error against the plain FP64 path on the same body, where its dense FP64
        # matrix (3 ne x 3 ne x 8 B) fits the free device memory
        fp64 = None
        if args.large_fp64_eps > 0:
            try:
                import torch
                free_b = torch.cuda.mem_get_info(0)[0]
            except Exception:
                free_b = None
            need = 72.0 * ne * ((ne + 31) // 32 * 32) * 1.02
            if free_b is None or need < 0.9 * free_b + 24.0 * ne * ne:
                C.set_solver(A.SOLVER_LSQR)
                R64, nit64, info64 = C.resistance_tensor(A.FP64, 1, 2, eps=args.large_fp64_eps)
                fp64 = {"rel_err_vs_fp64": float(np.max(np.abs(R - R64)) / np.max(np.abs(R64))),
                        "fp64_eps": args.large_fp64_eps, "fp64_nit": [int(v) for v in nit64],
                        "fp64_istop": [int(v) for v in info64["istop"]], "fp64_device_ms": info64["device_ms"],
                        "force_torque_rel_err": {
                            "drag": float(np.max(np.abs(np.diag(R)[:3] - np.diag(R64)[:3]) / np.abs(np.diag(R64)[:3]))),
                            "torque": float(np.max(np.abs(np.diag(R)[3:] - np.diag(R64)[3:]) /
                                                   np.abs(np.diag(R64)[3:])))}}
            else:
                fp64 = {"skipped": f"the FP64 matrix ({need / 1e9:.0f} GB) does not fit"}
        line = {"metric": "Stokes resistance-tensor solves/s, single large body (mixed, packed matrix resident)",
                "value": 1000.0 / info["device_ms"], "unit": "solves/s", "n_gpus": 1, "steps": 1, "warmup": 0,
                "ms_per_step": info["device_ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "fp32 (fp64 singular/free-term/reductions)", "data": "synthetic",
                "config": {"workload": workload + ", " + solver_text(args.solver, args.large_eps), "unknowns": C.n,
                           "packed_matrix_gb": alg / 1e9, "l2": "inputs larger than L2, no flush"},
                "assemble_ms": info["assemble_ms"], "rhs_ms": info["rhs_ms"], "solve_ms": info["solve_ms"],
                "nit": [int(v) for v in nit], "istop": info["istop"],
                "tensor_asymmetry": sym, "fp64_check": fp64, "R": R.tolist(),
                "sweep_ms": {"av": av_ms, "atu": atu_ms},
                "roofline": {"bound": "hbm", "kernel": "k_avp (packed A*V sweep, 253 GB per launch)",
                             "achieved": alg / (av_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": alg / (av_ms * 1e-3) / 1e9 / peak, "traffic": None, "peak_source": peak_kind,
                             "algorithmic_bytes_per_launch": alg,
                             "other_sweep": ({"kernel": "k_atup", "achieved": alg / (atu_ms * 1e-3) / 1e9,
                                              "frac": alg / (atu_ms * 1e-3) / 1e9 / peak} if atu_ms > 0 else None)},
                "clocks": clk.summary(), "gpu_launches": kt["launches"], "host_s": t1 - t0}
        print(json.dumps(line), flush=True)
        C.close()
        return
    C.set_solver(A.SOLVER_LSQR)  # the matrix-free operator runs the reference's LSQR only
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        C.kernel_times(reset=True)
        R, nit, info = C.resistance_tensor(A.MATRIX_FREE, 1, 2, maxit=args.mf_iters, eps=args.batch_eps)
        t1 = time.perf_counter()
    kt = C.kernel_times(reset=True)
    av_ms = kt["av_ms"] / max(kt["av_launches"], 1)
    atu_ms = kt["atu_ms"] / max(kt["atu_launches"], 1)
    # FP32 work of one sweep: ne^2 pairs x Q points x 28 flops (the point kernel) + the 8-RHS contraction
    Q = 126
    flops = float(ne) * ne * Q * 28.0 + float(ne) * ne * 2 * 9 * 8
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    line = {"metric": "matrix-free LSQR sweep rate (FP32 recomputed single layer)", "value": 1000.0 / (av_ms + atu_ms),
            "unit": "iterations/s", "n_gpus": 1, "steps": args.mf_iters, "warmup": 0,
            "ms_per_step": av_ms + atu_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (fp64 self blocks, reductions, recurrences)", "data": "synthetic",
            "config": {"workload": workload, "unknowns": C.n, "matrix_fp32_gb_if_stored": C.n * C.n * 4 / 1e9},
            "assemble_ms": info["assemble_ms"], "rhs_ms": info["rhs_ms"], "nit": [int(v) for v in nit],
            "sweep_ms": {"av": av_ms, "atu": atu_ms},
            "roofline": {"bound": "fp32 pipe", "kernel": "k_mf_av / k_mf_atu",
                         "achieved": flops / (av_ms * 1e-3) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": flops / (av_ms * 1e-3) / 1e12 / fp32_peak, "traffic": None,
                         "peak_source": "nominal FP32 (152 SM x 128 FMA/clk x 2 x 2.07 GHz)",
                         "other_sweep": {"achieved": flops / (atu_ms * 1e-3) / 1e12,
                                         "frac": flops / (atu_ms * 1e-3) / 1e12 / fp32_peak}},
            "clocks": clk.summary(), "gpu_launches": kt["launches"], "host_s": t1 - t0,
            "note": "a bounded number of iterations (maxit) is timed; the solve itself is not run to convergence"}
    print(json.dumps(line), flush=True)
    C.close()


def run_laplace(args):
    """Laplace case of the reference (its own CPU-runnable configuration):
    unit icosphere level 3 (642 nodes, 1 280 flat triangles), Dirichlet
    u = x + 2y + 3z on the whole surface, unknown flux, FP64, ITRI --itri
    (1 = 7-point rule), LSQR eps --laplace-eps.  A step is assembly + solve on
    the GPU (FP64 path, host arrays in and out).  The oracle port of the
    reference's CPU path (integration of all nsp rows, CRS system,
    lsqr_precon + lsqr_solve) runs in full on the host cores beside it, and
    its flux is the parity check of the step's."""
    import numpy as np
    import andromeda_gb300 as A
    from andromeda_gb300 import mesh as M
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    m = M.icosphere(3)
    u = m["xyz"] @ np.array([1.0, 2.0, 3.0])
    C = A.Context(0)
    C.set_mesh(m)
    C.set_problem(A.LAPLACE, [1], A.dirichlet_known(A.LAPLACE, 1), itri=args.itri)

    def step():
        C.assemble(A.FP64)
        return C.solve(u[None], eps=args.laplace_eps)

    for _ in range(max(args.warmup, 1)):
        step()
    C.kernel_times(reset=True)
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            x, nit, istop = step()
            times.append(time.perf_counter() - t0)
    kt = C.kernel_times(reset=True)
    n, _, _ = C.geometry()
    qex = -(n @ np.array([1.0, 2.0, 3.0]))
    C.close()
    # the oracle (reference algorithm, FP64, host cores), timed in full
    t0 = time.perf_counter()
    P = oracle.Problem(1, m, walls=[1], known=[[1]], itri=args.itri)
    P.form_integrals()
    P.form_system()
    _, q_ref, nit_ref, _ = P.laplace_solve(u, np.zeros(P.nelem), maxit=0, eps=args.laplace_eps)
    t_cpu = time.perf_counter() - t0
    P.close()
    ms = 1000.0 * statistics.median(times)
    line = {"metric": "Laplace BEM solves/s (assembly + LSQR, FP64)", "value": 1000.0 / ms, "unit": "solves/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 1), "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"unit icosphere L3 (1280 tri), Laplace, u = x+2y+3z, ITRI {args.itri}, "
                                   f"LSQR eps {args.laplace_eps:g}"},
            "nit": int(nit[0]), "istop": int(istop[0]), "nit_oracle": int(nit_ref),
            "rel_err_vs_oracle": float(np.max(np.abs(x[0] - q_ref)) / np.max(np.abs(q_ref))),
            "flux_rel_err_vs_analytic": float(np.linalg.norm(x[0] - qex) / np.linalg.norm(qex)),
            "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "solves/s", "cores": oracle.num_threads(), "kind": "port",
                             "sample": "the whole solve (integration of all rows, CRS system, lsqr_precon + "
                                       "lsqr_solve), not scaled"},
            "e2e": {"value": 1000.0 / ms, "unit": "solves/s", "h2d_bytes_per_step": int(u.nbytes),
                    "d2h_bytes_per_step": int(x.nbytes)},
            "clocks": clk.summary(), "gpu_launches": kt["launches"] // max(args.steps, 1)}
    print(json.dumps(line), flush=True)


def run_surrogate(args):
    """Learned part: BEM tensors of the many-body workload's shapes (the batched
    mixed BEM on config-4 bodies: superellipsoids of --sur-elements triangles in
    level-2 containers of radius 200) train an ensemble of MLPs on the GPU; a
    held-out set calibrates the members' agreement threshold; one batch of
    queries is answered by the ensemble (the BEM outside the training hull or
    where the members disagree), and a random audit fraction is re-solved by
    the BEM."""
    import numpy as np
    import andromeda_gb300 as A
    from andromeda_gb300 import surrogate as S
    bem = dict(n_elem=args.sur_elements, outer_level=2, outer_radius=200.0, eps=args.batch_eps,
               solver=solver_id(A, args.solver))
    t0 = time.perf_counter()
    P = S.sample_params(args.train_bodies, seed=20260101)
    R, st_bem = S.bem_tensors(P, **bem)
    t1 = time.perf_counter()
    sur = S.Surrogate(device=0, seed=7, bem_kwargs=bem, members=args.members)
    ncal = max(200, int(0.05 * len(P)))
    ntr = len(P) - ncal
    hist, st_tr = sur.fit(P[:ntr], R[:ntr], epochs=args.epochs, batch=512, lr=2e-3, lr_final=2e-5)
    t2 = time.perf_counter()
    cal = sur.calibrate(P[ntr:], R[ntr:], target=1e-3, margin=args.sur_margin)
    Q = S.sample_params(args.queries, seed=99)
    Xq = S.features(Q)
    for _ in range(max(args.warmup, 1)):
        sur.ensemble(Xq[:65536])
    with ClockSampler(0) as clk:
        times, times1 = [], []
        for _ in range(max(args.steps, 1)):
            _, _, ms_e = sur.ensemble(Xq)
            times.append(ms_e)
            _, ms1 = sur.net.predict(Xq)
            times1.append(ms1)
    # end to end on a sample of the queries (the BEM answers every rejected one:
    # on the full million that alone takes tens of minutes); the ensemble's
    # acceptance over all queries is counted without the BEM
    npred = min(args.queries, max(1, args.predict_queries))
    _, acc_all, info_all = sur.predict(Q, bem=False)
    t3 = time.perf_counter()
    Rq, accq, info_q = sur.predict(Q[:npred])  # accepted by the ensemble, the rest by the BEM
    t4 = time.perf_counter()
    aud, idx, aacc, st_aud = sur.audit(Q, frac=args.audit, seed=3)
    t5 = time.perf_counter()
    ms = statistics.median(times)
    ms1 = statistics.median(times1)
    flops1 = 2.0 * (5 * 256 + 2 * 256 * 256 + 256 * 21) * args.queries * 3  # split-BF16: three products per GEMM
    bf16 = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16 = json.load(f).get("bf16_tflops")
    except Exception:
        pass
    bem_rate = len(P) / (st_bem["device_ms"] / 1000.0)
    nm = len(sur.nets)
    line = {"metric": f"surrogate resistance-tensor inferences/s (ensemble of {nm} MLPs 5-256-256-256-21, BEM "
                      "fallback outside the hull or above the calibrated disagreement)",
            "value": args.queries / (ms / 1000.0), "unit": "inferences/s", "n_gpus": 1, "steps": max(args.steps, 1),
            "warmup": max(args.warmup, 1), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 tensor cores (split hi+lo, fp32 accumulation)",
            "data": "synthetic (shapes b,c~U(0.2,1), e1,e2~U(0.3,1.8), seeds 20260101 / 99)",
            "config": {"workload": f"{args.queries} queries; {nm} networks trained on {ntr} BEM tensors of the "
                                   f"many-body workload's shapes ({args.sur_elements}-triangle superellipsoids in L2 "
                                   f"containers r=200, batched mixed BEM, {solver_text(args.solver, args.batch_eps)}); "
                                   f"{ncal} "
                                   f"held-out tensors calibrate the agreement threshold",
                       "epochs": args.epochs, "batch": 512, "members": nm},
            "bem_training_set": {"bodies": len(P), "bem_solves_per_s": bem_rate, "host_s": t1 - t0},
            "training": {"device_ms": st_tr["device_ms"], "launches": st_tr["launches"],
                         "adam_steps": st_tr["adam_steps"], "loss_first": float(hist[0]),
                         "loss_last": float(hist[-1]), "host_s": t2 - t1},
            "calibration": cal,
            "queries_accepted": int(info_all["n_mlp"]), "queries_bem_fallback": int(info_all["n_bem"]),
            "fallback_outside_hull": int(info_all["n_outside_hull"]),
            "fallback_disagreement": int(info_all["n_spread_rejected"]),
            "fallback_rate": info_all["n_bem"] / args.queries,
            "predict_sample_host_s": t4 - t3,
            "audit": {"fraction": args.audit, "n": int(len(idx)), "accepted": int(aacc.sum()),
                      "rel_err_median": float(np.median(aud)) if len(aud) else None,
                      "rel_err_p95": float(np.percentile(aud, 95)) if len(aud) else None,
                      "rel_err_max": float(np.max(aud)) if len(aud) else None,
                      "within_1e-3": float(np.mean(aud <= 1e-3)) if len(aud) else None, "host_s": t5 - t4},
            "speedup_over_bem": (args.queries / (ms / 1000.0)) / bem_rate,
            "single_network": {"inferences_per_s": args.queries / (ms1 / 1000.0), "ms": ms1},
            "roofline": {"bound": "tensor", "achieved": flops1 / (ms1 * 1e-3) / 1e12, "peak": bf16,
                         "unit": "TFLOP/s", "frac": (flops1 / (ms1 * 1e-3) / 1e12 / bf16) if bf16 else None,
                         "traffic": None, "peak_source": "measured bf16 (cuBLAS burst)" if bf16 else None,
                         "kernel": "k_mlp_infer_tc (all four layers in one kernel, 128 queries per CTA, "
                                   "activations on chip; tcgen05.mma bf16, FP32 accumulators in TMEM), one network",
                         "note": "split-BF16: the three products per GEMM are counted"},
            "cpu_baseline": None, "clocks": clk.summary(),
            "gpu_launches": int(sum(n._L.agb_mlp_launches(n.h) for n in sur.nets)),
            "e2e": {"value": npred / (t4 - t3), "queries": npred,
                    "unit": "inferences/s (predict with hull and agreement check, "
                                                             "BEM fallback included, host arrays)",
                    "h2d_bytes_per_step": int(npred * 5 * 4 * nm),
                    "d2h_bytes_per_step": int(npred * 21 * 4 * nm)}}
    print(json.dumps(line), flush=True)
    sur.close()


def run_mlp(args):
    """The fused surrogate inference kernel alone: --queries queries through a
    randomly initialised 5-256-256-256-21 network (weights and biases drawn
    once, seed 3), split-BF16 products; the kernel's CUDA-event time per call.
    The outputs are checked against the layer-by-layer split-BF16 GEMMs."""
    import numpy as np
    from andromeda_gb300.surrogate import MLP
    net = MLP(device=0, seed=3)
    rng = np.random.default_rng(0)
    p = net.params()
    net.set_params(p + rng.normal(scale=0.05, size=p.shape).astype(np.float32))
    X = rng.uniform(0.2, 1.8, (args.queries, 5)).astype(np.float32)
    net.set_normalization(X.mean(0), X.std(0) + 1e-3, np.zeros(21, np.float32), np.ones(21, np.float32))
    for _ in range(max(args.warmup, 1)):
        net.predict(X)
    with ClockSampler(0) as clk:
        ms = [net.predict(X)[1] for _ in range(max(args.steps, 1))]
    Yf, _ = net.predict(X)
    Yg, _ = net.predict(X, fused=False)
    med = statistics.median(ms)
    flops = 2.0 * (5 * 256 + 2 * 256 * 256 + 256 * 21) * args.queries * 3
    peak, _ = measured_peaks("bf16_tflops")
    line = {"metric": "surrogate inference kernel inferences/s (one MLP 5-256-256-256-21, split-BF16 tcgen05)",
            "value": args.queries / (med / 1000.0), "unit": "inferences/s", "n_gpus": 1, "steps": len(ms),
            "warmup": max(args.warmup, 1), "ms_per_step": med, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 tensor cores (split hi+lo, fp32 accumulation)",
            "data": "synthetic (random weights, seed 3; inputs U(0.2, 1.8))",
            "config": {"workload": f"{args.queries} queries, one network", "l2": "weights L2-resident by design"},
            "roofline": {"bound": "tensor", "achieved": flops / (med * 1e-3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                         "frac": flops / (med * 1e-3) / 1e12 / peak if peak else None, "traffic": None,
                         "kernel": "k_mlp_infer_tc", "note": "split-BF16: the three products per GEMM are counted"},
            "max_abs_diff_vs_layer_gemms": float(np.max(np.abs(Yf - Yg))),
            "clocks": clk.summary(), "cpu_baseline": None}
    print(json.dumps(line), flush=True)
    net.close()


# ---------------------------------------------------------------------------
def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "surrogate":
        if rank == 0:
            run_surrogate(args)
        return
    if args.workload == "large":
        if rank == 0:
            run_large(args)
        return
    if args.workload == "laplace":
        if rank == 0:
            run_laplace(args)
        return
    if args.workload == "mlp":
        if rank == 0:
            run_mlp(args)
        return
    if args.workload == "batch":
        if world > 1:
            import torch
            import torch.distributed as dist
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        run_batch(args, rank, world, local)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return
    import numpy as np
    import andromeda_gb300 as A
    from andromeda_gb300 import build as B
    if not os.path.exists(A.LIB_PATH):
        B.build()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    m, name = workload(args)
    C = A.Context(local if world > 1 else 0)
    C.set_mesh(m)
    C.set_problem(A.STOKES, [1, 2], A.dirichlet_known(A.STOKES, 2), itri=5)
    set_solver(A, C, args.solver, args)

    def step():
        return C.resistance_tensor(A.MIXED, 1, 2, eps=args.eps)

    for _ in range(args.warmup):
        step()
    C.kernel_times(reset=True)
    if dist is not None:
        dist.barrier()
    dev_ms, host_ms, Rs, nits = [], [], [], []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            R, nit, info = step()
            dev_ms.append(info["device_ms"])
            Rs.append(R)
            nits.append(nit)
        t1 = time.perf_counter()
    kt = C.kernel_times(reset=True)
    elapsed = sum(dev_ms) / 1000.0
    if dist is not None:
        from andromeda_gb300.ranks import max_over_ranks
        elapsed = max_over_ranks([elapsed], device="cuda")[0]
    value = world * args.steps / elapsed
    R = Rs[-1]
    nit = nits[-1]

    # accuracy against the FP64 GPU path (frozen truth of this workload)
    rel_err = None
    if os.path.exists(GOLDEN_TRUTH):
        with open(GOLDEN_TRUTH) as f:
            g = json.load(f)
        if g.get("workload") == mesh_part(name):  # the mesh and BCs only
            Rt = np.array(g["R"])
            rel_err = float(np.max(np.abs(R - Rt)) / np.max(np.abs(Rt)))
    lam = 1.0 / args.outer_radius
    K = (1 - lam ** 5) / (1 - 9 / 4 * lam + 5 / 2 * lam ** 3 - 9 / 4 * lam ** 5 + lam ** 6)
    drag_ratio = float(np.mean(np.diag(R[:3, :3])) / (6 * np.pi * K))
    torque_ratio = float(np.mean(np.diag(R[3:, 3:])) / (8 * np.pi / (1 - lam ** 3)))

    # roofline of the dominant kernel (A*V sweep of LSQR), live CUDA-event timing
    peak, peak_kind = measured_peaks()
    lda = (C.n + 31) // 32 * 32
    # packed symmetric 3x3 blocks: 6 FP32 values per (collocation point, element) pair
    ne_sys = C.m // 3
    a_bytes = 6 * ne_sys * ne_sys * 4
    av_ms = kt["av_ms"] / max(kt["av_launches"], 1)
    atu_ms = kt["atu_ms"] / max(kt["atu_launches"], 1)
    traffic = None
    if os.path.exists(PROFILE_TRAFFIC) and args.level == 5:
        with open(PROFILE_TRAFFIC) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch_k_avp_c2:"):
                    traffic = float(line.split(":")[1])
    which = {"lsqr": "LSQR A*V sweep", "lsqr_block": "LSQR A*V sweep", "gmres": "GMRES A M^-1 v sweep"}.get(
        args.solver, "BiCGSTAB A D^-1 p / A D^-1 s sweeps")
    roofline = {"bound": "hbm", "kernel": f"k_avp ({which} over the packed symmetric 3x3 blocks, FP32, TMA, 8 RHS)",
                "achieved": a_bytes / (av_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                "frac": a_bytes / (av_ms * 1e-3) / 1e9 / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": a_bytes,
                "other_sweep": ({"kernel": "k_atup (A^T*U, packed, TMA)", "achieved": a_bytes / (atu_ms * 1e-3) / 1e9,
                                 "frac": a_bytes / (atu_ms * 1e-3) / 1e9 / peak} if atu_ms > 0 else None)}

    # end to end through the C ABI with host buffers (mesh upload + solve + R back)
    e2e_vals = []
    h2d = (m["xyz"].nbytes + m["etype"].nbytes + m["con"].nbytes + m["bcid"].nbytes +
           6 * 3 * len(m["xyz"]) * 8 + 2 * 4 + 2 * 8 + 6 * 4)
    d2h = 36 * 8 + 6 * 4 * 2 + 6 * 8
    for _ in range(args.e2e_steps):
        t2 = time.perf_counter()
        C2 = A.Context(local if world > 1 else 0)
        C2.set_mesh(m)
        C2.set_problem(A.STOKES, [1, 2], A.dirichlet_known(A.STOKES, 2), itri=5)
        set_solver(A, C2, args.solver, args)
        C2.resistance_tensor(A.MIXED, 1, 2, eps=args.eps)
        C2.close()
        e2e_vals.append(time.perf_counter() - t2)
    e2e = {"value": (world / statistics.median(e2e_vals)) if e2e_vals else None, "unit": "solves/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": len(e2e_vals)}

    # the other solvers of the same system, timed beside the headline: the
    # reference's column-scaled LSQR, the block-preconditioned LSQR and the LIS
    # path's solver (BiCGSTAB-Jacobi with FP64 true-residual restarts, LSQR for a
    # system where it does not converge)
    others = {}
    if args.lis_compare and rank == 0:
        truth = None
        if os.path.exists(GOLDEN_TRUTH):
            with open(GOLDEN_TRUTH) as f:
                g = json.load(f)
            if g.get("workload") == mesh_part(name):
                truth = np.array(g["R"])
        for other in ("lsqr", "lsqr_block", "hybrid", "gmres"):
            if other == args.solver:
                continue
            set_solver(A, C, other, args)
            ms_l, R_l, nit_l, ist_l = [], None, None, None
            for _ in range(args.lis_compare + 1):
                R_l, nit_l, info_l = C.resistance_tensor(A.MIXED, 1, 2, eps=args.eps)
                ms_l.append(info_l["device_ms"])
                ist_l = info_l["istop"]
            ms_med = statistics.median(ms_l[1:])
            others[other] = {"solver": solver_text(other, args.eps), "solves_per_s": 1000.0 / ms_med,
                             "ms_per_solve": ms_med,
                             "rel_err_vs_fp64": (float(np.max(np.abs(R_l - truth)) / np.max(np.abs(truth)))
                                                 if truth is not None else None),
                             "nit": [int(v) for v in nit_l], "istop": [int(v) for v in ist_l],
                             "steps": len(ms_l) - 1, "ratio_to_headline": (1000.0 / ms_med) / (value / world)}
        set_solver(A, C, args.solver, args)

    # assembly roofline: k_stokes_G<float, packed>, the regular quadrature of
    # every (collocation point, element) pair of the single layer; 28 flop per
    # (pair, quadrature point), an FMA counted as 2 and the rsqrt as 1:
    # r (3), r.r (5), rsqrt (1), w/r (1), 1/r^2 (1), w/r^3 (1), G accumulation
    # (1), w r_a / r^3 (2), six symmetric r_a r_b sums (12: five FMAs and a
    # multiply-add)
    asm_ms = kt["assemble_ms"] / max(kt["assemble_launches"], 1)
    q_pts = 126
    asm_flops = float(ne_sys) ** 2 * q_pts * STOKES_G_FLOPS_PER_POINT
    fp32_peak, fp32_kind = fp32_peak_tflops()
    roofline_asm = {"bound": "fp32", "kernel": "k_stokes_G<float, packed> (single-layer regular quadrature, "
                                               "ITRI 5: 126 points per pair)",
                    "flops_per_launch": asm_flops, "ms": asm_ms,
                    "achieved": asm_flops / (asm_ms * 1e-3) / 1e12 if asm_ms > 0 else None,
                    "peak": fp32_peak, "unit": "TFLOP/s", "peak_source": fp32_kind,
                    "frac": asm_flops / (asm_ms * 1e-3) / 1e12 / fp32_peak if asm_ms > 0 else None,
                    "flops_per_pair_point": STOKES_G_FLOPS_PER_POINT}

    # plain FP64 GPU comparator: FP64 assembly + FP64 LSQR to the same eps, to
    # convergence, timed in full on the device
    fp64 = None
    if args.fp64 == "full" and rank == 0:
        C.set_solver(A.SOLVER_LSQR)  # the FP64 path solves with LSQR
        C.kernel_times(reset=True)
        R64, nit64, info64 = C.resistance_tensor(A.FP64, 1, 2, eps=args.eps)
        kt64 = C.kernel_times(reset=True)
        err64 = None
        if os.path.exists(GOLDEN_TRUTH) and rel_err is not None:
            with open(GOLDEN_TRUTH) as f:
                Rt = np.array(json.load(f)["R"])
            err64 = float(np.max(np.abs(R64 - Rt)) / np.max(np.abs(Rt)))
        per_it = (kt64["av_ms"] + kt64["atu_ms"]) / max(kt64["av_launches"], 1)
        fp64 = {"solves_per_s": 1000.0 / info64["device_ms"], "device_ms": info64["device_ms"],
                "assemble_ms": info64["assemble_ms"], "nit": [int(v) for v in nit64],
                "istop": [int(v) for v in info64["istop"]], "ms_per_iteration_sweeps": per_it,
                "rel_err_vs_fp64_truth": err64,
                "ratio_mixed_over_fp64": value / world / (1000.0 / info64["device_ms"]),
                "how": "FP64 assembly (k_stokes_G<double>) + FP64 block LSQR (k_av2/k_atu2) to the same eps, "
                       "converged, CUDA events"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            ms_small, name_small = small_body(args.cpu_level, args.outer_level, args.outer_radius)
            runs = [cpu_complete_solve(ms_small, args.eps) for _ in range(max(1, args.cpu_solves))]
            cpu_s = statistics.median(r["seconds"] for r in runs)
            threads = os.cpu_count() or 1
            # the GPU on the same small body: mixed path, complete solves, device time
            Cs = A.Context(0)
            Cs.set_mesh(ms_small)
            Cs.set_problem(A.STOKES, [1, 2], A.dirichlet_known(A.STOKES, 2), itri=5)
            set_solver(A, Cs, args.solver, args)
            Cs.resistance_tensor(A.MIXED, 1, 2, eps=args.eps)
            gs, gR = [], None
            for _ in range(5):
                gR, _, gi = Cs.resistance_tensor(A.MIXED, 1, 2, eps=args.eps)
                gs.append(gi["device_ms"])
            Cs.set_solver(A.SOLVER_LSQR)
            R64s, _, g64 = Cs.resistance_tensor(A.FP64, 1, 2, eps=args.eps)
            Cs.close()
            Rc = runs[-1]["R"]
            cpu = {"value": 1.0 / cpu_s, "unit": "solves/s", "cores": threads, "kind": "port",
                   "sample": f"{len(runs)} complete solves (median) of {name_small}, LSQR eps {args.eps:g}, nothing "
                             f"scaled: integration on {threads} threads, the reference's serial CRS LSQR per "
                             f"right-hand side",
                   "seconds": cpu_s, "integration_s": runs[-1]["integration_s"], "nit": runs[-1]["nit"],
                   "same_body_gpu": {"mixed_solves_per_s": 1000.0 / statistics.median(gs),
                                     "fp64_solves_per_s": 1000.0 / g64["device_ms"],
                                     "ratio_mixed_gpu_over_cpu": cpu_s * 1000.0 / statistics.median(gs),
                                     "ratio_fp64_gpu_over_cpu": cpu_s * 1000.0 / g64["device_ms"],
                                     "rel_diff_fp64_gpu_vs_cpu": float(np.max(np.abs(R64s - Rc)) /
                                                                       np.max(np.abs(Rc))),
                                     "rel_diff_mixed_gpu_vs_cpu": float(np.max(np.abs(gR - Rc)) /
                                                                        np.max(np.abs(Rc)))}}
            cpu["single_thread"] = single_thread_leg(ms_small, args.eps)
            if args.c2_estimate and fp64 is not None:
                cpu["c2_estimate"] = cpu_c2_estimate(m, fp64["nit"], args.cpu_seconds)
        except Exception as ex:  # the baseline must not hide the GPU line
            cpu = {"value": None, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {ex}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (fp64 singular/free-term/reductions)",
                "data": "synthetic (meshes generated in-process)",
                "config": {"workload": name, "precision": "mixed", "solver": args.solver, "unknowns": C.n,
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "l2": "inputs larger than L2 (10.4 GB packed matrix), no flush"},
                "rel_err_vs_fp64": rel_err, "drag_over_analytic": drag_ratio, "torque_over_analytic": torque_ratio,
                "nit": [int(v) for v in nit], "e2e": e2e, "roofline": roofline, "roofline_assembly": roofline_asm,
                "cpu_baseline": cpu,
                "clocks": clk.summary(), "gpu_launches": kt["launches"] * world,
                "kernel_ms": {"assemble_single_layer": kt["assemble_ms"] / max(kt["assemble_launches"], 1),
                              "rhs": kt["rhs_ms"] / max(kt["rhs_calls"], 1), "av_sweep": av_ms,
                              "atu_sweep": atu_ms},
                "host_s": t1 - t0, "fp64_gpu": fp64, "other_solvers": others}
        print(json.dumps(line), flush=True)
    C.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
