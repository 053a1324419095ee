/*
 * andromeda_gb300 -- C ABI of the GB300-native BEM hot path (assembly of the
 * Laplace/Stokes influence matrices and their LSQR solve).
 *
 * Every entry point takes plain pointers and sizes, returns 0 (AGB_OK) on
 * success and a nonzero status otherwise; agb_last_error() then describes the
 * failure.  No exception and no CUDA/torch type crosses the boundary.  Arrays
 * are owned by the caller; the library copies what it needs.
 *
 * The entry points replace the following reference routines (Fortran,
 * src/ of WildSmilodon/Andromeda):
 *
 *   agb_set_mesh        mMesh module state built by ReadMesh, CalMeshArea
 *                       (lib_mesh.f90:956), CalMeshNormals (lib_mesh.f90:695) and
 *                       CalQMesh (lib_mesh.f90:577)
 *   agb_set_problem     subdomain/BC state of ReadsdBIC + SetUpSubdomains
 *                       (lib_sdBem.f90:319) + sdSetUpXandB (lib_sdBem.f90:4) and
 *                       StokesBigSystemXB (lib_Stokes.f90:1180); the ITRI/IQUD
 *                       rules of ReadParameters (mod_par.f90:230-234)
 *   agb_assemble        CoR_Integrals (lib_int.f90:4) / CoR_Integrals_Stokes
 *                       (lib_Stokes.f90:2664) fused with the BC routing of
 *                       sdSetUpSysMrhsM_CRS (lib_CRS.f90:148) /
 *                       stokesFormCRSsysMrhsM (lib_Stokes.f90:475) and the column
 *                       scaling lsqr_precon (lib_lsqr.f:131); the system matrix
 *                       stays resident on the GPU
 *   agb_rhs             formStokesLeftRightHandSideVectors (lib_StokesFull.f90:379)
 *                       + CRSxV(rhsM, b) (lib_CRS.f90:764); Laplace: CRSxV(rhsM,-b)
 *   agb_solve           lsqr_solve (lib_lsqr.f:33) for nrhs right-hand sides in
 *                       one block solve, + StokesDistributeUnknowns
 *                       (lib_StokesFull.f90:446) numbering of the result
 *   agb_force_torque    getForceIntegrateFluxes / getTorqueIntegrateFluxes
 *                       (lib_particle.f90:1751,1793)
 *   agb_resistance_tensor  the 3-sides resistance workflows
 *                       StokesInlet3sidesForceCRS / ...TorqueOmegaCRS
 *                       (lib_particle.f90:341,176) as one 6-RHS solve
 *   agb_lsqr_precon     lsqr_precon(m,n,nnz,q,ia,ja,a)      (lib_lsqr.f:131)
 *   agb_lsqr_solve      lsqr_solve(m,n,nnz,maxit,eps,nit,ierr,q,ia,ja,a,b,x)
 *                                                           (lib_lsqr.f:33)
 */
#ifndef ANDROMEDA_GB300_H
#define ANDROMEDA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct agb_context agb_context;

/* status codes */
#define AGB_OK 0
#define AGB_ERR_ARG 1
#define AGB_ERR_CUDA 2
#define AGB_ERR_STATE 3
#define AGB_ERR_UNSUPPORTED 4
#define AGB_ERR_NUMERIC 5

/* problem kinds (PRTY of and.inp) */
#define AGB_LAPLACE 1
#define AGB_STOKES 2

/* precision of the assembled system */
#define AGB_FP64 0  /* everything FP64 (the reference's arithmetic) */
#define AGB_MIXED 1 /* FP32 regular quadrature + FP32 matrix; FP64 singular
                       integrals, free-term row sums, norms/recurrences and
                       the refinement residual */
#define AGB_MATRIX_FREE 2 /* AGB_MIXED arithmetic without a stored matrix: every
                       LSQR sweep recomputes the single-layer entries (Stokes,
                       velocity known on every wall, triangles; zero warm start) */

/* solver of the assembled system (agb_set_solver; the SLET key of and.inp) */
#define AGB_SOLVER_LSQR 0     /* lsqr_solve with lsqr_precon's column scaling (SLET CRS) */
#define AGB_SOLVER_BICGSTAB 1 /* BiCGSTAB with the Jacobi preconditioner (SLET LIS with the
                                 reference's default LIS options) */
#define AGB_SOLVER_HYBRID 2   /* BiCGSTAB-Jacobi first; LSQR (as AGB_SOLVER_LSQR, zero start,
                                 the reference's default iteration limit) for every right-hand
                                 side of a system whose BiCGSTAB did not converge on all of them
                                 (no counterpart in the reference) */
#define AGB_SOLVER_LSQR_BLOCK 3 /* LSQR (lsqr_solve's recurrence and stopping tests) on A M^-1
                                   with M the elements' 3x3 self blocks (block-Jacobi right
                                   preconditioner) in place of lsqr_precon's column scaling;
                                   packed mixed system only, also in agb_batch_resistance
                                   (no counterpart in the reference) */
#define AGB_SOLVER_GMRES 4      /* restarted GMRES (SLET LIS with the LIS options "-i gmres
                                   -restart m", the restart length set by agb_set_gmres_restart,
                                   default 40 as LIS) with the 3x3 self-block right
                                   preconditioner; packed mixed system only */

/* boundary-condition types (mod_mesh.f90:110) */
#define AGB_BC_FUNCTION 1
#define AGB_BC_FLUX 2
#define AGB_BC_CONTACT 3

/* Library version string. */
const char* agb_version(void);

/* Create a context bound to CUDA device `device` (one stream per context). */
int agb_create(agb_context** ctx, int device);
int agb_destroy(agb_context* ctx);
/* Text of the last failure on this context ("" if none).  ctx may be NULL for
 * the context-free entry points (agb_lsqr_*), whose last error is per thread. */
const char* agb_last_error(const agb_context* ctx);

/* Mesh.  xyz: 3*nnodes doubles (node-major: x,y,z of node 0, then node 1 ...).
 * etype: 2 = 3-node triangle, 3 = 4-node quad.  con: 4*nelem 0-based node ids
 * (4th entry ignored for triangles).  bcid: wall id of each element.
 * Rejected with AGB_ERR_ARG before the context is used (so with ctx NULL the
 * message is in agb_last_error(NULL)): a coordinate that is not finite,
 * connectivity out of range, an unknown element type, and a degenerate element
 * (nodes 1-3, which give the element normal as in CalElementNormal,
 * lib_mesh.f90:716, coincident or collinear to rounding: the normal shorter
 * than 1e-12 of the product of the two edges). */
int agb_set_mesh(agb_context* ctx, int nnodes, const double* xyz, int nelem, const int* etype, const int* con,
                 const int* bcid);

/* One subdomain made of `nwalls` walls (ids `walls`), normal multipliers
 * normMul (NORMMUL of the .bic file, 1.0 by default), diffusivity/viscosity
 * diff, and known[en*nwalls + k] = BC type of equation en (0 for Laplace;
 * 0,1,2 = x,y,z for Stokes) on wall walls[k].  itri = 1..5 (triangle rule),
 * iqud = 1..8 (Gauss rule index for quads). */
int agb_set_problem(agb_context* ctx, int kind, int nwalls, const int* walls, const double* normMul, double diff,
                    const int* known, int itri, int iqud);

/* Walls of the subdomain's nodes as the driver placed them: the reference's
 * subdomain%BCidList after the BiC file's EDGE / CORNER directives
 * (HandleCornersEdges, lib_sdBem.f90:112-310), which move a node shared by
 * walls of different boundary conditions to a named wall.  Without this call a
 * node takes the wall of the last element touching it in subdomain order, the
 * reference's assignment before those directives (SetUpSubdomains,
 * lib_sdBem.f90:388-394).  node_wall[i] = the wall id (bcid) of global node i,
 * or < 0 to keep that assignment; NULL restores it for every node.  Every id
 * must be a wall of the problem.  Call after agb_set_problem (agb_set_mesh and
 * agb_set_problem reset it); an assembled system is released, as its numbering
 * changes.  Only the general path (some wall with a known flux) sees the node
 * walls: with every value known, all walls route alike. */
int agb_set_node_walls(agb_context* ctx, int nnodes, const int* node_wall);

/* Integration options of the triangle integrals (default: sing_mode 0,
 * near_eta 0 -- the reference's assembly).  Replaces the commented-out
 * alternative of sdIntRowU/Q and sdIntRowU/QStokes (lib_sdBem.f90:510,668;
 * lib_Stokes.f90:1697,2030) and parTriRecur (mod_par.f90:232):
 *   sing_mode 0: analytic self-element integrals (si_tri_lap / si_tri_stk);
 *   sing_mode 1: recursive midpoint subdivision toward the source, rec_depth
 *                levels (Triangle_BEMInt lib_sdBem.f90:775, Triangle_StokesInt
 *                lib_Stokes.f90:2251); rec_depth 0..30; a quad's own node or
 *                centre by the polar Gauss scheme of the singular branch of
 *                Quad_BEMInt / Quad_StokesInt (lib_int.f90:408,
 *                lib_Stokes.f90:3494) with the problem's quad rule iqud (the
 *                reference's parQuadIntegSing, default 4 as parQuadIntegRegu);
 *   near_eta > 0, near_depth 1..20: adaptive near-singular rule for the other
 *                triangles (no reference counterpart): a (sub-)triangle whose
 *                centroid is closer to the source than near_eta x its longest
 *                edge is split into its four midpoint children, up to near_depth
 *                levels, all in FP64.
 * Non-default options send agb_assemble through the general FP64 assembly
 * (for AGB_MIXED the routed system is then copied to FP32).  Call after
 * agb_set_problem; it clears the assembled system. */
int agb_set_integration(agb_context* ctx, int sing_mode, int rec_depth, double near_eta, int near_depth);

/* Solver of agb_solve / agb_resistance_tensor (the SLET key, mod_par.f90):
 * AGB_SOLVER_LSQR (default; lsqr_solve, lib_lsqr.f:33) or AGB_SOLVER_BICGSTAB,
 * the LIS path's solver (StokesBigSystemSOLVElis lib_StokesLis.f90:4 with the
 * default options "-i bicgstab -p jacobi", mod_par.f90:288): every equation in
 * the row of its own unknown, preconditioned BiCGSTAB (van der Vorst 1992) with
 * M = diag(A), x0 = 0 (the warm start is not used), stop at
 * ||b - A x|| <= eps ||b|| or maxit iterations (0: 1000, the LIS default).  With
 * BiCGSTAB, istop[r] is 0 converged, 1 iteration limit, 2 breakdown, 3 diverged
 * or stagnated (the recursive residual rose 1e3 times above its best, or did
 * not fall by 10 % in 64 iterations: the FP32 products of an ill-conditioned
 * system), 4 the true residual stayed above eps.  The recursive residual of the
 * FP32 products can drift from the true one, so after BiCGSTAB stops the true
 * residual b - A x is formed with FP64 accumulation, and a right-hand side
 * whose true residual is above eps ||b|| is solved again from x on that
 * residual (FP64 refinement, at most 4 restarts).  AGB_SOLVER_HYBRID: as BiCGSTAB where every right-hand side of the
 * system converges; otherwise all of them are solved again by LSQR and
 * istop[r] = 10 + LSQR's istop, nit[r] the sum of both iteration counts.  BiCGSTAB
 * needs the packed mixed system (Stokes, velocity known on every wall,
 * triangles, default integration, AGB_MIXED); other systems return
 * AGB_ERR_UNSUPPORTED from the solve.  agb_batch_resistance on this context
 * solves its bodies with BiCGSTAB too (istop as above, with the same FP64
 * true-residual check and restarts, batched over the bodies that need them;
 * AGB_SOLVER_HYBRID re-solves by LSQR every body with a right-hand side that
 * does not end at 0; no autotuning). */
int agb_set_solver(agb_context* ctx, int solver);

/* AGB_SOLVER_GMRES (the LIS path with "-i gmres", lis_solver_set_option at
 * mod_plis.f90:235 taking the options of mod_par.f90:418): restarted GMRES(m)
 * (Saad and Schultz 1986) on A M^-1, M the elements' 3x3 self blocks, x0 = 0,
 * stop at ||b - A x|| <= eps ||b|| or maxit Arnoldi steps (0: 1000, the LIS
 * default).  A cycle's steps run until the residual estimate is below
 * eps/2 ||b|| (with FP32 products the estimate runs ahead of the true
 * residual); at the end of every cycle the true residual is formed over the
 * stored matrix (agb_set_residual_mode) and decides: within eps the
 * right-hand side is done, otherwise the next cycle starts from it.  istop[r]:
 * 0 converged (by the true residual), 1 iteration limit, 3 a cycle that did
 * not lower the true residual by 10 %.  restart = m, 1..512 (default 40, the
 * LIS default). */
int agb_set_gmres_restart(agb_context* ctx, int restart);

/* Arithmetic of the true residual b - A x over the packed FP32 single layer
 * (GMRES and BiCGSTAB restarts, refinement, LSQR warm starts): 0 (default)
 * float-float products and sums on the FP32 pipe (TwoSum, flushed into FP64
 * every 256 terms; within about 2^-33 of sum |a_ij x_j| of the exact residual
 * in the worst case, below 2^-44 with random rounding),
 * 1 FP64 products and sums (the FP64 pipe, ~10x slower on this part). */
int agb_set_residual_mode(agb_context* ctx, int mode);

/* Element geometry in global element order (normal 3*nelem, area nelem,
 * centroid 3*nelem); elements outside the subdomain are zero. */
int agb_get_geometry(agb_context* ctx, double* normal, double* area, double* centroid);

/* Size of the assembled system: m rows (equations), n unknowns.  For the
 * all-Dirichlet problems m == n == nelem (Laplace) or 3*nelem (Stokes), in the
 * reference numbering: rows source-major/component-minor, unknowns
 * component-major (x of every element, then y, then z). */
int agb_system_size(agb_context* ctx, int* m, int* n);

/* Assemble the system matrix on the GPU in the given precision and apply the
 * reference's column scaling (lsqr_precon).  Walls with known function values
 * only, triangles (Stokes) / FP64 (Laplace): fused single-layer assembly of the
 * used rows.  Any other case (known fluxes, contact, Stokes quads, mixed
 * Laplace): every source row in FP64 + BC routing (general path); AGB_MIXED
 * then stores the routed system in FP32. */
int agb_assemble(agb_context* ctx, int precision);

/* Copy the assembled system to the host (m x n row-major), with (scaled=1) or
 * without (scaled=0) the column scaling; and the scaling q (n) if not NULL. */
int agb_get_system(agb_context* ctx, int scaled, double* A, double* q);

/* Right-hand sides for nrhs known nodal fields u[r][en][nnodes]:
 * rhs[r][m] = rhsM * b (Stokes) / rhsM * (-b) (Laplace). */
int agb_rhs(agb_context* ctx, int nrhs, const double* u, double* rhs);

/* Solve for nrhs fields at once.  x[r][n] holds the warm start on entry (the
 * reference warm-starts from the previous solution) and the unknowns on exit.
 * maxit = 0 -> 10*(m+n+50); eps as the SOLVER line.  refine = number of
 * iterative-refinement passes after the solve (no counterpart in the
 * reference): each computes r = b - A x with FP64 accumulation over the stored
 * matrix, solves A d = r by LSQR from zero to the relative tolerance 1e-2 and
 * sets x += d (LSQR solves only).  nit[r] counts every LSQR iteration, istop[r]
 * is that of the first solve; per right-hand side. */
int agb_solve(agb_context* ctx, int nrhs, const double* u, double* x, int maxit, double eps, int refine, int* nit,
              int* istop);

/* Force (3) and torque (3, about the origin) of the tractions x[r][n] on the
 * elements of wall `wall`: ft[r][6]. */
int agb_force_torque(agb_context* ctx, int nrhs, const double* x, int wall, double* ft);

/* Resistance tensor of the body on `particle_wall` inside the container
 * `outer_wall`: assembles (precision), imposes the six rigid motions on the
 * container (unit translations e_x,e_y,e_z, then rotations e_i x r), solves the
 * six right-hand sides in one block LSQR and integrates force and torque on
 * the particle.  R[r][6] = (F, T) of motion r; nit[6], istop[6] per motion
 * (istop > 3: iteration or condition limit -- reported, not an error, as the
 * reference only logs it).  times_ms (may be NULL, 6 doubles): host
 * {assemble, rhs, solve, reduce, total} and [5] the device time of the whole
 * call between two CUDA events on the context stream. */
int agb_resistance_tensor(agb_context* ctx, int precision, int particle_wall, int outer_wall, int maxit, double eps,
                          int refine, double* R, int* nit, int* istop, double* times_ms);

/* Live kernel timing (instrumentation; plays the role of the reference's
 * TIMER stopwatches, stokes.f90:88-92, at kernel granularity).  Cumulative
 * CUDA-event times on the context stream since the last reset:
 * out[0] ms in the A*V sweep, out[1] its launches, out[2] ms in the A^T*U
 * sweep, out[3] its launches, out[4] ms in the Stokes single-layer assembly
 * kernel, out[5] its launches, out[6] ms building right-hand sides, out[7]
 * its calls, out[8] number of kernels this library launched, out[9] = 0
 * (reserved).  out holds 10 doubles.  reset != 0 zeroes the counters after
 * reading. */
int agb_kernel_times(agb_context* ctx, int reset, double* out);

/* Self-test of the bounded barrier wait of the TMA-fed kernels (no counterpart
 * in the reference; it tests this library's failure path).  One CTA of 32
 * threads waits on the first phase of an mbarrier with the kernels' wait
 * function and a limit of `polls` failed tries (1..2^22).  arrive = 0: nothing
 * arrives and no copy is issued, the wait gives up, sets the launch's error
 * word and returns; the call returns AGB_ERR_CUDA with "a bounded barrier wait
 * gave up" in agb_last_error(NULL), as a solve whose wait gave up does, and the
 * device stays usable.  arrive = 1: one thread arrives, every wait completes,
 * AGB_OK.  *waits_completed: threads whose wait completed (0 or 32). */
int agb_selftest_bounded_wait(int device, unsigned polls, int arrive, int* waits_completed);

/* Drop-ins with the reference signatures (1-based CRS, int64 row pointers).
 * agb_lsqr_precon scales a in place like lsqr_precon; agb_lsqr_solve
 * warm-starts from x like lsqr_solve.  Both run on the current CUDA device. */
int agb_lsqr_precon(int m, int n, int64_t nnz, double* q, const int64_t* ia, const int* ja, double* a);
int agb_lsqr_solve(int m, int n, int64_t nnz, int* maxit, double eps, int* nit, int* ierr, const double* q,
                   const int64_t* ia, const int* ja, double* a, const double* b, double* x);

/* Integral matrices of every source row -- the drop-in of CoR_Integrals
 * (lib_int.f90:4, sdFormIntegralMatrices :225) and CoR_Integrals_Stokes
 * (lib_Stokes.f90:2664, sdFormIntegralMatricesStokes :1391), FP64 on the GPU:
 * rows = the nn u-source points (subdomain nodes, ascending) then the nq
 * q-source points (element centroids, subdomain order); free terms included.
 * Each component matrix is column-major nsp x ncol like Hmat(nsp,nnodes).
 * Laplace: T = H (1 matrix, ncol = nn), G (1, ncol = nq).  Stokes: T = 9
 * matrices Txx,Txy,Txz,Tyy,Tyz,Tzz,prTx,prTy,prTz; G = 9 matrices
 * Gxx,Gxy,Gxz,Gyy,Gyz,Gzz,prGx,prGy,prGz.  errs[2] = the reference's fSP/qSP
 * self-check residuals (max over u-rows, over q-rows). */
int agb_integral_matrices(agb_context* ctx, double* T, double* G, double* errs);

/* Surface pressure of a solved Stokes field (pressureStokes, lib_Stokes.f90:4-94):
 * p at the centroid of every element of the subdomain (mesh order; 0 for an
 * element of no subdomain wall) from the pressure rows of the q-source points
 * (sdIntRowQStokes, lib_Stokes.f90:1562, self element left out as the
 * reference's analytic branch does) contracted with the velocity u[3][nnodes]
 * less the element's centre velocity and the traction q[3][nelem], times
 * -2 / (8 pi).  FP64. */
int agb_surface_pressure(agb_context* ctx, const double* u, const double* q, double* p);

/* Values at npts points inside the domain (GetStokesDomainValue,
 * lib_Stokes.f90:3043; GetSubDomainValue, lib_domain.f90:210) from the boundary
 * values u[neq][nnodes] and fluxes/tractions q[neq][nelem]: Stokes
 * out[4k..4k+3] = velocity, pressure; Laplace out[k].  err[k] is the
 * reference's check of the point (Stokes: stresslet diagonal against 8 pi and
 * sum G.n; getStokesDV treats err > 1e-2 as outside; Laplace: VerifyIntegrals).
 * Triangles with the problem's integration options, quads as one Gauss cell
 * (the regular branch of Quad_StokesInt / Quad_BEMInt).  FP64. */
int agb_domain_values(agb_context* ctx, int npts, const double* pts, const double* u, const double* q, double* out,
                      double* err);

/* ---- file formats of the reference (host code, no GPU work; errors via
 * agb_last_error(NULL)) ---------------------------------------------------- */

/* Surface mesh as ReadMesh reads it (lib_meshRead.f90:80-160): gmsh 2.x ASCII
 * (ReadGMSHv2 :244), gmsh 4.x ASCII (ReadGMSHv4Surface :385; element blocks of
 * a dimension other than 2 are skipped, where the reference refuses a gmsh 4
 * file whose entities include volumes) or the reference's "andromedaMesh" text
 * (ReadAndromedaMesh :165).  Lines are read as rOneTL (lib_mesh.f90:1804)
 * reads them: blank lines and lines holding '#' are skipped.  Node and element
 * tags give the positions (node(j), element(j)).  Call with xyz == NULL to get
 * sizes = {nnodes, nelem, nwalls}; then with arrays of those sizes: xyz
 * 3*nnodes, etype/bcid nelem, con 4*nelem (0-based, -1 as the 4th node of a
 * triangle: the layout of agb_set_mesh), wall_ids nwalls and wall_names
 * nwalls x name_len bytes (NUL-padded; both may be NULL).  Element types other
 * than 2/3 and node tags out of range are AGB_ERR_ARG (the reference stops). */
int agb_mesh_read(const char* path, int* sizes, double* xyz, int* etype, int* con, int* bcid, int* wall_ids,
                  char* wall_names, int name_len);

/* ParaView result file (OutputMeshParaview, lib_mesh.f90:218-392): ASCII VTK
 * UnstructuredGrid with point data u (3-vector for Stokes), node, u<name> per
 * equation; cell data normale, pressure (Stokes), elemBCid, q<name>; points and
 * cells (VTK types 5 triangle / 9 quad).  u [neq][nnodes], q [neq][nelem],
 * normal [nelem][3], p [nelem] (Stokes; NULL for Laplace), names: neq equation
 * names (x, y, z for Stokes). */
int agb_vtu_write(const char* path, int kind, int nnodes, const double* xyz, int nelem, const int* etype,
                  const int* con, const int* bcid, const double* normal, int neq, const char* const* names,
                  const double* u, const double* q, const double* p);

/* The integral-matrix cache and.integrals.bin (WriteIntegralsToDisk /
 * ReadIntegralsFile lib_int.f90:136-221; WriteIntegralsToDiskStokes /
 * ReadIntegralsFileStokes lib_Stokes.f90:2742-2876) in the record layout
 * gfortran writes for FORM='UNFORMATTED' sequential files, one subdomain:
 * [Stokes: parStokes = 1407], (nsp, nnodes, nqnodes), (FspCerr, QspCerr), then
 * the matrices column by column in records of at most 8192 values (WrSMat,
 * lib_util.f90:201) -- Laplace H, G; Stokes Txx,Tyy,Tzz,Txy,Txz,Tyz,
 * Gxx,Gyy,Gzz,Gxy,Gxz,Gyz, prTx..z, prGx..z.  T and G are laid out as
 * agb_integral_matrices returns them.  Reading: with T == NULL only sizes and
 * errs are returned; otherwise sizes must equal the file's (the reference's
 * check, lib_int.f90:152-157). */
int agb_integrals_file_write(const char* path, int kind, int nsp, int nnodes, int nqnodes, const double* errs,
                             const double* T, const double* G);
int agb_integrals_file_read(const char* path, int kind, int* sizes, double* errs, double* T, double* G);

/* Sizes of the subdomain numbering: {nsp, nn, nq, rows, unknowns, knowns}. */
int agb_layout_sizes(agb_context* ctx, int* sizes);

/* Solve with any boundary-condition mix of the subdomain (sdSolveCRS
 * lib_CRS.f90:4 / StokesBigSystemSOLVEcrs lib_Stokes.f90:417 +
 * StokesDistributeUnknowns lib_StokesFull.f90:446): u_in[r][neq][nnodes] and
 * q_in[r][neq][nelem] (may be NULL = 0) hold the known values and the warm
 * start of the unknowns; u_out/q_out receive the fields with the unknowns
 * filled in.  Works after agb_assemble on either assembly path. */
int agb_solve_fields(agb_context* ctx, int nrhs, const double* u_in, const double* q_in, double* u_out,
                     double* q_out, int maxit, double eps, int refine, int* nit, int* istop);

/* Allocation-free column scaling for callers that cannot call cudaMalloc (a
 * host program that owns all device memory through its own pool or an
 * OpenACC runtime, code in an allocation-free phase, an embedding whose device
 * memory is fully reserved).  No counterpart in the reference: it is the
 * lsqr_precon column scaling (q_j = 1/||A(:,j)||, A <- A diag(q)) applied to a
 * dense row-major m x n matrix the caller already holds on the current device
 * (leading dimension lda >= n, FP64), writing q (n doubles, device).  It
 * allocates nothing: its scratch is a fixed 8 MiB array in the library's
 * device image (held by every GPU that loads the library until exit), so n is
 * limited to AGB_NOALLOC_MAX_COLUMNS and larger n is rejected with
 * AGB_ERR_ARG.  The first call in each CUDA context (per device, and again
 * in a context re-created after cudaDeviceReset or in a non-primary context
 * made current by the host) looks up the array's device address (make it
 * before any stream capture).  All calls on a device share the array:
 * calls that overlap on the GPU race on it.  Runs on the legacy default stream
 * and returns after the work is done; errors via agb_last_error(NULL). */
#define AGB_NOALLOC_SCRATCH_DOUBLES (1 << 20)
#define AGB_NOALLOC_MAX_COLUMNS AGB_NOALLOC_SCRATCH_DOUBLES
int agb_lsqr_precon_dense_noalloc(int m, int n, int64_t lda, double* A, double* q);

/* Batched resistance tensors (many bodies of uneven size, one container each).
 * Body i is nodes node_off[i]..node_off[i+1]-1 of xyz (3 doubles per node)
 * and elements elem_off[i]..elem_off[i+1]-1 of etype/con/bcid (con: 4 ints per
 * element, 0-based node ids LOCAL to the body; triangles only), with the wall
 * ids particle_wall and outer_wall.  For every body the reference's 6-RHS
 * resistance workflow (StokesInlet3sidesForceCRS / ...TorqueOmegaCRS,
 * lib_particle.f90:341,176; CoR_Integrals_Stokes lib_Stokes.f90:2664;
 * lsqr_solve lib_lsqr.f:33) is run in mixed precision: R[36*i + 6*r + j] is
 * component j (Fx,Fy,Fz,Tx,Ty,Tz) on the particle for rigid motion r of the
 * container; nit/istop: 6 per body.  Bodies are assembled per body (the
 * single layer as packed symmetric 3x3 blocks, FP32) and solved together in
 * waves that fit mem_gb of device memory (0: 80 % of the free memory): every
 * LSQR sweep of a wave is one launch over the tiles of all of its bodies,
 * replayed from a CUDA graph; autotune != 0 times the candidate tile shapes on
 * the first wave.  stats (16 doubles, may be NULL): host ms of assembly+rhs,
 * solve, total; waves; device ms and launches of the A*V and A^T*U sweeps;
 * algorithmic bytes of all A*V launches; kernel launches; chosen block rows
 * per A*V CTA, per A^T*U stage and per A^T*U row group; graph iterations;
 * device ms of the whole call; host ms of the force/torque step.  ctx only carries the
 * device and the error text (its own mesh/problem are untouched).  Each body's
 * mesh is checked like agb_set_mesh's before the context is used. */
int agb_batch_resistance(agb_context* ctx, int nbodies, const int* node_off, const double* xyz, const int* elem_off,
                         const int* etype, const int* con, const int* bcid, int particle_wall, int outer_wall,
                         int itri, int maxit, double eps, double mem_gb, int autotune, double* R, int* nit,
                         int* istop, double* stats);

/* Direct solver of the FULL path (LINPACK LU, FP64, on the GPU).
 * agb_form_pre_fm replaces FormPREfm(pret,neq,q,a,cpu,ierr) (lib_solveFM.f:102):
 *   pret 0 none; 1 diagonal, q = 1/a(i,i) (frmdiafm); 2 LU with partial pivoting
 *   (dgefa, lib_solveFM.f:198) of the column-major neq x neq matrix a in place,
 *   q = 1-based pivot rows as doubles, ierr = index of the first zero pivot or 0.
 *   The pivots are dgefa's (same elimination order and tie rule); the factors
 *   are stored in LAPACK form (positive multipliers, later interchanges applied
 *   to L) and are meant for agb_solv_eqn_fm only.  cpu += elapsed seconds.
 * agb_solv_eqn_fm replaces SolvEQNfm(slvt,pret,prep,maxit,stopt,eps,neq,q,a,b,
 *   x,nit,cpu,ierr) (lib_solveFM.f:3): slvt 0 (direct) only; b = 0 gives x = 0,
 *   nit = 0; prep 1 factors inside (as FormPREfm), prep 2 uses a/q from
 *   agb_form_pre_fm; x = A^-1 b (dgesl, lib_solveFM.f:318).  maxit, stopt and eps
 *   are ignored by the direct solver, as in the reference.
 * agb_solve_lu: the same direct solve for the context's assembled FP64 square
 *   system (the FULL path after CoR_Integrals: lib_StokesFull.f90:566-570,
 *   lib_particle.f90:549,614): factors the unscaled system once per assembly,
 *   then solves nrhs fields given as in agb_solve; x has agb_solve's layout;
 *   info = first zero pivot or 0. */
int agb_form_pre_fm(int pret, int neq, double* q, double* a, float* cpu, int* ierr);
int agb_solv_eqn_fm(int slvt, int pret, int prep, int maxit, int stopt, double eps, int neq, double* q, double* a,
                    const double* b, double* x, int* nit, double* cpu, int* ierr);
int agb_solve_lu(agb_context* ctx, int nrhs, const double* u, double* x, int* info);

/* MLP surrogate of the resistance tensor (no reference counterpart; the
 * learned part of the many-body workflow): nin -> nhidden -> nhidden -> nhidden
 * -> nout with SiLU, FP32 master weights, BF16 tensor-core GEMMs with FP32
 * accumulation (split-BF16 hi+lo products on request), Adam.  Inputs and
 * outputs are row-major float arrays (n x nin, n x nout) in physical units; the
 * network works on (x - x_mean)/x_std and predicts (y - y_mean)/y_std.
 * Parameters (agb_mlp_get/set_params, agb_mlp_gradient): W1 [nh][nin], b1,
 * W2 [nh][nh], b2, W3 [nh][nh], b3, W4 [nout][nh], b4, concatenated.
 * agb_mlp_gradient: one forward + backward of the mean squared normalised
 * error on n rows (split != 0: split-BF16 products); gradient and loss out.
 * agb_mlp_train: epochs over n rows in shuffled mini-batches (full batches
 * only), loss_hist[epoch] = mean squared normalised error; stats[3]: device ms,
 * kernel launches, Adam steps so far.  agb_mlp_predict: split 1 = split-BF16
 * products in one fused kernel on the 5th-generation tensor cores (128
 * queries per CTA, accumulators in tensor memory, activations kept on chip;
 * needs nhidden = 256, nin <= 16, nout <= 32), split 2 = split-BF16 through
 * the layer-by-layer GEMMs of the training forward (same results), split 0 =
 * plain BF16 products; device_ms = kernel time of the n inferences. */
typedef struct agb_mlp agb_mlp;
int agb_mlp_create(agb_mlp** out, int device, int nin, int nhidden, int nout, unsigned long long seed);
int agb_mlp_destroy(agb_mlp* m);
int agb_mlp_num_params(agb_mlp* m, long long* n);
int agb_mlp_get_params(agb_mlp* m, float* p);
int agb_mlp_set_params(agb_mlp* m, const float* p);
int agb_mlp_set_normalization(agb_mlp* m, const float* x_mean, const float* x_std, const float* y_mean,
                              const float* y_std);
int agb_mlp_gradient(agb_mlp* m, int n, const float* X, const float* Y, int split, float* grad, double* loss);
int agb_mlp_train(agb_mlp* m, int n, const float* X, const float* Y, int epochs, int batch, float lr,
                  unsigned long long seed, double* loss_hist, double* stats);
int agb_mlp_predict(agb_mlp* m, int n, const float* X, float* Y, int split, double* device_ms);
long long agb_mlp_launches(agb_mlp* m);

#ifdef __cplusplus
}
#endif
#endif /* ANDROMEDA_GB300_H */
