// Batched block LSQR: many Stokes single-layer systems of uneven size (packed
// symmetric-block FP32 layout), each with up to 8 right-hand sides, solved together -- every sweep of an iteration is ONE
// launch over the tiles of all systems still iterating, and the iterations are
// replayed from one captured CUDA graph.
#pragma once
#include "agb_lsqr.cuh"
#include <string>
#include <vector>

namespace agb {

// One system of the batch (device pointers, owned by the caller).
struct BatchBody {
  const float* A = nullptr;   // packed symmetric 3x3 blocks (pk_idx layout), unscaled
  int pk_ne = 0, pk_ldp = 0;  // block rows = block columns; columns per plane (multiple of 64, >= pk_ne)
  int m = 0, n = 0;           // 3 pk_ne each
  int64_t lda = 0;            // length of the column vectors: multiple of 32, >= n
  const double* b = nullptr;  // [k][m] right-hand sides
  const double* q = nullptr;  // [n] lsqr_precon column scales (applied on the fly)
  double* x = nullptr;        // [k][n] solution (zero warm start)
};

// Tile shapes and schedule of the batched sweeps (picked by batch_autotune).
struct BatchTune {
  int atup_rows = 1024;    // block rows per A^T*U row group
  int check_every = 8;     // iterations per graph replay
};

struct BatchStats {
  double av_ms = 0.0, atu_ms = 0.0;  // summed device time of the two sweeps (CUDA events in the graph)
  long av_launches = 0, atu_launches = 0;
  long launches = 0;                 // all kernels launched
  long iterations = 0;               // graph iterations run (max over systems)
  double bytes_av = 0.0;             // algorithmic bytes of the timed A*V launches (LSQR, BiCGSTAB: all of
                                     // them; GMRES: the first of every cycle): sum over the systems
                                     // each covered of 6 pk_ne^2 x 4
  int av_rows = 0, atu_rs = 0, atu_rows = 0;  // tile shapes used: block rows per A*V CTA, per A^T*U
                                              // stage, per A^T*U row group
  long cycles = 0;                   // GMRES restart cycles run
};

// Solves A_i x_i = b_i (least squares) for all systems with the reference's
// lsqr_solve semantics (zero warm start, atol = btol = eps, conlim 1e8,
// itnlim = maxit or 10(m+n+50)); nit/istop receive k entries per system.
bool batch_lsqr_solve(const std::vector<BatchBody>& bodies, int k, double eps, int maxit, const BatchTune& tune,
                      cudaStream_t s, std::vector<int>& nit, std::vector<int>& istop, BatchStats* st,
                      std::string& err, bool bj = false);

// BiCGSTAB with the Jacobi preconditioner (the solver of the reference's LIS path,
// as DenseLsqr::bicgstab) on all systems together: x0 = 0, stop at
// ||b - A x|| <= tol ||b|| or maxit iterations (0: 1000).  b: [k][m] in the row
// numbering 3i+a; x: [k][n] in the unknown numbering a ne + i (as
// batch_lsqr_solve).  status per column: 0 converged, 1 iteration limit, 2
// breakdown, 3 diverged or stagnated, 4 converged by the recursive residual but
// not by the FP64 true residual.  tol_cols (null, or [nb][k]): a tolerance per
// right-hand side in place of tol (the restarts on the true residual solve each
// correction to its own column's tolerance).
bool batch_bicgstab_solve(const std::vector<BatchBody>& bodies, int k, double tol, int maxit, cudaStream_t s,
                          std::vector<int>& nit, std::vector<int>& status, BatchStats* st, std::string& err,
                          const std::vector<double>* tol_cols = nullptr);

// Restarted GMRES(restart) with the 3x3 self-block right preconditioner on all
// systems together (as DenseLsqr::gmres per system): x0 = 0, stop at the FP64-
// accurate true residual ||b - A x|| <= tol ||b|| (formed in float-float form
// at the end of every cycle) or maxit Arnoldi steps (0: 1000).  b, x as
// batch_lsqr_solve.  status per column: 0 converged, 1 iteration limit, 3 a
// cycle without a 10 % gain of the true residual.
bool batch_gmres_solve(const std::vector<BatchBody>& bodies, int k, double tol, int maxit, int restart,
                       cudaStream_t s, std::vector<int>& nit, std::vector<int>& status, BatchStats* st,
                       std::string& err);

// Times the candidate row groups of the A^T*U sweep on these systems (a few
// launches each, CUDA events) and returns the fastest; `report` lists the
// candidates and their times.  Results are cached per (systems, total size)
// class for the process.
// r = b - A x for every system (FP64 products and sums over the FP32 packed
// blocks; A, b, x as in BatchBody), written to r_out[i] ([k][m], may be null),
// and rel[i * k + c] = ||r|| / ||b|| per right-hand side (0 for b = 0).
bool batch_residual(const std::vector<BatchBody>& bodies, int k, cudaStream_t s, const std::vector<double*>& r_out,
                    std::vector<double>& rel, std::string& err);
// x_i += d_i (k n values) for every system
bool batch_axpy(const std::vector<BatchBody>& bodies, int k, const std::vector<double*>& d, cudaStream_t s,
                std::string& err);

bool batch_autotune(const std::vector<BatchBody>& bodies, cudaStream_t s, BatchTune& best, std::string& report,
                    std::string& err);

// lsqr_precon column norms of a packed FP32 matrix (pk_idx layout, ne block
// rows): q_j = 1/||A(:,j)|| for the 3 ne columns (q_j = 0 for ne..lda-1); the
// matrix is not scaled -- the packed sweeps apply q on the fly.
cudaError_t packed_colnorms(const float* Ap, int ne, int ldp, int64_t lda, double* q, double* P, int groups,
                            cudaStream_t s);

// 3-D tensor map of the packed layout: dims {64 columns, 6 x ldp/64 (plane,
// column block), ne rows}, box {64, box_y, box_z}.
bool make_packed_map(CUtensorMap* tm, const void* Ap, int ldp, int ne, int box_y, int box_z, std::string& err);

// 2-D tensor map of a row-major FP32 matrix (dims {lda, m}, box box_cols x box_rows).
bool make_tensor_map_2d(CUtensorMap* tm, const void* A, int64_t lda, int m, int box_cols, int box_rows,
                        std::string& err);

}  // namespace agb
