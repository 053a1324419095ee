// Block LSQR on a dense row-major matrix resident in HBM (host-side driver).
#pragma once
#include "agb_common.cuh"
#include <cuda.h>
#include <vector>
#include <string>

namespace agb {

// Per right-hand-side LSQR recurrence state (lib_lsqr.f:900-1231), FP64.
struct LsqrScalars {
  double alpha, beta, rhobar, phibar, anorm, dnorm, res2, xnorm, xnorm1, cs2, sn2, z, bnorm, rnorm, arnorm, acond;
  double atol, btol, ctol;
  double t1, t2, t3;       // x/w update coefficients of the current iteration
  double gamma;            // coefficient of Y_old in Y = A V + gamma Y_old
  double dxmax;
  int itn, istop, active, itnlim;
};

// Per right-hand-side BiCGSTAB state (DenseLsqr::bicgstab), FP64.  status: -1
// running, 0 converged, 1 iteration limit, 2 breakdown, 3 diverged or
// stagnated (best: the smallest relative residual so far; since: iterations
// since it last fell by 10 %).
struct BicgScalars {
  double rho, rho_old, alpha, omega, bnorm, relres, snorm, best;
  int its, status, active, half, since;
};
// Per right-hand side GMRES state (DenseLsqr::gmres), FP64.  status: -1
// running, 0 converged, 1 iteration limit, 3 a cycle without a 10 % gain of
// the true residual.  jc: Arnoldi steps of the current cycle; hnext: the norm
// that normalises the next basis vector; prev: the true relative residual at
// the start of the cycle.
// terms of a lane summed in float-float form before they move into FP64 (true residuals)
constexpr int kFFTerms = 256;
struct GmresScalars {
  double bnorm, beta, hnext, relres, prev;
  int its, jc, active, status, cycles;
};
// BiCGSTAB stops a right-hand side whose residual grew BICG_DIVERGE times
// above its best, or did not fall by 10 % within BICG_STALL iterations.
constexpr double BICG_DIVERGE = 1.0e3;
constexpr int BICG_STALL = 64;

// Dense block LSQR.  A is m x n row-major with leading dimension lda (lda is
// a multiple of 32 and columns n..lda-1 are zero).  T = float (mixed path)
// or double (FP64 path).  Up to AGB_MAX_RHS right-hand sides share every
// sweep over A.
struct DenseLsqr {
  int m = 0, n = 0, k = 0;
  int64_t lda = 0;
  bool fp32 = false;
  const void* A = nullptr;     // device, T
  cudaStream_t stream = 0;
  // device work buffers (FP64 unless noted)
  double *Y = nullptr, *V = nullptr, *W = nullptr, *X = nullptr, *Z = nullptr;
  void *Ys = nullptr, *Vs = nullptr;  // T copies used by the sweeps (Ys [m][8], Vs [8][lda])
  double* XsD = nullptr;       // x0./q packed [lda][8] for the FP64-accumulated residual
  float* Xff = nullptr;        // q.XsD split into FP32 high and low parts [2][lda][8] (packed residual)
  bool resid_fp64 = false;     // packed residual on the FP64 pipe (k_residp) instead of float-float
  int* errflag = nullptr;      // set by a kernel whose bounded wait gave up
  double* part = nullptr;      // per-CTA partial sums
  double* Zp = nullptr;        // per-row-group partial products of A^T Y
  LsqrScalars* sc = nullptr;   // k entries
  int* nactive = nullptr;      // device counter
  int* h_nactive = nullptr;    // pinned host mirror
  int zgroups = 0;
  // live per-kernel timing of the two sweeps (CUDA events recorded inside the
  // iteration graph on the solver stream)
  cudaEvent_t pev[4 * 32] = {};
  bool pev_ready = false;
  // TMA descriptors of A for the FP32 sweeps (2-D tiles: 256 columns x 64
  // rows for A*V, 256 columns x 32 rows for A^T*U)
  CUtensorMap tm_av{};
  CUtensorMap tm_atu{};
  bool use_tma = false;
  // packed symmetric-block single layer (A = Ap[i][6][ldp], m = n = 3 ne): the
  // sweeps read 6 of the 9 entries of every 3x3 block; q is applied on the fly
  bool packed = false;
  int pk_ne = 0, pk_ldp = 0;
  float* Vp = nullptr;          // [3][8][ldp] = q.V, sweep-1 operand of the packed layout
  CUtensorMap tm_vp{};
  // matrix-free operator (A == nullptr): the sweeps recompute A's entries
  const struct MfOp* mf = nullptr;
  float* Yp = nullptr;          // [col blocks][m][8] partial products of A V
  int mf_cb = 0;
  const double* mf_q = nullptr; // column scales applied on the fly
  // block-Jacobi right preconditioner of the packed LSQR (bj): the inverses of
  // the elements' 3x3 self blocks [ne][3][3], in place of the column scales q
  double* pc9 = nullptr;
  bool bj = false;
  bool pc9_ready = false;  // computed for the current matrix
  // BiCGSTAB work (bicgstab): R, Rt, P, S, T, X ([m][8] each) and 1/diag(A) [m]
  double* bg = nullptr;
  double* bg_part = nullptr;    // per-CTA partial sums
  BicgScalars* bsc = nullptr;
  LsqrScalars* sc0 = nullptr;   // zero gammas: the packed sweep writes Y = A W
  bool bg_diag = false;         // 1/diag(A) computed for the current matrix
  // GMRES work (gmres): basis, w, X, r, Hessenberg and rotations; partial sums
  double* gm = nullptr;
  double* gm_part = nullptr;
  size_t gm_cap = 0;
  int gm_mr = 0;
  GmresScalars* gsc = nullptr;
  double t_av = 0.0, t_atu = 0.0;
  long n_av = 0, n_atu = 0;
  long launches = 0;           // kernels launched by precon/solve
  size_t part_cap = 0;
  std::string err;

  ~DenseLsqr();
  bool setup(const void* A_dev, bool is_fp32, int m, int n, int64_t lda, int k, cudaStream_t s);
  // Column scaling of lsqr_precon: q_j = 1/||A(:,j)||, A <- A diag(q) (in place).
  bool precon(void* A_dev, double* q_dev);
  // lsqr_solve semantics per column c: x0 = X_in(:,c) warm start, b(:,c);
  // x_out = q .* dx + x0.  b and x are device FP64, column-major n x k / m x k.
  // x0_zero: the caller guarantees a zero warm start, so r0 = b and the
  // FP64-accumulated residual sweep over A is skipped.
  bool solve(const double* b_dev, double* x_dev, const double* q_dev, double eps, int maxit, int* nit_host,
             int* istop_host, double* rnorm_host = nullptr, int check_every = 8, bool x0_zero = false);
  // BiCGSTAB with the Jacobi preconditioner on the packed layout (the solver of
  // the reference's LIS path): per column c, A x = b from x0 = 0 until
  // ||b - A x|| <= tol ||b|| (recursive residual) or maxit iterations (0: 1000).
  // b: column-major m x k in the row numbering 3i+a; x: column-major n x k in the
  // unknown numbering a ne + i (that of solve).  status per column: 0 converged,
  // 1 iteration limit, 2 breakdown.
  bool bicgstab(const double* b_dev, double* x_dev, double tol, int maxit, int* nit_host, int* status_host,
                double* relres_host = nullptr);
  // restarted GMRES(restart) with the 3x3 self-block right preconditioner on
  // the packed layout: per column c, A x = b from x0 = 0 until the FP64 true
  // residual ||b - A x|| <= tol ||b|| (checked at the end of every cycle) or
  // maxit Arnoldi steps (0: 1000).  b, x as bicgstab; q: the column scales the
  // residual sweep takes (those of solve).  status per column: 0 converged, 1
  // iteration limit, 3 a cycle without a 10 % gain of the true residual.
  bool gmres(const double* b_dev, double* x_dev, const double* q_dev, double tol, int maxit, int restart,
             int* nit_host, int* status_host, double* relres_host = nullptr, int* cycles_host = nullptr);
  // inverses of the packed matrix's 3x3 self blocks into pc9 (once per matrix)
  bool block_precon();
  // r = b - A (x ./ q) with FP64 accumulation (refinement residual): the true
  // residual of x for the matrix scaled by q; q_dev may be null on the packed
  // system, whose matrix stays unscaled.
  bool residual(const double* b_dev, const double* x_dev, const double* q_dev, double* r_dev);
  void release();
};

// Y = A W over the packed layout (k_avp with the gammas of sc), W the solver's Vp;
// nothing while *gate == 0 (device counter of active right-hand sides).
void launch_avp(const DenseLsqr& L, const LsqrScalars* sc, double* Y, const int* gate);

bool crs_lsqr_precon(int m, int n, int64_t nnz, double* q, const int64_t* ia, const int* ja, double* a, std::string& err);
bool crs_lsqr_solve(int m, int n, int64_t nnz, int& maxit, double eps, int& nit, int& ierr, const double* q,
                    const int64_t* ia, const int* ja, const double* a, const double* b, double* x, std::string& err);

}  // namespace agb
