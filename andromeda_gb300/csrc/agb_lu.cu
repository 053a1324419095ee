// Dense direct solver of the reference's FULL path (lib_solveFM.f: FormPREfm
// :102 with pret = 2 -> dgefa :198; SolvEQNfm :3 with slvt = 0 -> dgesl :318)
// on the GPU, FP64.
//
// Factorisation: blocked right-looking LU with partial pivoting (panels of 64
// columns).  The panel is factored column by column by two kernels -- a
// one-CTA pivot search (first index of the largest |a|, as idamax) with the
// row interchange inside the panel, then a multi-CTA scale + rank-1 update of
// the panel's remaining columns; the interchanges are applied to the other
// columns, then U12 = L11^-1 A12 (cuBLAS dtrsm) and A22 -= A21 U12 (cuBLAS
// dgemm, the O(n^3) part).  Pivots are those of dgefa (same elimination order
// and tie rule); the factors are kept in LAPACK form (positive multipliers,
// every later interchange applied to L), which is what the solve consumes.
// Solve: x = P b (gather), L y = x, U x = y (cuBLAS dtrsm), for many
// right-hand sides at once.
#include "agb_lu.cuh"

#include <cublas_v2.h>
#include <algorithm>
#include <vector>

namespace agb {

constexpr int LU_NB = 64;

// Pivot search of column j (rows j..n-1) by one CTA; interchange of rows j and
// p inside the panel columns [j0, j0+jb); 1/pivot into *recip (0 for a zero
// pivot, which also records info).
__global__ void __launch_bounds__(1024) k_lu_pivot(double* __restrict__ A, int64_t lda, int n, int j, int j0, int jb,
                                                   int* __restrict__ ipiv, double* __restrict__ recip,
                                                   int* __restrict__ info) {
  __shared__ double sv[32];
  __shared__ int si[32];
  const double* col = A + (int64_t)j * lda;
  double best = -1.0;
  int bi = n;
  for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
    const double v = fabs(col[i]);
    if (v > best) { best = v; bi = i; }  // strided scan: first maximum of this thread's rows
  }
  // warp and block reduction: largest |a|, smallest row index among equals
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sv[warp] = best; si[warp] = bi; }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    best = (lane < nw) ? sv[lane] : -1.0;
    bi = (lane < nw) ? si[lane] : n;
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { si[0] = bi; sv[0] = best; }
  }
  __syncthreads();
  const int p = si[0];
  const bool zero = !(sv[0] > 0.0);
  if (threadIdx.x == 0) {
    ipiv[j] = (zero ? j : p) + 1;
    if (zero && *info == 0) *info = j + 1;
  }
  if (!zero && p != j && threadIdx.x < jb) {
    double* r = A + (int64_t)(j0 + threadIdx.x) * lda;
    const double t = r[p];
    r[p] = r[j];
    r[j] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) *recip = zero ? 0.0 : 1.0 / col[j];
}

// Rows j+1..n-1: multiplier l = a(i,j) / pivot, and a(i,c) -= l a(j,c) for the
// panel columns c in (j, j0+jb).
__global__ void k_lu_panel_update(double* __restrict__ A, int64_t lda, int n, int j, int j0, int jb,
                                  const double* __restrict__ recip) {
  const double t = *recip;
  if (t == 0.0) return;  // zero pivot: column already eliminated (dgefa skips the step)
  const int i = j + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double* colj = A + (int64_t)j * lda;
  const double l = colj[i] * t;
  colj[i] = l;
  for (int c = j + 1; c < j0 + jb; ++c) {
    double* cc = A + (int64_t)c * lda;
    cc[i] -= l * cc[j];
  }
}

// Interchanges of the panel (steps j0..j0+jb-1) applied to the columns
// [c0, c1) outside the panel, in step order; one thread per column.
__global__ void k_lu_swap_cols(double* __restrict__ A, int64_t lda, const int* __restrict__ ipiv, int j0, int jb,
                               int c0, int c1) {
  const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= c1) return;
  double* col = A + (int64_t)c * lda;
  for (int j = j0; j < j0 + jb; ++j) {
    const int p = ipiv[j] - 1;
    if (p != j) {
      const double t = col[p];
      col[p] = col[j];
      col[j] = t;
    }
  }
}

// x[i][c] = b[perm[i]][c] (column-major n x nrhs)
__global__ void k_lu_gather(const double* __restrict__ b, const int* __restrict__ perm, int n, int nrhs,
                            double* __restrict__ x) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int c = (int)(t / n), i = (int)(t % n);
  x[t] = b[(int64_t)c * n + perm[i]];
}

static const char* cublas_str(cublasStatus_t s) {
  switch (s) {
    case CUBLAS_STATUS_SUCCESS: return "success";
    case CUBLAS_STATUS_NOT_INITIALIZED: return "not initialized";
    case CUBLAS_STATUS_ALLOC_FAILED: return "alloc failed";
    case CUBLAS_STATUS_INVALID_VALUE: return "invalid value";
    case CUBLAS_STATUS_EXECUTION_FAILED: return "execution failed";
    default: return "error";
  }
}

#define LCK(x)                                                                   \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      goto done;                                                                 \
    }                                                                            \
  } while (0)
#define BLK(x)                                                                   \
  do {                                                                           \
    cublasStatus_t s_ = (x);                                                     \
    if (s_ != CUBLAS_STATUS_SUCCESS) {                                           \
      err = std::string(#x) + ": " + cublas_str(s_);                             \
      goto done;                                                                 \
    }                                                                            \
  } while (0)

bool lu_factor_dev(double* A, int64_t lda, int n, int* ipiv, int* info_host, cudaStream_t s, long* launches,
                   std::string& err) {
  cublasHandle_t h = nullptr;
  double* recip = nullptr;
  int* info = nullptr;
  bool ok = false;
  long nl = 0;
  if (n < 1 || lda < n) { err = "lu: bad sizes"; return false; }
  if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) { err = "cublasCreate failed"; return false; }
  BLK(cublasSetStream(h, s));
  LCK(cudaMallocAsync(&recip, sizeof(double), s));
  LCK(cudaMallocAsync(&info, sizeof(int), s));
  LCK(cudaMemsetAsync(info, 0, sizeof(int), s));
  for (int j0 = 0; j0 < n; j0 += LU_NB) {
    const int jb = std::min(LU_NB, n - j0);
    for (int j = j0; j < j0 + jb; ++j) {
      k_lu_pivot<<<1, 1024, 0, s>>>(A, lda, n, j, j0, jb, ipiv, recip, info);
      if (j + 1 < n) k_lu_panel_update<<<(unsigned)((n - j - 1 + 255) / 256), 256, 0, s>>>(A, lda, n, j, j0, jb, recip);
      nl += (j + 1 < n) ? 2 : 1;
    }
    LCK(cudaGetLastError());
    if (j0 > 0) {
      k_lu_swap_cols<<<(unsigned)((j0 + 255) / 256), 256, 0, s>>>(A, lda, ipiv, j0, jb, 0, j0);
      ++nl;
    }
    const int rest = n - j0 - jb;
    if (rest > 0) {
      k_lu_swap_cols<<<(unsigned)((rest + 255) / 256), 256, 0, s>>>(A, lda, ipiv, j0, jb, j0 + jb, n);
      ++nl;
      const double one = 1.0, mone = -1.0;
      BLK(cublasDtrsm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, jb, rest, &one,
                      A + j0 + (int64_t)j0 * lda, (int)lda, A + j0 + (int64_t)(j0 + jb) * lda, (int)lda));
      BLK(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, rest, rest, jb, &mone, A + (j0 + jb) + (int64_t)j0 * lda, (int)lda,
                      A + j0 + (int64_t)(j0 + jb) * lda, (int)lda, &one, A + (j0 + jb) + (int64_t)(j0 + jb) * lda,
                      (int)lda));
      nl += 2;
    }
    LCK(cudaGetLastError());
  }
  LCK(cudaMemcpyAsync(info_host, info, sizeof(int), cudaMemcpyDeviceToHost, s));
  LCK(cudaStreamSynchronize(s));
  ok = true;
done:
  if (recip) cudaFreeAsync(recip, s);
  if (info) cudaFreeAsync(info, s);
  cudaStreamSynchronize(s);
  cublasDestroy(h);
  if (launches) *launches += nl;
  return ok;
}

bool lu_solve_dev(const double* A, int64_t lda, int n, const int* ipiv_host, int nrhs, double* B, cudaStream_t s,
                  long* launches, std::string& err) {
  cublasHandle_t h = nullptr;
  int* perm = nullptr;
  double* X = nullptr;
  bool ok = false;
  std::vector<int> p(n);
  for (int i = 0; i < n; ++i) p[i] = i;
  for (int k = 0; k < n; ++k) {
    const int l = ipiv_host[k] - 1;
    if (l < 0 || l >= n) { err = "lu: pivot out of range"; return false; }
    std::swap(p[k], p[l]);
  }
  if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) { err = "cublasCreate failed"; return false; }
  BLK(cublasSetStream(h, s));
  LCK(cudaMallocAsync(&perm, n * sizeof(int), s));
  LCK(cudaMallocAsync(&X, (size_t)n * nrhs * sizeof(double), s));
  LCK(cudaMemcpyAsync(perm, p.data(), n * sizeof(int), cudaMemcpyHostToDevice, s));
  k_lu_gather<<<(unsigned)(((int64_t)n * nrhs + 255) / 256), 256, 0, s>>>(B, perm, n, nrhs, X);
  LCK(cudaGetLastError());
  {
    const double one = 1.0;
    BLK(cublasDtrsm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, n, nrhs, &one, A,
                    (int)lda, X, n));
    BLK(cublasDtrsm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, nrhs, &one, A,
                    (int)lda, X, n));
  }
  LCK(cudaMemcpyAsync(B, X, (size_t)n * nrhs * sizeof(double), cudaMemcpyDeviceToDevice, s));
  LCK(cudaStreamSynchronize(s));
  ok = true;
done:
  if (perm) cudaFreeAsync(perm, s);
  if (X) cudaFreeAsync(X, s);
  cudaStreamSynchronize(s);
  cublasDestroy(h);
  if (launches) *launches += 1;
  return ok;
}

}  // namespace agb
