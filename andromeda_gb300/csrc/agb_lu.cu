// Dense direct solver of the reference's FULL path (lib_solveFM.f: FormPREfm
// :102 with pret = 2 -> dgefa :198; SolvEQNfm :3 with slvt = 0 -> dgesl :318)
// on the GPU, FP64.
//
// Factorisation: blocked right-looking LU with partial pivoting (panels of 64
// columns).  The panel is factored column by column by two kernels -- a
// one-CTA pivot search (first index of the largest |a|, as idamax) with the
// row interchange inside the panel, then a multi-CTA scale + rank-1 update of
// the panel's remaining columns; the interchanges are applied to the other
// columns, then U12 = L11^-1 A12 (k_lu_trsm_blk: a warp per column, the 64 x 64
// triangle in shared memory) and A22 -= A21 U12 (k_lu_gemm_sub: 64 x 64 output
// tiles, 4 x 4 FP64 accumulators per thread, the O(n^3) part; GB300's FP64 pipe
// bounds it).  Pivots are those of dgefa (same elimination order and tie
// rule); the factors are kept in LAPACK form (positive multipliers, every later
// interchange applied to L), which is what the solve consumes.  Solve: x = P b
// (gather), then L y = x and U x = y blockwise (the same two kernels: a block
// triangle solve, then the update of the remaining rows), for many right-hand
// sides at once.
#include "agb_lu.cuh"

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

// B (jb x ncols, column-major, leading dimension ldb) <- T^-1 B for the jb x jb
// (jb <= 64) triangle T (column-major, ldt): lower with unit diagonal (UPPER
// false, forward substitution) or upper (UPPER true, backward).  One warp per
// column; lane l holds rows l and l + 32; the triangle sits in shared memory.
template <bool UPPER>
__global__ void __launch_bounds__(256) k_lu_trsm_blk(int jb, const double* __restrict__ T, int64_t ldt,
                                                   double* __restrict__ B, int64_t ldb, int ncols) {
  __shared__ double sT[LU_NB][LU_NB + 1];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int r = t % jb, c = t / jb;
    sT[r][c] = T[r + (int64_t)c * ldt];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int col = blockIdx.x * nw + warp; col < ncols; col += gridDim.x * nw) {
    double* b = B + (int64_t)col * ldb;
    const int r0 = lane, r1 = lane + 32;
    double x0 = (r0 < jb) ? b[r0] : 0.0;
    double x1 = (r1 < jb) ? b[r1] : 0.0;
    if (!UPPER) {
      for (int k = 0; k < jb; ++k) {
        const double xk = __shfl_sync(0xffffffffu, k < 32 ? x0 : x1, k & 31);
        if (r0 > k && r0 < jb) x0 -= sT[r0][k] * xk;
        if (r1 > k && r1 < jb) x1 -= sT[r1][k] * xk;
      }
    } else {
      for (int k = jb - 1; k >= 0; --k) {
        if (k < 32) {
          if (lane == k) x0 /= sT[k][k];
        } else if (lane == k - 32) {
          x1 /= sT[k][k];
        }
        const double xk = __shfl_sync(0xffffffffu, k < 32 ? x0 : x1, k & 31);
        if (r0 < k) x0 -= sT[r0][k] * xk;
        if (r1 < k) x1 -= sT[r1][k] * xk;
      }
    }
    if (r0 < jb) b[r0] = x0;
    if (r1 < jb) b[r1] = x1;
  }
}

// C (m x n) -= A (m x k) B (k x n), all column-major, k <= 64: 64 x 64 output
// tiles per CTA of 256 threads, 4 x 4 FP64 accumulators per thread, the
// operands staged through shared memory in chunks of 32 of k.
constexpr int LU_GT = 64, LU_GK = 32;
__global__ void __launch_bounds__(256) k_lu_gemm_sub(int m, int n, int k, const double* __restrict__ A, int64_t lda,
                                                   const double* __restrict__ B, int64_t ldb, double* __restrict__ C,
                                                   int64_t ldc) {
  __shared__ double sA[LU_GK][LU_GT + 1];  // [kk][row]
  __shared__ double sB[LU_GT][LU_GK + 1];  // [col][kk]
  const int r0 = blockIdx.x * LU_GT, c0 = blockIdx.y * LU_GT;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < k; k0 += LU_GK) {
    const int kc = min(LU_GK, k - k0);
    for (int t = threadIdx.x; t < LU_GT * LU_GK; t += 256) {
      const int rr = t % LU_GT, kk = t / LU_GT;
      sA[kk][rr] = (r0 + rr < m && kk < kc) ? A[(r0 + rr) + (int64_t)(k0 + kk) * lda] : 0.0;
      const int k2 = t % LU_GK, cc = t / LU_GK;
      sB[cc][k2] = (k2 < kc && c0 + cc < n) ? B[(k0 + k2) + (int64_t)(c0 + cc) * ldb] : 0.0;
    }
    __syncthreads();
    for (int kk = 0; kk < kc; ++kk) {
      double a[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = sB[ty + 16 * j][kk];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = r0 + tx + 16 * i, c = c0 + ty + 16 * j;
      if (r < m && c < n) C[r + (int64_t)c * ldc] -= acc[i][j];
    }
}

static void launch_trsm(bool upper, int jb, const double* T, int64_t ldt, double* B, int64_t ldb, int ncols,
                        cudaStream_t s) {
  const unsigned blocks = (unsigned)std::min<int64_t>(((int64_t)ncols + 7) / 8, 152 * 8);
  if (upper)
    k_lu_trsm_blk<true><<<blocks, 256, 0, s>>>(jb, T, ldt, B, ldb, ncols);
  else
    k_lu_trsm_blk<false><<<blocks, 256, 0, s>>>(jb, T, ldt, B, ldb, ncols);
}
static void launch_gemm_sub(int m, int n, int k, const double* A, int64_t lda, const double* B, int64_t ldb,
                            double* C, int64_t ldc, cudaStream_t s) {
  const dim3 grid((unsigned)((m + LU_GT - 1) / LU_GT), (unsigned)((n + LU_GT - 1) / LU_GT));
  k_lu_gemm_sub<<<grid, 256, 0, s>>>(m, n, k, A, lda, B, ldb, C, ldc);
}

#define LCK(x)                                                                   \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      goto done;                                                                 \
    }                                                                            \
  } while (0)

bool lu_factor_dev(double* A, int64_t lda, int n, int* ipiv, int* info_host, cudaStream_t s, long* launches,
                   std::string& err) {
  double* recip = nullptr;
  int* info = nullptr;
  bool ok = false;
  long nl = 0;
  if (n < 1 || lda < n) { err = "lu: bad sizes"; return false; }
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
      // U12 = L11^-1 A12, then A22 -= A21 U12
      double* A11 = A + j0 + (int64_t)j0 * lda;
      double* A12 = A + j0 + (int64_t)(j0 + jb) * lda;
      double* A21 = A + (j0 + jb) + (int64_t)j0 * lda;
      double* A22 = A + (j0 + jb) + (int64_t)(j0 + jb) * lda;
      launch_trsm(false, jb, A11, lda, A12, lda, rest, s);
      launch_gemm_sub(rest, rest, jb, A21, lda, A12, lda, A22, lda, s);
      nl += 3;
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
  if (launches) *launches += nl;
  return ok;
}

bool lu_solve_dev(const double* A, int64_t lda, int n, const int* ipiv_host, int nrhs, double* B, cudaStream_t s,
                  long* launches, std::string& err) {
  int* perm = nullptr;
  double* X = nullptr;
  bool ok = false;
  long nl = 0;
  std::vector<int> p(n);
  for (int i = 0; i < n; ++i) p[i] = i;
  for (int k = 0; k < n; ++k) {
    const int l = ipiv_host[k] - 1;
    if (l < 0 || l >= n) { err = "lu: pivot out of range"; return false; }
    std::swap(p[k], p[l]);
  }
  LCK(cudaMallocAsync(&perm, n * sizeof(int), s));
  LCK(cudaMallocAsync(&X, (size_t)n * nrhs * sizeof(double), s));
  LCK(cudaMemcpyAsync(perm, p.data(), n * sizeof(int), cudaMemcpyHostToDevice, s));
  k_lu_gather<<<(unsigned)(((int64_t)n * nrhs + 255) / 256), 256, 0, s>>>(B, perm, n, nrhs, X);
  ++nl;
  LCK(cudaGetLastError());
  // L y = x: diagonal block, then the rows below
  for (int k0 = 0; k0 < n; k0 += LU_NB) {
    const int jb = std::min(LU_NB, n - k0);
    launch_trsm(false, jb, A + k0 + (int64_t)k0 * lda, lda, X + k0, n, nrhs, s);
    ++nl;
    if (k0 + jb < n) {
      launch_gemm_sub(n - k0 - jb, nrhs, jb, A + (k0 + jb) + (int64_t)k0 * lda, lda, X + k0, n, X + k0 + jb, n, s);
      ++nl;
    }
  }
  // U x = y: from the last diagonal block up, then the rows above
  for (int k0 = ((n - 1) / LU_NB) * LU_NB; k0 >= 0; k0 -= LU_NB) {
    const int jb = std::min(LU_NB, n - k0);
    launch_trsm(true, jb, A + k0 + (int64_t)k0 * lda, lda, X + k0, n, nrhs, s);
    ++nl;
    if (k0 > 0) {
      launch_gemm_sub(k0, nrhs, jb, A + (int64_t)k0 * lda, lda, X + k0, n, X, n, s);
      ++nl;
    }
  }
  LCK(cudaGetLastError());
  LCK(cudaMemcpyAsync(B, X, (size_t)n * nrhs * sizeof(double), cudaMemcpyDeviceToDevice, s));
  LCK(cudaStreamSynchronize(s));
  ok = true;
done:
  if (perm) cudaFreeAsync(perm, s);
  if (X) cudaFreeAsync(X, s);
  cudaStreamSynchronize(s);
  if (launches) *launches += nl;
  return ok;
}

}  // namespace agb
