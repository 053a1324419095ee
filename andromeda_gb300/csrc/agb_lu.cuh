// Dense LU direct solver (FP64) of the FULL path: factorisation in place of a
// column-major matrix and multi-RHS solve from its factors.
#pragma once
#include "agb_common.cuh"
#include <string>

namespace agb {

// LU with partial pivoting of the column-major n x n matrix A (device, leading
// dimension lda) in place; ipiv (device, n ints) receives 1-based pivot rows
// (dgefa's ipvt), *info_host the first zero pivot (1-based) or 0.  Factors in
// LAPACK form (unit lower L with positive multipliers and every later
// interchange applied, U on and above the diagonal).
bool lu_factor_dev(double* A, int64_t lda, int n, int* ipiv, int* info_host, cudaStream_t s, long* launches,
                   std::string& err);
// B (device, column-major n x nrhs) <- A^-1 B from lu_factor_dev's factors.
bool lu_solve_dev(const double* A, int64_t lda, int n, const int* ipiv_host, int nrhs, double* B, cudaStream_t s,
                  long* launches, std::string& err);

}  // namespace agb
