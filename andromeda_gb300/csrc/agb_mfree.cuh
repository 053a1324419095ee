// Matrix-free Stokes single-layer operator (FP32 quadrature recomputed in
// every LSQR sweep) for systems too large to store.
#pragma once
#include "agb_assembly.cuh"
#include "agb_lsqr.cuh"

namespace agb {

struct MfOp {
  int ne = 0, Q = 0, ldp = 0;
  const QPt<float>* pts = nullptr;  // [Q][ldp] quadrature points (x, y, z, w*area)
  const float* src = nullptr;       // [3][ldp] collocation points (centroids)
  const float* colscale = nullptr;  // [ldp] -(multi_j / mu)
  float* self6 = nullptr;           // [ne][6] scaled analytic self blocks (xx,xy,xz,yy,yz,zz)
};

cudaError_t mf_setup_self(MfOp& op, const ElemGeom* geom, double diff, cudaStream_t s);
int mf_row_groups(const MfOp& op);  // source-row groups (256 rows) = partial groups of A^T U
int mf_col_blocks(const MfOp& op);  // element-column blocks (256 columns) = partial blocks of A V
// Yp[cb][3 ne][8] partial products of A diag(q) V (Vs RHS-major [8][lda])
cudaError_t mf_av(const MfOp& op, const float* Vs, const double* q, int64_t lda, float* Yp, cudaStream_t s);
// Y = sum Yp + gamma Y (FP64 [m][8]), Ys (FP32), per-CTA partial sums of Y^2 (cdiv(m*8,256) CTAs)
cudaError_t mf_av_reduce(int m, int ncb, const float* Yp, const LsqrScalars* sc, double* Y, float* Ys, double* part,
                         cudaStream_t s);
// colsq = false: Zp[g][lda][8] = diag(q) A^T U per row group (U = Us [m][8]);
// colsq = true:  Zp[g][lda] = column sums of squares of A per row group
cudaError_t mf_atu(const MfOp& op, const float* Us, const double* q, int64_t lda, double* Zp, bool colsq,
                   cudaStream_t s);

}  // namespace agb
