// Matrix-free Stokes single-layer operator for LSQR (systems too large to
// store: 102 400 triangles give a 307 200^2 FP32 matrix of 377 GB).  Every
// sweep recomputes the entries A[3i+a][b*ne+j] = -(multi_j/mu) int_{e_j}
// G_ab(x_i, y) dy exactly as the stored-matrix assembly does (same FP32
// quadrature on the expanded point table, the same analytic FP64 self blocks)
// and contracts them with the 8 right-hand-side vectors on the fly:
//
//   mf_av   Y = A diag(q) V : a CTA takes 256 source rows x 256 element
//           columns (8 tiles of 32 staged in shared memory); a warp computes
//           the 3x3 blocks of 8 rows against its lane's column, contracts them
//           with q.V of that column, reduces the 24 row values over the 32
//           lanes and adds them to the CTA's row partials in shared memory;
//           partials per column block go to Yp and are summed in a fixed
//           order by mf_av_reduce (which also forms Y = Yp + gamma Y_old);
//   mf_atu  Z = diag(q) A^T U : a CTA takes 32 element columns (one per lane)
//           x 256 rows; each lane accumulates its column's 24 values over the
//           rows, the 8 warps are combined in shared memory and the FP64
//           partials per row group go to Zp in the layout of the stored
//           sweep (reduced by the same k_atu_reduce);
//   mf_colsq  column sums of squares for lsqr_precon's q.
// The work per sweep is the assembly's (ne^2 x Q point evaluations), so the
// sweeps are FP32-pipe bound; the partial buffers cost a few GB of traffic.
#include "agb_mfree.cuh"
#include "agb_singular.cuh"

namespace agb {

constexpr int MF_RS = 8;        // rows per warp step
constexpr int MF_NW = 8;        // warps per CTA
constexpr int MF_ROWS = 256;    // source rows per CTA
constexpr int MF_TILES = 8;     // 32-column tiles per A*V CTA
constexpr int MF_K = 8;         // right-hand sides

static inline unsigned mcdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

__global__ void k_mf_self(int ne, const ElemGeom* __restrict__ geom, double diff, float* __restrict__ self6) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ne) return;
  const ElemGeom& G = geom[p];
  double g[6];
  agb_sing::tri_stokes(G.v[0], G.v[1], G.v[2], G.area, 4, g);
  const double sc = -G.multi / diff;
  for (int k = 0; k < 6; ++k) self6[(int64_t)p * 6 + k] = (float)(sc * g[k]);
}

cudaError_t mf_setup_self(MfOp& op, const ElemGeom* geom, double diff, cudaStream_t s) {
  k_mf_self<<<mcdiv(op.ne, 128), 128, 0, s>>>(op.ne, geom, diff, op.self6);
  return cudaGetLastError();
}

// 3x3 block of rows i (RS of them) against the lane's column j; g[r][6] = {xx,xy,xz,yy,yz,zz} (scaled)
__device__ __forceinline__ void mf_blocks(const QPt<float>* __restrict__ sp, int Q, int lane, const float (&sx)[MF_RS],
                                          const float (&sy)[MF_RS], const float (&sz)[MF_RS], float (&acc)[MF_RS][7]) {
#pragma unroll
  for (int r = 0; r < MF_RS; ++r)
#pragma unroll
    for (int c = 0; c < 7; ++c) acc[r][c] = 0.f;
#pragma unroll 2
  for (int q = 0; q < Q; ++q) {
    const QPt<float> p = sp[q * 32 + lane];
#pragma unroll
    for (int r = 0; r < MF_RS; ++r) {
      const float rx = p.x - sx[r], ry = p.y - sy[r], rz = p.z - sz[r];
      const float r2 = rx * rx + ry * ry + rz * rz;
      const float ir = rsqrtf(r2);
      const float wi = p.w * ir;
      const float wi3 = wi * (ir * ir);
      acc[r][0] += wi;
      const float ax = wi3 * rx, ay = wi3 * ry;
      acc[r][1] += ax * rx;
      acc[r][2] += ax * ry;
      acc[r][3] += ax * rz;
      acc[r][4] += ay * ry;
      acc[r][5] += ay * rz;
      acc[r][6] += (wi3 * rz) * rz;
    }
  }
}

__device__ __forceinline__ void mf_sym(const float (&a)[7], float scale, float (&g)[6]) {
  g[0] = scale * (a[0] + a[1]); g[1] = scale * a[2]; g[2] = scale * a[3];
  g[3] = scale * (a[0] + a[4]); g[4] = scale * a[5]; g[5] = scale * (a[0] + a[6]);
}
// component (a, b) of the symmetric block
__device__ __forceinline__ float mf_g(const float (&g)[6], int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return lo == 0 ? g[hi] : (lo == 1 ? g[2 + hi] : g[5]);
}

// Y partials: Yp[cb][3i+a][c] = sum over the CTA's 256 element columns of A(3i+a, b ne + j) q V
__global__ void __launch_bounds__(MF_NW * 32, 2) k_mf_av(MfOp op, const float* __restrict__ Vs, const double* __restrict__ q,
                                                      int64_t lda, float* __restrict__ Yp) {
  extern __shared__ __align__(16) unsigned char mf_smem[];
  QPt<float>* sp = reinterpret_cast<QPt<float>*>(mf_smem);
  float* part = reinterpret_cast<float*>(mf_smem + (size_t)op.Q * 32 * sizeof(QPt<float>));  // [MF_ROWS][24]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i0 = blockIdx.y * MF_ROWS;
  const int ne = op.ne;
  for (int t = threadIdx.x; t < MF_ROWS * 24; t += MF_NW * 32) part[t] = 0.f;
  for (int tile = 0; tile < MF_TILES; ++tile) {
    const int j0 = (blockIdx.x * MF_TILES + tile) * 32;
    if (j0 >= ne) break;
    __syncthreads();
    for (int t = threadIdx.x; t < op.Q * 32; t += MF_NW * 32) sp[t] = op.pts[(int64_t)(t >> 5) * op.ldp + j0 + (t & 31)];
    __syncthreads();
    const int j = j0 + lane;
    const bool jv = j < ne;
    const float scale = jv ? op.colscale[j] : 0.f;
    // the lane's column values q.V for the three components b and 8 right-hand sides
    float w[3][MF_K];
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = 0; c < MF_K; ++c) {
        const int64_t col = (int64_t)b * ne + j;
        w[b][c] = jv ? (float)q[col] * Vs[(int64_t)c * lda + col] : 0.f;
      }
    for (int ib = i0 + warp * MF_RS; ib < min(ne, i0 + MF_ROWS); ib += MF_NW * MF_RS) {
      float sx[MF_RS], sy[MF_RS], sz[MF_RS];
#pragma unroll
      for (int r = 0; r < MF_RS; ++r) {
        const int i = min(ib + r, ne - 1);
        sx[r] = op.src[i]; sy[r] = op.src[op.ldp + i]; sz[r] = op.src[2 * op.ldp + i];
      }
      float acc[MF_RS][7];
      mf_blocks(sp, op.Q, lane, sx, sy, sz, acc);
#pragma unroll
      for (int r = 0; r < MF_RS; ++r) {
        const int i = ib + r;
        if (i >= min(ne, i0 + MF_ROWS)) break;  // warp-uniform
        float g[6];
        if (jv && i == j) {
#pragma unroll
          for (int k = 0; k < 6; ++k) g[k] = op.self6[(int64_t)j * 6 + k];
        } else {
          mf_sym(acc[r], scale, g);
        }
        // y[a][c] = sum_b g_ab w_b[c], reduced over the 32 columns of the tile
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int c = 0; c < MF_K; ++c) {
            float y = mf_g(g, a, 0) * w[0][c] + mf_g(g, a, 1) * w[1][c] + mf_g(g, a, 2) * w[2][c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
            if (lane == a * MF_K + c) part[(i - i0) * 24 + lane] += y;
          }
      }
    }
  }
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * (3 * (int64_t)ne) * MF_K;
  for (int t = threadIdx.x; t < MF_ROWS * 24; t += MF_NW * 32) {
    const int il = t / 24, k = t % 24, a = k / MF_K, c = k % MF_K;
    const int i = i0 + il;
    if (i < ne) Yp[base + ((int64_t)(3 * i + a)) * MF_K + c] = part[t];
  }
}

// Y = sum_cb Yp + gamma Y_old (FP64), Ys = (float)Y, partial ||Y||^2 per CTA
__global__ void __launch_bounds__(256) k_mf_av_reduce(int m, int ncb, const float* __restrict__ Yp,
                                                      const LsqrScalars* sc, double* __restrict__ Y,
                                                      float* __restrict__ Ys, double* __restrict__ part) {
  __shared__ double sP[8][MF_K];
  const int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x;
  const int64_t row = t / MF_K;
  const int c = (int)(t % MF_K);
  double y2 = 0.0;
  if (row < m) {
    double s = 0.0;
    for (int b = 0; b < ncb; ++b) s += (double)Yp[((int64_t)b * m + row) * MF_K + c];
    const double y = s + sc[c].gamma * Y[t];
    Y[t] = y;
    Ys[t] = (float)y;
    y2 = y * y;
  }
  y2 += __shfl_xor_sync(0xffffffffu, y2, 8);
  y2 += __shfl_xor_sync(0xffffffffu, y2, 16);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < MF_K) sP[warp][lane] = y2;
  __syncthreads();
  if (threadIdx.x < MF_K) {
    double a = 0.0;
    for (int w = 0; w < 8; ++w) a += sP[w][threadIdx.x];
    part[(int64_t)blockIdx.x * MF_K + threadIdx.x] = a;
  }
}

// COLSQ = false: Zp[g][b ne + j][c] = q_{b ne + j} sum_{rows of group g} A(3i+a, b ne + j) U[3i+a][c]
// COLSQ = true:  Zp[g][b ne + j]    = sum_{rows of group g} A(3i+a, b ne + j)^2
template <bool COLSQ>
__global__ void __launch_bounds__(MF_NW * 32, 2) k_mf_atu(MfOp op, const float* __restrict__ Us,
                                                       const double* __restrict__ q, int64_t lda,
                                                       double* __restrict__ Zp) {
  extern __shared__ __align__(16) unsigned char mf_smem[];
  QPt<float>* sp = reinterpret_cast<QPt<float>*>(mf_smem);
  constexpr int NV = COLSQ ? 3 : 24;
  float* red = reinterpret_cast<float*>(mf_smem);  // [MF_NW][NV][32], reuses the point table after the sweep
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ne = op.ne;
  const int j0 = blockIdx.x * 32;
  const int g = blockIdx.y;
  const int i0 = g * MF_ROWS, i1 = min(ne, i0 + MF_ROWS);
  for (int t = threadIdx.x; t < op.Q * 32; t += MF_NW * 32) sp[t] = op.pts[(int64_t)(t >> 5) * op.ldp + j0 + (t & 31)];
  __syncthreads();
  const int j = j0 + lane;
  const bool jv = j < ne;
  const float scale = jv ? op.colscale[j] : 0.f;
  float z[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) z[k] = 0.f;
  for (int ib = i0 + warp * MF_RS; ib < i1; ib += MF_NW * MF_RS) {
    float sx[MF_RS], sy[MF_RS], sz[MF_RS];
#pragma unroll
    for (int r = 0; r < MF_RS; ++r) {
      const int i = min(ib + r, ne - 1);
      sx[r] = op.src[i]; sy[r] = op.src[op.ldp + i]; sz[r] = op.src[2 * op.ldp + i];
    }
    float acc[MF_RS][7];
    mf_blocks(sp, op.Q, lane, sx, sy, sz, acc);
#pragma unroll
    for (int r = 0; r < MF_RS; ++r) {
      const int i = ib + r;
      if (i >= i1) break;
      float gb[6];
      if (jv && i == j) {
#pragma unroll
        for (int k = 0; k < 6; ++k) gb[k] = op.self6[(int64_t)j * 6 + k];
      } else {
        mf_sym(acc[r], scale, gb);
      }
      if (COLSQ) {
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float v = mf_g(gb, a, b);
            z[b] += v * v;
          }
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float4 u0 = *reinterpret_cast<const float4*>(Us + (int64_t)(3 * i + a) * MF_K);
          const float4 u1 = *reinterpret_cast<const float4*>(Us + (int64_t)(3 * i + a) * MF_K + 4);
          const float uu[MF_K] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            const float v = mf_g(gb, a, b);
#pragma unroll
            for (int c = 0; c < MF_K; ++c) z[b * MF_K + c] += v * uu[c];
          }
        }
      }
    }
  }
  // combine the 8 warps in shared memory (the point table is no longer needed)
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) red[(warp * NV + k) * 32 + lane] = z[k];
  __syncthreads();
  for (int t = threadIdx.x; t < NV * 32; t += MF_NW * 32) {
    const int k = t / 32, l = t % 32;
    const int jj = j0 + l;
    if (jj >= ne) continue;
    double s = 0.0;
    for (int w = 0; w < MF_NW; ++w) s += (double)red[(w * NV + k) * 32 + l];
    if (COLSQ) {
      Zp[(int64_t)g * lda + (int64_t)k * ne + jj] = s;
    } else {
      const int b = k / MF_K, c = k % MF_K;
      const int64_t col = (int64_t)b * ne + jj;
      Zp[((int64_t)g * lda + col) * MF_K + c] = q[col] * s;
    }
  }
}

static size_t av_smem(const MfOp& op) { return (size_t)op.Q * 32 * sizeof(QPt<float>) + MF_ROWS * 24 * sizeof(float); }
static size_t atu_smem(const MfOp& op, bool colsq) {
  const size_t pts = (size_t)op.Q * 32 * sizeof(QPt<float>);
  const size_t red = (size_t)MF_NW * (colsq ? 3 : 24) * 32 * sizeof(float);
  return pts > red ? pts : red;  // the warp reduction reuses the point table's space
}

int mf_row_groups(const MfOp& op) { return (int)mcdiv(op.ne, MF_ROWS); }
int mf_col_blocks(const MfOp& op) { return (int)mcdiv(op.ne, 32 * MF_TILES); }

cudaError_t mf_av(const MfOp& op, const float* Vs, const double* q, int64_t lda, float* Yp, cudaStream_t s) {
  const size_t sm = av_smem(op);
  cudaError_t e = cudaFuncSetAttribute(k_mf_av, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  dim3 grid(mf_col_blocks(op), mf_row_groups(op));
  k_mf_av<<<grid, MF_NW * 32, sm, s>>>(op, Vs, q, lda, Yp);
  return cudaGetLastError();
}

cudaError_t mf_av_reduce(int m, int ncb, const float* Yp, const LsqrScalars* sc, double* Y, float* Ys, double* part,
                         cudaStream_t s) {
  k_mf_av_reduce<<<mcdiv((int64_t)m * MF_K, 256), 256, 0, s>>>(m, ncb, Yp, sc, Y, Ys, part);
  return cudaGetLastError();
}

cudaError_t mf_atu(const MfOp& op, const float* Us, const double* q, int64_t lda, double* Zp, bool colsq,
                   cudaStream_t s) {
  const size_t sm = atu_smem(op, colsq);
  dim3 grid(mcdiv(op.ne, 32), mf_row_groups(op));
  cudaError_t e;
  if (colsq) {
    e = cudaFuncSetAttribute(k_mf_atu<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) k_mf_atu<true><<<grid, MF_NW * 32, sm, s>>>(op, Us, q, lda, Zp);
  } else {
    e = cudaFuncSetAttribute(k_mf_atu<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) k_mf_atu<false><<<grid, MF_NW * 32, sm, s>>>(op, Us, q, lda, Zp);
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace agb
