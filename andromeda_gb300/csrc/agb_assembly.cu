// Assembly of the BEM influence matrices on the GPU.
//
// Reference path (behaviour restated, src/ file:line):
//   geometry           CalElementNormal lib_mesh.f90:716, CalElementArea lib_int.f90:606,
//                      CalQMesh lib_mesh.f90:577
//   Laplace rows       sdIntRowQ lib_sdBem.f90:589 (regular: Triangle_3DLapInt :859,
//                      BemKernel :911; quads Quad_BEMIntNum lib_intAna.f90:219;
//                      self element si_tri_lap / si_qua_lap mod_singInt.f90:127,172)
//   Stokes rows        sdIntRowQStokes lib_Stokes.f90:1562 (regular: Triangle_3DStokesInt
//                      :2341, StokesKernel :2450; self element si_tri_stk mod_singInt.f90:34)
//   BC routing         formQrow lib_StokesFull.f90:4, sdSetUpSysMrhsM_CRS lib_CRS.f90:148
//
// GB300 layout: the system matrix of an all-Dirichlet problem is written
// directly in the reference's unknown numbering (rows source-major /
// component-minor, columns component-major) as a dense row-major matrix in
// HBM.  The regular part is computed by tiles of 32 elements x many
// collocation points: the tile's quadrature points are staged once in shared
// memory and re-used by every collocation point of the CTA, kernels are
// evaluated in registers (8 collocation points per warp in flight), and a warp
// stores 32 consecutive columns (128 B segments) per matrix row.
#include "agb_assembly.cuh"
#include "agb_singular.cuh"
#include "quad_tables.h"

namespace agb {

__constant__ double cGaussGi[156];
__constant__ double cGaussOme[156];
__constant__ int cGaussNg1[8];
__constant__ int cGaussNg2[8];

cudaError_t upload_gauss_tables() {
  cudaError_t e = cudaMemcpyToSymbol(cGaussGi, agb_tables::kGaussGi, sizeof(agb_tables::kGaussGi));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(cGaussOme, agb_tables::kGaussOme, sizeof(agb_tables::kGaussOme));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(cGaussNg1, agb_tables::kGaussNg1, sizeof(agb_tables::kGaussNg1));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(cGaussNg2, agb_tables::kGaussNg2, sizeof(agb_tables::kGaussNg2));
  return e;
}

static inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Bilinear quad map at (gii, gij): position X, unnormalised normal N, shape f4.
__device__ __forceinline__ void quad_point(const double (*P)[3], double gii, double gij, double* X, double* N,
                                           double* f4) {
  const double e1m = 1.0 - gii, e1p = 1.0 + gii, e2m = 1.0 - gij, e2p = 1.0 + gij;
  f4[0] = 0.25 * e1m * e2m; f4[1] = 0.25 * e1p * e2m; f4[2] = 0.25 * e1p * e2p; f4[3] = 0.25 * e1m * e2p;
  double KS[3], ET[3];
  for (int k = 0; k < 3; ++k) {
    X[k] = f4[0] * P[0][k] + f4[1] * P[1][k] + f4[2] * P[2][k] + f4[3] * P[3][k];
    KS[k] = 0.25 * (-e2m * P[0][k] + e2m * P[1][k] + e2p * P[2][k] - e2p * P[3][k]);
    ET[k] = 0.25 * (-e1m * P[0][k] - e1p * P[1][k] + e1p * P[2][k] + e1m * P[3][k]);
  }
  N[0] = KS[1] * ET[2] - ET[1] * KS[2];
  N[1] = ET[0] * KS[2] - KS[0] * ET[2];
  N[2] = KS[0] * ET[1] - ET[0] * KS[1];
}

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------
__global__ void k_geometry(int ne, const double* __restrict__ xyz, const int* __restrict__ etype,
                           const int* __restrict__ con, const int* __restrict__ wall_of_elem,
                           const double* __restrict__ normMul, ElemGeom* __restrict__ g) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ne) return;
  ElemGeom G;
  G.type = etype[p];
  G.nno = (G.type == AGB_TRI) ? 3 : 4;
  for (int k = 0; k < 4; ++k) G.con[k] = (k < G.nno) ? con[4 * p + k] : -1;
  for (int k = 0; k < 4; ++k)
    for (int i = 0; i < 3; ++i) G.v[k][i] = (k < G.nno) ? xyz[3 * G.con[k] + i] : 0.0;
  const double v1[3] = {G.v[1][0] - G.v[0][0], G.v[1][1] - G.v[0][1], G.v[1][2] - G.v[0][2]};
  const double v2[3] = {G.v[2][0] - G.v[0][0], G.v[2][1] - G.v[0][1], G.v[2][2] - G.v[0][2]};
  double n[3] = {v1[1] * v2[2] - v1[2] * v2[1], -v1[0] * v2[2] + v1[2] * v2[0], v1[0] * v2[1] - v1[1] * v2[0]};
  const double d = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  for (int i = 0; i < 3; ++i) G.n[i] = n[i] / d;
  if (G.type == AGB_TRI) {
    G.area = agb_sing::heron(G.v[0], G.v[1], G.v[2]);
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += (1.0 / 3.0) * G.v[k][i];
      G.c[i] = s;
    }
  } else {
    // 8x8 Gauss area (CalElementArea, Gauss index 4)
    const int ng1 = cGaussNg1[3], ng2 = cGaussNg2[3];
    double integral = 0.0;
    for (int i = ng1; i <= ng2; ++i)
      for (int j = ng1; j <= ng2; ++j) {
        double X[3], N[3], f4[4];
        quad_point(G.v, cGaussGi[i - 1], cGaussGi[j - 1], X, N, f4);
        const double ajac = cGaussOme[i - 1] * cGaussOme[j - 1] * sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        for (int s = 0; s < 4; ++s) integral += ajac * f4[s];
      }
    G.area = integral;
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s += 0.25 * G.v[k][i];
      G.c[i] = s;
    }
  }
  G.wall = wall_of_elem[p];
  G.multi = normMul[G.wall];
  g[p] = G;
}

cudaError_t launch_geometry(int ne, const double* xyz, const int* etype, const int* con, const int* wall_of_elem,
                            const double* normMul, ElemGeom* geom, cudaStream_t s) {
  if (ne <= 0) return cudaSuccess;
  k_geometry<<<cdiv(ne, 128), 128, 0, s>>>(ne, xyz, etype, con, wall_of_elem, normMul, geom);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// quadrature points of the triangles, [q][ldp]
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_expand(int ne, int ldp, int Q, const ElemGeom* __restrict__ geom, const double* __restrict__ rl,
                         const double* __restrict__ rw, QPt<T>* __restrict__ pts, T* __restrict__ src,
                         T* __restrict__ nrm) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ldp) return;
  if (p >= ne) {
    for (int q = 0; q < Q; ++q) pts[(int64_t)q * ldp + p] = QPt<T>{T(0), T(0), T(0), T(0)};
    for (int i = 0; i < 3; ++i) { src[i * ldp + p] = T(0); nrm[i * ldp + p] = T(0); }
    return;
  }
  const ElemGeom& G = geom[p];
  for (int i = 0; i < 3; ++i) { src[i * ldp + p] = (T)G.c[i]; nrm[i * ldp + p] = (T)(G.multi * G.n[i]); }
  for (int q = 0; q < Q; ++q) {
    const double l1 = rl[q], l2 = rl[Q + q], l3 = rl[2 * Q + q];
    QPt<T> P;
    if (G.type == AGB_TRI) {
      P.x = (T)(l1 * G.v[0][0] + l2 * G.v[1][0] + l3 * G.v[2][0]);
      P.y = (T)(l1 * G.v[0][1] + l2 * G.v[1][1] + l3 * G.v[2][1]);
      P.z = (T)(l1 * G.v[0][2] + l2 * G.v[1][2] + l3 * G.v[2][2]);
      P.w = (T)(rw[q] * G.area);
    } else {
      P.x = P.y = P.z = P.w = T(0);
    }
    pts[(int64_t)q * ldp + p] = P;
  }
}

template <typename T>
cudaError_t launch_expand_points(int ne, int ldp, const ElemGeom* geom, const RuleDev& rule, QPt<T>* pts, T* src,
                                 T* nrm, cudaStream_t s) {
  k_expand<T><<<cdiv(ldp, 128), 128, 0, s>>>(ne, ldp, rule.Q, geom, rule.l, rule.w, pts, src, nrm);
  return cudaGetLastError();
}
template cudaError_t launch_expand_points<float>(int, int, const ElemGeom*, const RuleDev&, QPt<float>*, float*, float*,
                                                 cudaStream_t);
template cudaError_t launch_expand_points<double>(int, int, const ElemGeom*, const RuleDev&, QPt<double>*, double*,
                                                  double*, cudaStream_t);

// ---------------------------------------------------------------------------
// Stokes single layer, regular quadrature, tiled (the hot kernel)
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T rsq(T v);
template <> __device__ __forceinline__ float rsq<float>(float v) { return rsqrtf(v); }
template <> __device__ __forceinline__ double rsq<double>(double v) { return rsqrt(v); }

template <typename T> struct StkTile;
template <> struct StkTile<float> { static constexpr int RS = 8; static constexpr int NW = 8; };
template <> struct StkTile<double> { static constexpr int RS = 4; static constexpr int NW = 8; };

// PACKED: the 3x3 blocks are symmetric, so the matrix is stored with six
// values per block in the layout of pk_idx (lda = 6 x the plane length), 2/3
// of the bytes of the full row-major A[3i+a][b ne + j].
template <typename T, bool PACKED = false>
__global__ void __launch_bounds__(StkTile<T>::NW * 32) k_stokes_G(int ne, int Q, int ldp, const QPt<T>* __restrict__ pts,
                                                                 const T* __restrict__ src, const T* __restrict__ colscale,
                                                                 int src_per_cta, T* __restrict__ A, int64_t lda) {
  constexpr int RS = StkTile<T>::RS, NW = StkTile<T>::NW;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  QPt<T>* sp = reinterpret_cast<QPt<T>*>(smem_raw);
  const int j0 = blockIdx.x * 32;
  for (int t = threadIdx.x; t < Q * 32; t += NW * 32) sp[t] = pts[(int64_t)(t >> 5) * ldp + j0 + (t & 31)];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = j0 + lane;
  const T scale = (j < ne) ? colscale[j] : T(0);
  const int sBeg = blockIdx.y * src_per_cta;
  const int sEnd = min(ne, sBeg + src_per_cta);
  const T* sxp = src;
  const T* syp = src + ldp;
  const T* szp = src + 2 * ldp;
  for (int ib = sBeg + warp * RS; ib < sEnd; ib += NW * RS) {
    T sx[RS], sy[RS], sz[RS];
#pragma unroll
    for (int r = 0; r < RS; ++r) {
      const int i = min(ib + r, sEnd - 1);
      sx[r] = sxp[i]; sy[r] = syp[i]; sz[r] = szp[i];
    }
    T acc[RS][7];
#pragma unroll
    for (int r = 0; r < RS; ++r)
#pragma unroll
      for (int c = 0; c < 7; ++c) acc[r][c] = T(0);
#pragma unroll 2
    for (int q = 0; q < Q; ++q) {
      const QPt<T> p = sp[q * 32 + lane];
#pragma unroll
      for (int r = 0; r < RS; ++r) {
        const T rx = p.x - sx[r], ry = p.y - sy[r], rz = p.z - sz[r];
        const T r2 = rx * rx + ry * ry + rz * rz;
        const T ir = rsq<T>(r2);
        const T wi = p.w * ir;
        const T wi3 = wi * (ir * ir);
        acc[r][0] += wi;
        const T ax = wi3 * rx, ay = wi3 * ry;
        acc[r][1] += ax * rx;
        acc[r][2] += ax * ry;
        acc[r][3] += ax * rz;
        acc[r][4] += ay * ry;
        acc[r][5] += ay * rz;
        acc[r][6] += (wi3 * rz) * rz;
      }
    }
    if (j < ne) {
#pragma unroll
      for (int r = 0; r < RS; ++r) {
        const int i = ib + r;
        if (i < sEnd) {
          const T gxx = scale * (acc[r][0] + acc[r][1]), gxy = scale * acc[r][2], gxz = scale * acc[r][3];
          const T gyy = scale * (acc[r][0] + acc[r][4]), gyz = scale * acc[r][5];
          const T gzz = scale * (acc[r][0] + acc[r][6]);
          if (PACKED) {
            const int pl = (int)(lda / 6);  // plane length of the packed layout
            T* pr = A + pk_idx(i, 0, j, pl);
            pr[0] = gxx; pr[64] = gxy; pr[128] = gxz; pr[192] = gyy; pr[256] = gyz; pr[320] = gzz;
          } else {
            T* r0 = A + (int64_t)(3 * i) * lda + j;
            T* r1 = r0 + lda;
            T* r2p = r1 + lda;
            r0[0] = gxx; r0[ne] = gxy; r0[2 * ne] = gxz;
            r1[0] = gxy; r1[ne] = gyy; r1[2 * ne] = gyz;
            r2p[0] = gxz; r2p[ne] = gyz; r2p[2 * ne] = gzz;
          }
        }
      }
    }
  }
}

template <typename T>
cudaError_t launch_stokes_G(int ne, int Q, int ldp, const QPt<T>* pts, const T* src, const T* colscale, T* A,
                            int64_t lda, cudaStream_t s) {
  constexpr int NW = StkTile<T>::NW;
  const size_t smem = (size_t)Q * 32 * sizeof(QPt<T>);
  cudaError_t e = cudaFuncSetAttribute(k_stokes_G<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int tiles = (int)cdiv(ne, 32);
  const int want = 152 * 6;
  int ychunks = std::max(1, std::min((want + tiles - 1) / tiles, (ne + 63) / 64));
  const int spc = (int)cdiv(ne, ychunks);
  ychunks = (int)cdiv(ne, spc);
  dim3 grid(tiles, ychunks);
  k_stokes_G<T><<<grid, NW * 32, smem, s>>>(ne, Q, ldp, pts, src, colscale, spc, A, lda);
  return cudaGetLastError();
}
template cudaError_t launch_stokes_G<float>(int, int, int, const QPt<float>*, const float*, const float*, float*, int64_t,
                                            cudaStream_t);

cudaError_t launch_stokes_G_packed(int ne, int Q, int ldp, int pldp, const QPt<float>* pts, const float* src,
                                   const float* colscale, float* Ap, cudaStream_t s) {
  constexpr int NW = StkTile<float>::NW;
  const size_t smem = (size_t)Q * 32 * sizeof(QPt<float>);
  cudaError_t e = cudaFuncSetAttribute(k_stokes_G<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int tiles = (int)cdiv(ne, 32);
  const int want = 152 * 6;
  int ychunks = std::max(1, std::min((want + tiles - 1) / tiles, (ne + 63) / 64));
  const int spc = (int)cdiv(ne, ychunks);
  ychunks = (int)cdiv(ne, spc);
  k_stokes_G<float, true><<<dim3(tiles, ychunks), NW * 32, smem, s>>>(ne, Q, ldp, pts, src, colscale, spc, Ap,
                                                                       6 * (int64_t)pldp);
  return cudaGetLastError();
}

__global__ void k_stokes_self_packed(int ne, int ldp, const ElemGeom* __restrict__ geom, double diff,
                                     float* __restrict__ Ap) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ne) return;
  const ElemGeom& G = geom[p];
  double g[6];
  agb_sing::tri_stokes(G.v[0], G.v[1], G.v[2], G.area, 4, g);
  const double sc = -G.multi / diff;
  float* pr = Ap + pk_idx(p, 0, p, ldp);
  for (int c = 0; c < 6; ++c) pr[c * 64] = (float)(sc * g[c]);
}
cudaError_t launch_stokes_self_packed(int ne, int ldp, const ElemGeom* geom, double diff, float* Ap, cudaStream_t s) {
  k_stokes_self_packed<<<cdiv(ne, 64), 64, 0, s>>>(ne, ldp, geom, diff, Ap);
  return cudaGetLastError();
}
template cudaError_t launch_stokes_G<double>(int, int, int, const QPt<double>*, const double*, const double*, double*,
                                             int64_t, cudaStream_t);

// Self-element blocks (analytic, FP64)
template <typename T>
__global__ void k_stokes_self(int ne, const ElemGeom* __restrict__ geom, double diff, T* __restrict__ A, int64_t lda) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ne) return;
  const ElemGeom& G = geom[p];
  double g[6];
  if (G.type == AGB_TRI) agb_sing::tri_stokes(G.v[0], G.v[1], G.v[2], G.area, 4, g);
  else agb_sing::quad_stokes(G.v, 5, g);
  const double sc = -G.multi / diff;
  T* r0 = A + (int64_t)(3 * p) * lda + p;
  T* r1 = r0 + lda;
  T* r2 = r1 + lda;
  r0[0] = (T)(sc * g[0]); r0[ne] = (T)(sc * g[1]); r0[2 * ne] = (T)(sc * g[2]);
  r1[0] = (T)(sc * g[1]); r1[ne] = (T)(sc * g[3]); r1[2 * ne] = (T)(sc * g[4]);
  r2[0] = (T)(sc * g[2]); r2[ne] = (T)(sc * g[4]); r2[2 * ne] = (T)(sc * g[5]);
}
template <typename T>
cudaError_t launch_stokes_self(int ne, const ElemGeom* geom, double diff, T* A, int64_t lda, cudaStream_t s) {
  k_stokes_self<T><<<cdiv(ne, 64), 64, 0, s>>>(ne, geom, diff, A, lda);
  return cudaGetLastError();
}
template cudaError_t launch_stokes_self<float>(int, const ElemGeom*, double, float*, int64_t, cudaStream_t);
template cudaError_t launch_stokes_self<double>(int, const ElemGeom*, double, double*, int64_t, cudaStream_t);

// ---------------------------------------------------------------------------
// Stokes right-hand sides with the rigid-body free term
// ---------------------------------------------------------------------------
__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// index of the symmetric pair (a, b) in {xx, xy, xz, yy, yz, zz}
__device__ __forceinline__ int sym_ab(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}

template <typename T>
__global__ void k_stokes_rhs(StokesRhsArgs a) {
  // barycentric coordinates of the rule in T (the points themselves come from
  // the expanded table, computed there in FP64 and rounded once)
  __shared__ T sL[3][AGB_MAX_Q];
  for (int t = threadIdx.x; t < 3 * a.Q; t += blockDim.x) sL[t / a.Q][t % a.Q] = (T)a.rule_l[t];
  __syncthreads();
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int i = warp;
  if (i >= a.ne) return;
  const QPt<T>* __restrict__ pts = static_cast<const QPt<T>*>(a.pts);
  const ElemGeom& Gi = a.geom[i];
  const T sx = (T)Gi.c[0], sy = (T)Gi.c[1], sz = (T)Gi.c[2];
  const int Q = a.Q;
  double acc[AGB_MAX_RHS][3];
  for (int c = 0; c < AGB_MAX_RHS; ++c) acc[c][0] = acc[c][1] = acc[c][2] = 0.0;
  // (A) T u over the elements carrying nonzero velocity (self element has T = 0)
  for (int t = lane; t < a.na; t += 32) {
    const int e = a.active[t];
    if (e == i) continue;
    const ElemGeom& G = a.geom[e];
    const T nx = (T)(G.multi * G.n[0]), ny = (T)(G.multi * G.n[1]), nz = (T)(G.multi * G.n[2]);
    // The stresslet applied to the linearly interpolated nodal velocities,
    // int cn (r . u) r_a with u = sum_k L_k u_k, is linear in the u_k:
    // accumulate the 18 moments m[k][ab] = int cn L_k r_a r_b over the element
    // once and contract them with every right-hand side's nodal velocities
    // afterwards (42 operations per point instead of ~110 for six fields).
    T mom[3][6];
#pragma unroll
    for (int kk = 0; kk < 3; ++kk)
#pragma unroll
      for (int s6 = 0; s6 < 6; ++s6) mom[kk][s6] = T(0);
    for (int q = 0; q < Q; ++q) {
      const QPt<T> P = pts[(int64_t)q * a.ldp + e];
      const T w = P.w;
      const T rx = P.x - sx, ry = P.y - sy, rz = P.z - sz;
      const T r2 = rx * rx + ry * ry + rz * rz;
      const T ir = rsq<T>(r2);
      const T ir2 = ir * ir;
      const T cn = T(-6) * w * (rx * nx + ry * ny + rz * nz) * (ir2 * ir2 * ir);
      const T rr[6] = {rx * rx, rx * ry, rx * rz, ry * ry, ry * rz, rz * rz};
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) {
        const T ck = cn * sL[kk][q];
#pragma unroll
        for (int s6 = 0; s6 < 6; ++s6) mom[kk][s6] += ck * rr[s6];
      }
    }
#pragma unroll
    for (int c = 0; c < AGB_MAX_RHS; ++c) {
      if (c < a.k) {
        T uv[3][3];  // [comp][local node] of right-hand side c
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) uv[b][kk] = (T)a.u[((int64_t)c * 3 + b) * a.nnodes + G.con[kk]];
#pragma unroll
        for (int ai = 0; ai < 3; ++ai) {
          T pe = T(0);
#pragma unroll
          for (int kk = 0; kk < 3; ++kk)
#pragma unroll
            for (int b = 0; b < 3; ++b) pe += mom[kk][sym_ab(ai, b)] * uv[b][kk];
          acc[c][ai] += (double)pe;
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < AGB_MAX_RHS; ++c)
#pragma unroll
    for (int b = 0; b < 3; ++b) acc[c][b] = wsum(acc[c][b]);
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < AGB_MAX_RHS; ++c)
      if (c < a.k)
        for (int b = 0; b < 3; ++b) a.rhs[(int64_t)c * 3 * a.ne + 3 * i + b] = acc[c][b];
  }
}

// Free term of the rows whose own element carries velocity: c_aa(i) =
// -sum over all elements e != i of int_e T_aa(x_i, y) dy, accumulated in FP64
// from per-element sums.  Grid: (active row, element chunk); partials per
// (row, chunk) are reduced in chunk order by k_stokes_freeterm_apply.
constexpr int FT_CHUNK = 2048;
template <typename T>
__global__ void __launch_bounds__(256) k_stokes_freeterm(StokesRhsArgs a, double* __restrict__ partial) {
  const int t = blockIdx.x;  // index into the active list
  const int i = a.active[t];
  const int e0 = blockIdx.y * FT_CHUNK;
  const QPt<T>* __restrict__ pts = static_cast<const QPt<T>*>(a.pts);
  const ElemGeom& Gi = a.geom[i];
  const T sx = (T)Gi.c[0], sy = (T)Gi.c[1], sz = (T)Gi.c[2];
  const int Q = a.Q;
  double ca[3] = {0.0, 0.0, 0.0};
  for (int e = e0 + threadIdx.x; e < min(a.ne, e0 + FT_CHUNK); e += blockDim.x) {
    if (e == i) continue;
    const ElemGeom& G = a.geom[e];
    const T nx = (T)(G.multi * G.n[0]), ny = (T)(G.multi * G.n[1]), nz = (T)(G.multi * G.n[2]);
    T s0 = T(0), s1 = T(0), s2 = T(0);
    for (int q = 0; q < Q; ++q) {
      const QPt<T> P = pts[(int64_t)q * a.ldp + e];
      const T w = P.w;
      const T rx = P.x - sx, ry = P.y - sy, rz = P.z - sz;
      const T r2 = rx * rx + ry * ry + rz * rz;
      const T ir = rsq<T>(r2);
      const T ir2 = ir * ir;
      const T cn = T(-6) * w * (rx * nx + ry * ny + rz * nz) * (ir2 * ir2 * ir);
      s0 += cn * rx * rx;
      s1 += cn * ry * ry;
      s2 += cn * rz * rz;
    }
    ca[0] += (double)s0; ca[1] += (double)s1; ca[2] += (double)s2;
  }
  __shared__ double sh[3][256];
  for (int b = 0; b < 3; ++b) sh[b][threadIdx.x] = ca[b];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int b = 0; b < 3; ++b) sh[b][threadIdx.x] += sh[b][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 3) partial[((int64_t)t * gridDim.y + blockIdx.y) * 3 + threadIdx.x] = sh[threadIdx.x][0];
}
// rhs(3i+b, c) += shpf * c_bb(i) * sum over the nodes of element i of u_b
__global__ void k_stokes_freeterm_apply(StokesRhsArgs a, const double* __restrict__ partial, int nchunks) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.na) return;
  const int i = a.active[t];
  const ElemGeom& Gi = a.geom[i];
  double ca[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < nchunks; ++k)
    for (int b = 0; b < 3; ++b) ca[b] += partial[((int64_t)t * nchunks + k) * 3 + b];
  const double shpf = (Gi.type == AGB_TRI) ? 1.0 / 3.0 : 0.25;
  for (int c = 0; c < a.k; ++c)
    for (int b = 0; b < 3; ++b) {
      double su = 0.0;
      for (int kk = 0; kk < Gi.nno; ++kk) su += a.u[((int64_t)c * 3 + b) * a.nnodes + Gi.con[kk]];
      a.rhs[(int64_t)c * 3 * a.ne + 3 * i + b] += shpf * (-ca[b]) * su;
    }
}

template <typename T>
cudaError_t launch_stokes_rhs(const StokesRhsArgs& a, cudaStream_t s) {
  const int threads = 128;
  k_stokes_rhs<T><<<cdiv((int64_t)a.ne * 32, threads), threads, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || a.na == 0) return e;
  const int nchunks = (int)cdiv(a.ne, FT_CHUNK);
  double* partial = nullptr;
  e = cudaMallocAsync(&partial, (size_t)a.na * nchunks * 3 * sizeof(double), s);
  if (e != cudaSuccess) return e;
  k_stokes_freeterm<T><<<dim3(a.na, nchunks), 256, 0, s>>>(a, partial);
  k_stokes_freeterm_apply<<<cdiv(a.na, 128), 128, 0, s>>>(a, partial, nchunks);
  e = cudaGetLastError();
  cudaFreeAsync(partial, s);
  return e;
}
template cudaError_t launch_stokes_rhs<float>(const StokesRhsArgs&, cudaStream_t);
template cudaError_t launch_stokes_rhs<double>(const StokesRhsArgs&, cudaStream_t);

// ---------------------------------------------------------------------------
// Laplace all-Dirichlet system, FP64: warp per collocation row
// ---------------------------------------------------------------------------
__global__ void k_laplace_system(LaplaceArgs a) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= a.ne) return;
  const ElemGeom& Gi = a.geom[i];
  const double s[3] = {Gi.c[0], Gi.c[1], Gi.c[2]};
  const double fpi = 0.25 / AGB_PI;
  double hu[AGB_MAX_RHS], hs = 0.0;
  for (int c = 0; c < AGB_MAX_RHS; ++c) hu[c] = 0.0;
  for (int j = lane; j < a.ne; j += 32) {
    const ElemGeom& G = a.geom[j];
    double g = 0.0;
    if (j == i) {
      g = (G.type == AGB_TRI) ? agb_sing::tri_laplace(G.v[0], G.v[1], G.v[2], G.area, 4)
                              : agb_sing::quad_laplace(G.v, 5);
    } else if (G.type == AGB_TRI) {
      const double n[3] = {G.multi * G.n[0], G.multi * G.n[1], G.multi * G.n[2]};
      double ul[AGB_MAX_RHS][3];
      for (int c = 0; c < a.k; ++c)
        for (int kk = 0; kk < 3; ++kk) ul[c][kk] = a.u[(int64_t)c * a.nnodes + G.con[kk]];
      for (int q = 0; q < a.Q; ++q) {
        const double l1 = a.rule_l[q], l2 = a.rule_l[a.Q + q], l3 = a.rule_l[2 * a.Q + q];
        const double x = l1 * G.v[0][0] + l2 * G.v[1][0] + l3 * G.v[2][0];
        const double y = l1 * G.v[0][1] + l2 * G.v[1][1] + l3 * G.v[2][1];
        const double z = l1 * G.v[0][2] + l2 * G.v[1][2] + l3 * G.v[2][2];
        const double RX = s[0] - x, RY = s[1] - y, RZ = s[2] - z;
        const double RA = sqrt(RX * RX + RY * RY + RZ * RZ);
        const double FG = fpi / RA;
        const double FH = (RX * n[0] + RY * n[1] + RZ * n[2]) / (RA * RA) * FG;
        const double w = a.rule_w[q] * G.area;
        g += w * FG;
        hs += w * FH;
        for (int c = 0; c < a.k; ++c) hu[c] += w * FH * (l1 * ul[c][0] + l2 * ul[c][1] + l3 * ul[c][2]);
      }
    } else {
      // Quad_BEMIntNum: uniform subdivision >= 2x2 by edge length, ng x ng Gauss
      const int ng1 = cGaussNg1[a.iqud - 1], ng2 = cGaussNg2[a.iqud - 1];
      auto dist = [&](int p, int q) {
        const double dx = G.v[p][0] - G.v[q][0], dy = G.v[p][1] - G.v[q][1], dz = G.v[p][2] - G.v[q][2];
        return sqrt(dx * dx + dy * dy + dz * dz);
      };
      const double d13 = fmax(dist(0, 1), dist(2, 3)), d24 = fmax(dist(1, 2), dist(3, 0));
      const int ndx = max(2, (int)(d13 / 1.0 + 0.5)), nde = max(2, (int)(d24 / 1.0 + 0.5));
      double ul[AGB_MAX_RHS][4];
      for (int c = 0; c < a.k; ++c)
        for (int kk = 0; kk < 4; ++kk) ul[c][kk] = a.u[(int64_t)c * a.nnodes + G.con[kk]];
      for (int ix = 1; ix <= ndx; ++ix)
        for (int ie = 1; ie <= nde; ++ie) {
          const double aa = -1.0 + (ix - 1) * 2.0 / ndx, bb = -1.0 + ix * 2.0 / ndx;
          const double cc = -1.0 + (ie - 1) * 2.0 / nde, dd = -1.0 + ie * 2.0 / nde;
          const double dex = 0.25 * (bb - aa) * (dd - cc);
          for (int gi = ng1; gi <= ng2; ++gi)
            for (int gj = ng1; gj <= ng2; ++gj) {
              const double gii = aa + 0.5 * (cGaussGi[gi - 1] + 1.0) * (bb - aa);
              const double gij = cc + 0.5 * (cGaussGi[gj - 1] + 1.0) * (dd - cc);
              double X[3], N[3], f4[4];
              quad_point(G.v, gii, gij, X, N, f4);
              const double aj = 1.0 / sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
              const double n1 = G.multi * N[0] * aj, n2 = G.multi * N[1] * aj, n3 = G.multi * N[2] * aj;
              const double jac = dex * cGaussOme[gi - 1] * cGaussOme[gj - 1] / aj;
              const double RX = s[0] - X[0], RY = s[1] - X[1], RZ = s[2] - X[2];
              const double RA = sqrt(RX * RX + RY * RY + RZ * RZ);
              const double FG = fpi / RA;
              const double FH = (RX * n1 + RY * n2 + RZ * n3) / (RA * RA) * FG;
              g += FG * jac;
              hs += FH * jac;
              for (int c = 0; c < a.k; ++c)
                hu[c] += FH * jac * (f4[0] * ul[c][0] + f4[1] * ul[c][1] + f4[2] * ul[c][2] + f4[3] * ul[c][3]);
            }
        }
    }
    if (a.A) a.A[(int64_t)i * a.lda + j] = G.multi / a.diff * g;
  }
  hs = wsum(hs);
  for (int c = 0; c < a.k; ++c) hu[c] = wsum(hu[c]);
  if (lane == 0) {
    const double cfree = -hs;
    const double shpf = (Gi.type == AGB_TRI) ? 1.0 / 3.0 : 0.25;
    for (int c = 0; c < a.k; ++c) {
      double su = 0.0;
      for (int kk = 0; kk < Gi.nno; ++kk) su += a.u[(int64_t)c * a.nnodes + Gi.con[kk]];
      a.rhs[(int64_t)c * a.ne + i] = -(hu[c] + shpf * cfree * su);
    }
  }
}

cudaError_t launch_laplace_system(const LaplaceArgs& a, cudaStream_t s) {
  k_laplace_system<<<cdiv((int64_t)a.ne * 32, 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// force and torque per right-hand side (CalFluxIntegralSingleWall,
// getTorqueIntegrateFluxes): fixed-order block reduction
// ---------------------------------------------------------------------------
__global__ void k_force_torque(int ne, const ElemGeom* __restrict__ geom, const double* __restrict__ x, int wall,
                               double* __restrict__ ft) {
  const int c = blockIdx.x;
  __shared__ double sh[6][256];
  double a[6] = {0, 0, 0, 0, 0, 0};
  const double* xc = x + (int64_t)c * 3 * ne;
  for (int p = threadIdx.x; p < ne; p += blockDim.x) {
    const ElemGeom& G = geom[p];
    if (G.wall != wall) continue;
    const double q[3] = {xc[p], xc[ne + p], xc[2 * ne + p]};
    double r[3] = {0, 0, 0};
    for (int k = 0; k < G.nno; ++k)
      for (int j = 0; j < 3; ++j) r[j] += G.v[k][j];
    for (int j = 0; j < 3; ++j) r[j] /= (double)G.nno;
    a[0] += G.area * q[0]; a[1] += G.area * q[1]; a[2] += G.area * q[2];
    a[3] += G.area * (r[1] * q[2] - r[2] * q[1]);
    a[4] += G.area * (-r[0] * q[2] + r[2] * q[0]);
    a[5] += G.area * (r[0] * q[1] - r[1] * q[0]);
  }
  for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 6) ft[c * 6 + threadIdx.x] = sh[threadIdx.x][0];
}

cudaError_t launch_force_torque(int ne, int k, const ElemGeom* geom, const double* x, int wall_index, double* ft,
                                cudaStream_t s) {
  k_force_torque<<<k, 256, 0, s>>>(ne, geom, x, wall_index, ft);
  return cudaGetLastError();
}

}  // namespace agb
