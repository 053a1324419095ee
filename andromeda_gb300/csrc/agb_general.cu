// General assembly path (FP64): the integral matrices of every source row --
// the drop-in of CoR_Integrals (lib_int.f90:4, sdFormIntegralMatrices :225)
// and CoR_Integrals_Stokes (lib_Stokes.f90:2664, sdFormIntegralMatricesStokes
// :1391) -- and the BC routing into a dense system (sdSetUpSysMrhsM_CRS
// lib_CRS.f90:148; formUrow/formQrow lib_StokesFull.f90:4,94).
//
// Two kernels per chunk of source rows:
//   k_gen_elem  one thread per (row, element): the element integral (regular
//               quadrature or analytic self element) into a scratch slab;
//   k_gen_row   one CTA per row: gathers the nodal (H/T) contributions of the
//               elements around each node in ascending element order (the
//               reference's accumulation order), copies the element (G)
//               columns, reduces the row sums and applies the rigid-body free
//               term / pressure correction of sdIntRowU/Q(Stokes), and records
//               the reference's self-check residual of the row.
#include "agb_general.cuh"
#include "quad_tables.h"

#include <algorithm>

namespace agb {
static __constant__ double gtGi[156];
static __constant__ double gtOme[156];
static __constant__ int gtNg1[8];
static __constant__ int gtNg2[8];
}  // namespace agb

#include "agb_elements.cuh"

namespace agb {

cudaError_t upload_general_tables() {
  cudaError_t e = cudaMemcpyToSymbol(gtGi, agb_tables::kGaussGi, sizeof(agb_tables::kGaussGi));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(gtOme, agb_tables::kGaussOme, sizeof(agb_tables::kGaussOme));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(gtNg1, agb_tables::kGaussNg1, sizeof(agb_tables::kGaussNg1));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(gtNg2, agb_tables::kGaussNg2, sizeof(agb_tables::kGaussNg2));
  return e;
}

static inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

constexpr int NV_LAP = 5;   // g, h[4]
constexpr int NV_STK = 45;  // G[6], prG[3], T[6][4], prT[3][4]

struct GenArgs {
  int kind, nn, nq, nsp, Q, iqud;
  const ElemGeom* geom;
  const double* xyz;
  const double* rl;
  const double* rw;
  const int* nodeList;
  const int* posOfNode;
  const int* adj_ptr;
  const int* adj_p;
  const int* adj_k;
  IntegOpt opt;
};

template <int STK>
__global__ void k_gen_elem(GenArgs a, int row0, int nrows, double* __restrict__ E) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int rl = blockIdx.y;
  if (p >= a.nq || rl >= nrows) return;
  const int r = row0 + rl;
  const ElemGeom& G = a.geom[p];
  double s[3];
  int isrc = 0;
  if (r < a.nn) {
    const int g = a.nodeList[r];
    for (int i = 0; i < 3; ++i) s[i] = a.xyz[3 * g + i];
    for (int k = 0; k < G.nno; ++k)
      if (G.con[k] == g) isrc = k + 1;
  } else {
    const int ps = r - a.nn;
    const ElemGeom& S = a.geom[ps];
    for (int i = 0; i < 3; ++i) s[i] = S.c[i];
    if (ps == p) isrc = (G.type == AGB_TRI) ? 4 : 5;
  }
  constexpr int NV = STK ? NV_STK : NV_LAP;
  double* out = E + ((int64_t)rl * a.nq + p) * NV;
  if constexpr (STK) {
    StkElem o;
    stk_element(G, s, isrc, a.rl, a.rw, a.Q, a.iqud, a.opt, o);
    if (isrc && r >= a.nn) {
      // sdIntRowQStokes adds no pressure terms of the self element (lib_Stokes.f90:1747-1760)
      for (int k = 0; k < 3; ++k) {
        o.prG[k] = 0.0;
        for (int j = 0; j < 4; ++j) o.prT[k][j] = 0.0;
      }
    }
    int t = 0;
    for (int k = 0; k < 6; ++k) out[t++] = o.G[k];
    for (int k = 0; k < 3; ++k) out[t++] = o.prG[k];
    for (int k = 0; k < 6; ++k)
      for (int j = 0; j < 4; ++j) out[t++] = o.T[k][j];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 4; ++j) out[t++] = o.prT[k][j];
  } else {
    LapElem o = lap_element(G, s, isrc, a.rl, a.rw, a.Q, a.iqud, a.opt);
    out[0] = o.g;
    for (int k = 0; k < 4; ++k) out[1 + k] = o.h[k];
  }
}

constexpr int ROW_THREADS = 256;
constexpr int NSUM = 12;

__device__ __forceinline__ void block_sums(double (&v)[NSUM], double (*sh)[ROW_THREADS]) {
  for (int k = 0; k < NSUM; ++k) sh[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int st = ROW_THREADS / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < NSUM; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + st];
    __syncthreads();
  }
}

template <int STK>
__global__ void __launch_bounds__(ROW_THREADS) k_gen_row(GenArgs a, int row0, const double* __restrict__ E,
                                                         double* __restrict__ T, double* __restrict__ Gm,
                                                         double* __restrict__ err_row) {
  __shared__ double sh[NSUM][ROW_THREADS];
  constexpr int NV = STK ? NV_STK : NV_LAP;
  constexpr int NT = STK ? 9 : 1;  // nodal components
  const int rl = blockIdx.x;
  const int r = row0 + rl;
  const int64_t nn = a.nn, nq = a.nq, nsp = a.nsp;
  const double* Er = E + (int64_t)rl * nq * NV;
  double v[NSUM];
  for (int k = 0; k < NSUM; ++k) v[k] = 0.0;
  // element columns (G) and, for u-rows, the G.n identity sums
  for (int p = threadIdx.x; p < a.nq; p += ROW_THREADS) {
    const double* e = Er + (int64_t)p * NV;
    const ElemGeom& G = a.geom[p];
    const double m = G.multi;
    if constexpr (STK) {
      for (int c = 0; c < 9; ++c) Gm[((int64_t)c * nsp + r) * nq + p] = e[c];
      if (r < a.nn) {
        const double* n = G.n;
        v[6] += -e[0] * n[0] * m - e[1] * n[1] * m - e[2] * n[2] * m;
        v[7] += -e[1] * n[0] * m - e[3] * n[1] * m - e[4] * n[2] * m;
        v[8] += -e[2] * n[0] * m - e[4] * n[1] * m - e[5] * n[2] * m;
      }
    } else {
      Gm[(int64_t)r * nq + p] = e[0];
      if (r < a.nn)
        for (int j = 0; j < 3; ++j) v[3 + j] += e[0] * G.n[j] * m;
    }
  }
  // nodal columns: gather over the elements around each node, ascending order
  for (int j = threadIdx.x; j < a.nn; j += ROW_THREADS) {
    double acc[NT];
    for (int c = 0; c < NT; ++c) acc[c] = 0.0;
    for (int t = a.adj_ptr[j]; t < a.adj_ptr[j + 1]; ++t) {
      const double* e = Er + (int64_t)a.adj_p[t] * NV;
      const int k = a.adj_k[t];
      if constexpr (STK) {
        for (int c = 0; c < 6; ++c) acc[c] += e[9 + c * 4 + k];
        for (int c = 0; c < 3; ++c) acc[6 + c] += e[33 + c * 4 + k];
      } else {
        acc[0] += e[1 + k];
      }
    }
    for (int c = 0; c < NT; ++c) T[((int64_t)c * nsp + r) * nn + j] = acc[c];
    if constexpr (STK) {
      v[0] += acc[0]; v[1] += acc[3]; v[2] += acc[5];   // diagonal sums
      v[3] += acc[1]; v[4] += acc[4]; v[5] += acc[2];   // xy, yz, xz sums
      v[9] += acc[6]; v[10] += acc[7]; v[11] += acc[8];  // pressure sums
    } else {
      v[0] += acc[0];
      const int g = a.nodeList[j];
      for (int q = 0; q < 3; ++q) v[6 + q] += acc[0] * a.xyz[3 * g + q];
    }
  }
  block_sums(v, sh);
  if (threadIdx.x != 0) return;
  __threadfence_block();
  double S[NSUM];
  for (int k = 0; k < NSUM; ++k) S[k] = sh[k][0];
  if constexpr (STK) {
    double err = -9.99;
    if (r < a.nn) {
      // sdIntRowUStokes: c_aa = -sum T_aa added at the source node
      const int jp = r;  // the source node of u-row r is sd node r
      T[((int64_t)0 * nsp + r) * nn + jp] += -S[0];
      T[((int64_t)3 * nsp + r) * nn + jp] += -S[1];
      T[((int64_t)5 * nsp + r) * nn + jp] += -S[2];
      err = fmax(err, fabs(S[6]));
      err = fmax(err, fabs(S[7]));
      err = fmax(err, fabs(S[8]));
    } else {
      // sdIntRowQStokes
      const double osemPi = (double)atanf(1.0f) * 4.0 * 8.0;  // single-precision pi, as the reference
      err = fmax(err, fabs(-S[3]));
      err = fmax(err, fabs(-S[4]));
      err = fmax(err, fabs(-S[5]));
      const double cx = -S[0], cy = -S[1], cz = -S[2];
      err = fmax(err, fabs(cx - 0.5 * osemPi));
      err = fmax(err, fabs(cy - 0.5 * osemPi));
      err = fmax(err, fabs(cz - 0.5 * osemPi));
      const ElemGeom& Gs = a.geom[r - a.nn];
      const double shpf = (Gs.type == AGB_TRI) ? 1.0 / 3.0 : 0.25;
      for (int k = 0; k < Gs.nno; ++k) {
        const int jp = a.posOfNode[Gs.con[k]];
        T[((int64_t)0 * nsp + r) * nn + jp] += shpf * cx;
        T[((int64_t)3 * nsp + r) * nn + jp] += shpf * cy;
        T[((int64_t)5 * nsp + r) * nn + jp] += shpf * cz;
        T[((int64_t)6 * nsp + r) * nn + jp] -= S[9] / Gs.nno;
        T[((int64_t)7 * nsp + r) * nn + jp] -= S[10] / Gs.nno;
        T[((int64_t)8 * nsp + r) * nn + jp] -= S[11] / Gs.nno;
      }
    }
    err_row[r] = err;
  } else {
    const double c = -S[0];
    double err = 0.0;
    if (r < a.nn) {
      // sdIntRowU: H_ii += -sum H; residual of u = x_j, q = n_j
      const int g = a.nodeList[r];
      const int jp = r;
      T[(int64_t)r * nn + jp] += c;
      for (int q = 0; q < 3; ++q) err = fmax(err, fabs(S[6 + q] + c * a.xyz[3 * g + q] - S[3 + q]));
    } else {
      // sdIntRowQ: c must be 1/2; distributed 1/3 (1/4) to the element's nodes
      err = fabs(0.5 - c);
      const ElemGeom& Gs = a.geom[r - a.nn];
      const double shpf = (Gs.type == AGB_TRI) ? 1.0 / 3.0 : 0.25;
      for (int k = 0; k < Gs.nno; ++k) {
        const int jp = a.posOfNode[Gs.con[k]];
        T[(int64_t)r * nn + jp] += shpf * c;
      }
    }
    err_row[r] = err;
  }
}

void GeneralDev::release() {
  cudaFree(adj_ptr); cudaFree(adj_p); cudaFree(adj_k); cudaFree(nodeList); cudaFree(posOfNode); cudaFree(row_src);
  cudaFree(row_een);
  posOfNode = nullptr;
  cudaFree(tmap_tgt); cudaFree(tmap_col); cudaFree(tmap_val); cudaFree(gmap_tgt); cudaFree(gmap_col); cudaFree(gmap_val);
  adj_ptr = adj_p = adj_k = nodeList = row_src = row_een = tmap_tgt = tmap_col = gmap_tgt = gmap_col = nullptr;
  tmap_val = gmap_val = nullptr;
}

template <typename T>
static cudaError_t up(T*& d, const std::vector<T>& h) {
  cudaError_t e = cudaMalloc((void**)&d, std::max<size_t>(h.size(), 1) * sizeof(T));
  if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

cudaError_t GeneralDev::upload(const GeneralLayout& L) {
  release();
  cudaError_t e;
  if ((e = up(adj_ptr, L.adj_ptr))) return e;
  if ((e = up(adj_p, L.adj_p))) return e;
  if ((e = up(adj_k, L.adj_k))) return e;
  if ((e = up(nodeList, L.nodeList))) return e;
  if ((e = up(posOfNode, L.posOfNode))) return e;
  if ((e = up(row_src, L.row_src))) return e;
  if ((e = up(row_een, L.row_een))) return e;
  if ((e = up(tmap_tgt, L.tmap_tgt))) return e;
  if ((e = up(tmap_col, L.tmap_col))) return e;
  if ((e = up(tmap_val, L.tmap_val))) return e;
  if ((e = up(gmap_tgt, L.gmap_tgt))) return e;
  if ((e = up(gmap_col, L.gmap_col))) return e;
  if ((e = up(gmap_val, L.gmap_val))) return e;
  return cudaSuccess;
}

cudaError_t general_integrals(const GeneralLayout& L, const GeneralDev& D, const ElemGeom* geom, const double* xyz,
                              const RuleDev& rule, int iqud, const IntegOpt& opt, double* T, double* G,
                              double* err_row, cudaStream_t s) {
  const bool stk = (L.kind == 2);
  const int NV = stk ? NV_STK : NV_LAP;
  GenArgs a;
  a.kind = L.kind; a.nn = L.nn; a.nq = L.nq; a.nsp = L.nsp; a.Q = rule.Q; a.iqud = iqud;
  a.geom = geom; a.xyz = xyz; a.rl = rule.l; a.rw = rule.w; a.nodeList = D.nodeList; a.posOfNode = D.posOfNode;
  a.adj_ptr = D.adj_ptr; a.adj_p = D.adj_p; a.adj_k = D.adj_k;
  a.opt = opt;
  const int64_t per_row = (int64_t)L.nq * NV * (int64_t)sizeof(double);
  int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(L.nsp, (int64_t)(1u << 30) / std::max<int64_t>(per_row, 1)));
  chunk = std::min(chunk, 65535);
  double* E = nullptr;
  cudaError_t e = cudaMalloc(&E, (size_t)chunk * per_row);
  if (e != cudaSuccess) return e;
  for (int r0 = 0; r0 < L.nsp; r0 += chunk) {
    const int nr = std::min(chunk, L.nsp - r0);
    dim3 g1(cdiv(L.nq, 128), nr);
    if (stk) {
      k_gen_elem<1><<<g1, 128, 0, s>>>(a, r0, nr, E);
      k_gen_row<1><<<nr, ROW_THREADS, 0, s>>>(a, r0, E, T, G, err_row);
    } else {
      k_gen_elem<0><<<g1, 128, 0, s>>>(a, r0, nr, E);
      k_gen_row<0><<<nr, ROW_THREADS, 0, s>>>(a, r0, E, T, G, err_row);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
  }
  cudaError_t e2 = cudaStreamSynchronize(s);
  cudaFree(E);
  return e != cudaSuccess ? e : e2;
}

__device__ __forceinline__ int sym3(int a, int b) {
  const int lo = min(a, b), hi = max(a, b);
  return (lo == 0) ? hi : (lo == 1 ? 2 + hi : 5);  // (0,0)0 (0,1)1 (0,2)2 (1,1)3 (1,2)4 (2,2)5
}

__global__ void k_gen_form(int kind, int neq, int nn, int nq, int nsp, const int* __restrict__ row_src,
                           const int* __restrict__ row_een, const int* __restrict__ tt, const int* __restrict__ tc,
                           const double* __restrict__ tv, const int* __restrict__ gt, const int* __restrict__ gc,
                           const double* __restrict__ gv, const double* __restrict__ T, const double* __restrict__ G,
                           double* __restrict__ sys, int64_t lda, double* __restrict__ rhsM, int nb) {
  const int i = blockIdx.x;
  const int r = row_src[i], een = row_een[i];
  for (int en = 0; en < neq; ++en) {
    const int comp = (kind == 2) ? sym3(een, en) : 0;
    const double* Tr = T + ((int64_t)comp * nsp + r) * nn;
    const double* Gr = G + ((int64_t)comp * nsp + r) * nq;
    for (int j = threadIdx.x; j < nn; j += blockDim.x) {
      const int t = tt[en * nn + j];
      if (t == 1) sys[(int64_t)i * lda + tc[en * nn + j]] = tv[en * nn + j] * Tr[j];
      else if (t == 2) rhsM[(int64_t)i * nb + tc[en * nn + j]] = tv[en * nn + j] * Tr[j];
    }
    for (int p = threadIdx.x; p < nq; p += blockDim.x) {
      const int t = gt[en * nq + p];
      if (t == 1) sys[(int64_t)i * lda + gc[en * nq + p]] = gv[en * nq + p] * Gr[p];
      else if (t == 2) rhsM[(int64_t)i * nb + gc[en * nq + p]] = gv[en * nq + p] * Gr[p];
    }
  }
}

cudaError_t general_form(const GeneralLayout& L, const GeneralDev& D, const double* T, const double* G, double* sys,
                         int64_t lda, double* rhsM, cudaStream_t s) {
  if (L.nrow == 0) return cudaSuccess;
  k_gen_form<<<L.nrow, 256, 0, s>>>(L.kind, L.neq, L.nn, L.nq, L.nsp, D.row_src, D.row_een, D.tmap_tgt, D.tmap_col,
                                    D.tmap_val, D.gmap_tgt, D.gmap_col, D.gmap_val, T, G, sys, lda, rhsM,
                                    std::max(L.nb, 1));
  return cudaGetLastError();
}

__global__ void k_dense_rhs(int nrow, int nb, const double* __restrict__ M, int k, const double* __restrict__ b,
                            double sign, double* __restrict__ y) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= nrow) return;
  for (int c = 0; c < k; ++c) {
    double s = 0.0;
    for (int j = lane; j < nb; j += 32) s += M[(int64_t)i * nb + j] * b[(int64_t)c * nb + j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[(int64_t)c * nrow + i] = sign * s;
  }
}

cudaError_t dense_rhs(int nrow, int nb, const double* rhsM, int k, const double* b, double sign, double* y,
                      cudaStream_t s) {
  if (nrow == 0) return cudaSuccess;
  k_dense_rhs<<<cdiv((int64_t)nrow * 32, 256), 256, 0, s>>>(nrow, nb, rhsM, k, b, sign, y);
  return cudaGetLastError();
}

__global__ void k_to_fp32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}
cudaError_t to_fp32(const double* a, float* b, int64_t count, cudaStream_t s) {
  k_to_fp32<<<std::min<int64_t>(cdiv(count, 256), 152 * 32), 256, 0, s>>>(a, b, count);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Post-processing of a solved field (not on the solve path): one CTA per
// evaluation point, its threads striding over the subdomain's elements with
// the element integrals of the assembly (no singular element), the sums
// reduced in a fixed order (warp shuffles, then warps in order).
// ---------------------------------------------------------------------------
constexpr int POST_THREADS = 256;

template <int NV>
__device__ __forceinline__ void post_reduce(double (&v)[NV], double (*sred)[POST_THREADS / 32]) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sred[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = 0.0;
      for (int w = 0; w < POST_THREADS / 32; ++w) t += sred[k][w];
      v[k] = t;
    }
}

// pressureStokes (lib_Stokes.f90:4-94) at the centroid of element r: the
// pressure rows of sdIntRowQStokes (self element left out, as its analytic
// branch leaves prG/prT zero) contracted with u - (the element's centre
// velocity) and q, times -2 / (8 pi).  With the pressure correction of the
// q-rows (lib_Stokes.f90:1851-1863) the reference's sum over nodes equals this
// differenced sum over elements.
__global__ void __launch_bounds__(POST_THREADS) k_surface_pressure(int ne, const ElemGeom* __restrict__ geom,
                                                                  const double* __restrict__ rl,
                                                                  const double* __restrict__ rw, int Q, int iqud,
                                                                  IntegOpt opt, const double* __restrict__ u,
                                                                  int nnodes, const double* __restrict__ q,
                                                                  double diff, double osemPi, double* __restrict__ p) {
  __shared__ double sred[2][POST_THREADS / 32];
  const int r = blockIdx.x;
  const ElemGeom& Er = geom[r];
  const double f = (Er.type == AGB_TRI) ? 1.0 / 3.0 : 0.25;
  double ubar[3];
  for (int c = 0; c < 3; ++c) {
    double a = 0.0;
    for (int k = 0; k < Er.nno; ++k) a += f * u[(int64_t)c * nnodes + Er.con[k]];
    ubar[c] = a;
  }
  const double s[3] = {Er.c[0], Er.c[1], Er.c[2]};
  double acc[2] = {0.0, 0.0};
  for (int e = threadIdx.x; e < ne; e += POST_THREADS) {
    if (e == r) continue;
    const ElemGeom& E = geom[e];
    StkElem o;
    stk_element(E, s, 0, rl, rw, Q, iqud, opt, o);
    for (int k = 0; k < E.nno; ++k)
      for (int c = 0; c < 3; ++c) acc[0] += o.prT[c][k] * (u[(int64_t)c * nnodes + E.con[k]] - ubar[c]);
    for (int c = 0; c < 3; ++c) acc[1] += o.prG[c] * q[(int64_t)c * ne + e];
  }
  post_reduce<2>(acc, sred);
  if (threadIdx.x == 0) p[r] = -(diff * acc[0] - acc[1]) / osemPi * 2.0;
}

// GetStokesDomainValue (lib_Stokes.f90:3043-3373) at point k: velocity, pressure
// and the reference's check of the point (stresslet diagonal sums 8 pi, sum G.n 0).
__global__ void __launch_bounds__(POST_THREADS) k_domain_stokes(int ne, const ElemGeom* __restrict__ geom,
                                                               const double* __restrict__ rl,
                                                               const double* __restrict__ rw, int Q, int iqud,
                                                               IntegOpt opt, const double* __restrict__ pts,
                                                               const double* __restrict__ u, int nnodes,
                                                               const double* __restrict__ q, double diff,
                                                               double osemPi, double* __restrict__ out,
                                                               double* __restrict__ err) {
  __shared__ double sred[10][POST_THREADS / 32];
  const int pk = blockIdx.x;
  const double s[3] = {pts[3 * (int64_t)pk], pts[3 * (int64_t)pk + 1], pts[3 * (int64_t)pk + 2]};
  // rx, ry, rz, p, sum Txx, sum Tyy, sum Tzz, sum G.n (x, y, z)
  double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int e = threadIdx.x; e < ne; e += POST_THREADS) {
    const ElemGeom& E = geom[e];
    StkElem o;
    stk_element(E, s, 0, rl, rw, Q, iqud, opt, o, 1);
    for (int k = 0; k < E.nno; ++k) {
      const int nd = E.con[k];
      const double ux = u[nd], uy = u[(int64_t)nnodes + nd], uz = u[2 * (int64_t)nnodes + nd];
      acc[0] += o.T[0][k] * ux + o.T[1][k] * uy + o.T[2][k] * uz;
      acc[1] += o.T[1][k] * ux + o.T[3][k] * uy + o.T[4][k] * uz;
      acc[2] += o.T[2][k] * ux + o.T[4][k] * uy + o.T[5][k] * uz;
      acc[3] += diff * (o.prT[0][k] * ux + o.prT[1][k] * uy + o.prT[2][k] * uz);
      acc[4] += o.T[0][k];
      acc[5] += o.T[3][k];
      acc[6] += o.T[5][k];
    }
    const double qx = q[e], qy = q[(int64_t)ne + e], qz = q[2 * (int64_t)ne + e];
    acc[0] += (o.G[0] * qx + o.G[1] * qy + o.G[2] * qz) / diff;
    acc[1] += (o.G[1] * qx + o.G[3] * qy + o.G[4] * qz) / diff;
    acc[2] += (o.G[2] * qx + o.G[4] * qy + o.G[5] * qz) / diff;
    acc[3] -= o.prG[0] * qx + o.prG[1] * qy + o.prG[2] * qz;
    const double n0 = E.n[0] * E.multi, n1 = E.n[1] * E.multi, n2 = E.n[2] * E.multi;
    acc[7] -= o.G[0] * n0 + o.G[1] * n1 + o.G[2] * n2;
    acc[8] -= o.G[1] * n0 + o.G[3] * n1 + o.G[4] * n2;
    acc[9] -= o.G[2] * n0 + o.G[4] * n1 + o.G[5] * n2;
  }
  post_reduce<10>(acc, sred);
  if (threadIdx.x == 0) {
    for (int c = 0; c < 4; ++c) out[4 * (int64_t)pk + c] = -acc[c] / osemPi;
    double e = -9.99;
    for (int c = 0; c < 3; ++c) e = fmax(e, fabs(-acc[4 + c] / osemPi - 1.0));
    for (int c = 0; c < 3; ++c) e = fmax(e, fabs(acc[7 + c]));
    err[pk] = e;
  }
}

// GetSubDomainValue (lib_domain.f90:210-344) with VerifyIntegrals (:354-391) at point k.
__global__ void __launch_bounds__(POST_THREADS) k_domain_laplace(int ne, const ElemGeom* __restrict__ geom,
                                                                const double* __restrict__ rl,
                                                                const double* __restrict__ rw, int Q, int iqud,
                                                                IntegOpt opt, const double* __restrict__ pts,
                                                                const double* __restrict__ xyz,
                                                                const double* __restrict__ u,
                                                                const double* __restrict__ q, double diff,
                                                                double* __restrict__ out, double* __restrict__ err) {
  __shared__ double sred[9][POST_THREADS / 32];
  const int pk = blockIdx.x;
  const double s[3] = {pts[3 * (int64_t)pk], pts[3 * (int64_t)pk + 1], pts[3 * (int64_t)pk + 2]};
  // sum H u, sum G q multi / diff, c = -sum H, sum H x_j (3), sum G n_j multi (3)
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int e = threadIdx.x; e < ne; e += POST_THREADS) {
    const ElemGeom& E = geom[e];
    const LapElem o = lap_element(E, s, 0, rl, rw, Q, iqud, opt, 1);
    for (int k = 0; k < E.nno; ++k) {
      const int nd = E.con[k];
      acc[0] += o.h[k] * u[nd];
      acc[2] -= o.h[k];
      for (int j = 0; j < 3; ++j) acc[3 + j] += o.h[k] * xyz[3 * (int64_t)nd + j];
    }
    acc[1] += o.g * q[e] * E.multi / diff;
    for (int j = 0; j < 3; ++j) acc[6 + j] += o.g * E.n[j] * E.multi;
  }
  post_reduce<9>(acc, sred);
  if (threadIdx.x == 0) {
    double e = 0.0;
    for (int j = 0; j < 3; ++j) e = fmax(e, fabs(acc[3 + j] + s[j] * acc[2] - acc[6 + j]));
    err[pk] = e;
    out[pk] = (-acc[0] - acc[1]) / acc[2];
  }
}

cudaError_t surface_pressure(int ne, const ElemGeom* geom, const RuleDev& rule, int iqud, const IntegOpt& opt,
                             const double* u, int nnodes, const double* q, double diff, double osemPi, double* p,
                             cudaStream_t s) {
  cudaError_t e = upload_general_tables();
  if (e != cudaSuccess || ne == 0) return e;
  k_surface_pressure<<<ne, POST_THREADS, 0, s>>>(ne, geom, rule.l, rule.w, rule.Q, iqud, opt, u, nnodes, q, diff,
                                                 osemPi, p);
  return cudaGetLastError();
}

cudaError_t domain_values(bool stokes, int ne, const ElemGeom* geom, const RuleDev& rule, int iqud, const IntegOpt& opt,
                          int npts, const double* pts, const double* xyz, const double* u, int nnodes,
                          const double* q, double diff, double osemPi, double* out, double* err, cudaStream_t s) {
  cudaError_t e = upload_general_tables();
  if (e != cudaSuccess || npts == 0) return e;
  if (stokes)
    k_domain_stokes<<<npts, POST_THREADS, 0, s>>>(ne, geom, rule.l, rule.w, rule.Q, iqud, opt, pts, u, nnodes, q,
                                                  diff, osemPi, out, err);
  else
    k_domain_laplace<<<npts, POST_THREADS, 0, s>>>(ne, geom, rule.l, rule.w, rule.Q, iqud, opt, pts, xyz, u, q, diff,
                                                   out, err);
  return cudaGetLastError();
}

}  // namespace agb
