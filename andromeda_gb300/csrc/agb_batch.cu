// Batched block LSQR over many Stokes single-layer systems of uneven size (the
// many-body resistance workflow: one particle-in-container system per body, 6
// rigid-body right-hand sides each), every matrix in the packed symmetric-block
// FP32 layout (pk_idx).
//
// The recurrence per system and right-hand side is the reference's LSQR
// (lsqr_solve / lsqr_LSQR, src/lib_lsqr.f:33-127,470-1231) exactly as the
// single-system solver runs it; what changes is the schedule:
//   * one launch per sweep covers the tiles of ALL systems: a CTA finds its
//     system by a binary search over a prefix table of tile counts, so a wave
//     of hundreds of small bodies fills the GPU as one large body does;
//   * systems whose right-hand sides have all stopped drop out (their tiles
//     exit at once), so the wave's cost follows the systems still iterating;
//   * the 7 launches of an iteration are captured once in a CUDA graph of
//     `check_every` iterations and replayed until no system is active;
//   * the row groups of the A^T*U tiles are picked by batch_autotune from
//     timed candidates (the A*V tile shape is fixed).
// The sweep tiles are the TMA-fed bodies avp_tile / atup_tile of
// agb_sweeps.cuh (tensor maps of every system kept in a device table, 64-byte
// aligned); the lsqr_precon column scaling q is applied on the fly: W = q.V is
// written by g_update into Vp, the A^T U partials are scaled by q in g_reduce.
#include "agb_batch.cuh"
#include "agb_sweeps.cuh"

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <cstdio>

namespace agb {

#define BCK(x)                                                                   \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      return false;                                                              \
    }                                                                            \
  } while (0)

static inline unsigned cdivu(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }
constexpr int BT = 256;  // threads of the element-wise kernels

// Device descriptor of one system.
struct GDesc {  // CUtensorMap members keep the 64-byte alignment TMA needs
  CUtensorMap tm_av;   // packed matrix, box {64, 6 x AVP_NB, AVP_R}
  CUtensorMap tm_atu;  // packed matrix, box {64, 24, ATUP_RS}
  CUtensorMap tm_vp;   // W = q.V as [3 x 8 rows][pk_ldp], box {64, 24}
  const double* b;
  const double* q;
  double* x;
  double *Y, *V, *W, *X, *Zp, *part;
  float *Ys, *Vp;
  int pk_ne, pk_ldp;  // block rows/columns, columns per plane of the packed store
  LsqrScalars* sc;
  int64_t lda, mpad;
  int m, n, k, itnlim;
  int cblocks, zgroups, rpg;
  int nb_b, nb_av, nb_red, nb_upd;
  // BiCGSTAB (batch_bicgstab_solve): vectors [mpad][8] in the row numbering 3i+a,
  // 1/diag(A), a second partial-sum array, the scalars; V is Y; sc0 zero gammas
  const float* A;
  double *Rb, *Rt, *Pb, *Sb, *Tb, *Xb, *dinv, *part2;
  double* rr;  // ||b - A x||^2 per right-hand side (the FP64 check after the solve)
  double* tolc;  // per right-hand side tolerances [K8] (BiCGSTAB restarts), or null: the launch's tol
  double* pc9; // block-Jacobi right preconditioner of the LSQR ([ne][3][3] inverse self blocks), or null
  // GMRES (batch_gmres_solve): basis [gmr][mpad][8], Hessenberg [gmr+1][gmr][8],
  // rotations cs, sn, g, y and the Gram-Schmidt coefficients hc [gmr+1][8],
  // the iterate X in the row numbering 3i+b of unknown b ne + i [mpad][8], x
  // split for the float-float residual [n][8] each, partial sums
  // [nb_b][gmr+1][8]; w = A M^-1 v is Y
  double *gV, *gH, *gcs, *gsn, *gg, *gy, *ghc, *gX, *gpart;
  float *gXh, *gXl;
  GmresScalars* gs;
  int gmr;
  BicgScalars* bs;
  const LsqrScalars* sc0;
};

struct GOffsets {
  const int* b;    // init tiles (mpad * 8 / 256 per system)
  const int* av;   // A*V tiles (pk_ne / AVP_R)
  const int* atu;  // A^T*U tiles (cblocks * zgroups)
  const int* red;  // reduce tiles (n * 8 / 256)
  const int* upd;  // update tiles (lda * 8 / 256)
};

__device__ __forceinline__ int find_body(const int* __restrict__ off, int nb, int blk) {
  int lo = 0, hi = nb;  // off[lo] <= blk < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= blk) lo = mid;
    else hi = mid;
  }
  return lo;
}

// per-CTA sums of squares of 8 interleaved columns (lanes with equal c are 8 apart)
__device__ __forceinline__ void block_sumsq8(double v, double* __restrict__ out) {
  __shared__ double sP[BT / 32][K8];
  double s = v * v;
  s += __shfl_xor_sync(0xffffffffu, s, 8);
  s += __shfl_xor_sync(0xffffffffu, s, 16);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < K8) sP[warp][lane] = s;
  __syncthreads();
  if (threadIdx.x < K8) {
    double a = 0.0;
    for (int w = 0; w < BT / 32; ++w) a += sP[w][threadIdx.x];
    out[threadIdx.x] = a;
  }
}

// Y = Ys = b (r0 = b for the zero warm start), partial ||b||^2.
__global__ void __launch_bounds__(BT) g_init_b(const GDesc* __restrict__ D, const int* __restrict__ off, int nb) {
  const int bi = find_body(off, nb, blockIdx.x);
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t r = t / K8;
  const int c = (int)(t % K8);
  double v = 0.0;
  if (r < d.m && c < d.k) v = d.b[(int64_t)c * d.m + r];
  if (r < d.mpad) {
    d.Y[t] = v;
    d.Ys[t] = (float)v;
  }
  block_sumsq8(v, d.part + (int64_t)blk * K8);
}

// Scalar phases, one CTA per system (same fixed-order reduction as the
// single-system k_scalars).  Phase 0 also sets the lsqr_solve tolerances.
__global__ void __launch_bounds__(256) g_scalars(const GDesc* __restrict__ D, int phase, int* __restrict__ bact,
                                                 int* nactive, double eps) {
  const int bi = blockIdx.x;
  if (phase != 0 && !bact[bi]) return;
  const GDesc& d = D[bi];
  const int nbp = phase == 0 ? d.nb_b : phase == 2 ? d.nb_av : phase == 4 ? d.nb_upd : d.nb_red;
  __shared__ double sred[256];
  __shared__ double ssum[K8];
  {
    const int t = threadIdx.x, cc = t % K8;
    double a = 0.0;
    for (int b = t / K8; b < nbp; b += 256 / K8) a += d.part[(int64_t)b * K8 + cc];
    sred[t] = a;
    __syncthreads();
    if (t < K8) {
      double tot = 0.0;
      for (int i = t; i < 256; i += K8) tot += sred[i];
      ssum[t] = tot;
    }
    __syncthreads();
  }
  const int c = threadIdx.x;
  if (c < K8) {
    LsqrScalars& s = d.sc[c];
    lsqr_phase(s, c, d.k, phase, ssum[c], nactive);
    if (phase == 0 && c < d.k) {
      // tolerances of lsqr_solve (r0 = b: ||b|| = beta0)
      const double nrm_b = sqrt(ssum[c]);
      s.atol = eps;
      s.btol = (s.beta > 0.0) ? eps * nrm_b / s.beta : eps;
      s.ctol = 1.0 / 1.0e8;
      s.itnlim = d.itnlim;
      s.active = (s.beta > 0.0) ? 1 : 0;
      s.istop = 0;
      s.itn = 0;
      s.alpha = 0.0;
    }
  }
  if (phase == 0 || phase == 4) {
    __syncthreads();
    if (threadIdx.x == 0) {
      int any = 0;
      for (int cc = 0; cc < K8; ++cc) any |= d.sc[cc].active;
      bact[bi] = any;
    }
  }
}

__global__ void __launch_bounds__(AVP_THREADS, 1) g_avp(const GDesc* __restrict__ D, const int* __restrict__ off,
                                                       int nb, const int* __restrict__ bact, int* errflag) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  avp_tile(&d.tm_av, &d.tm_vp, d.pk_ne, d.pk_ldp, d.sc, d.Y, d.Ys, d.part, errflag, (int)(blockIdx.x - off[bi]));
}

__global__ void __launch_bounds__(ATUP_C, 2) g_atup(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                                   const int* __restrict__ bact, int* errflag) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int local = blockIdx.x - off[bi];
  atup_tile(&d.tm_atu, d.pk_ne, d.lda, d.Ys, d.rpg, d.Zp, errflag, local % d.cblocks, local / d.cblocks);
}

// V <- q.(Z/beta) - beta V over the row-group partials (in order); partial ||V||^2
__global__ void __launch_bounds__(BT) g_reduce(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                               const int* __restrict__ bact, int init) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t j = t / K8;
  const int c = (int)(t % K8);
  double vn = 0.0;
  if (j < d.n) {
    double z = 0.0;
    if (d.pc9) {  // (A M^-1)^T u = M^-T (A^T u), the element's three components
      const int b = (int)(j / d.pk_ne);
      const int64_t i = j - (int64_t)b * d.pk_ne;
      const double* mi = d.pc9 + 9 * i + 3 * b;
      for (int bb = 0; bb < 3; ++bb) {
        double zb = 0.0;
        for (int g = 0; g < d.zgroups; ++g) zb += d.Zp[((int64_t)g * d.lda + (int64_t)bb * d.pk_ne + i) * K8 + c];
        z += mi[bb] * zb;
      }
    } else {
      for (int g = 0; g < d.zgroups; ++g) z += d.Zp[((int64_t)g * d.lda + j) * K8 + c];
      z *= d.q[j];
    }
    const double beta = d.sc[c].beta;
    if (d.sc[c].active && beta > 0.0) {
      vn = z / beta - (init ? 0.0 : beta * d.V[j * K8 + c]);
      d.V[j * K8 + c] = vn;
    } else {
      vn = d.V[j * K8 + c];
      if (!d.sc[c].active) vn = 0.0;
    }
  }
  block_sumsq8(vn, d.part + (int64_t)blk * K8);
}

// V <- V/alpha; X += t1 W; W <- t2 W + V; partial (t3 W_old)^2;
// Vp[b][k][jj] = q.V of column b pk_ne + jj
__global__ void __launch_bounds__(BT) g_update(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                               const int* __restrict__ bact, int init) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t j = t / K8;
  const int c = (int)(t % K8);
  double dk = 0.0;
  if (j < d.lda) {
    const int64_t id = j * K8 + c;
    if (j >= d.n) {
      d.V[id] = 0.0; d.W[id] = 0.0; d.X[id] = 0.0;
    } else {
      const LsqrScalars& s = d.sc[c];
      if (s.active) {
        double v = d.V[id];
        if (s.alpha > 0.0) v = v / s.alpha;
        d.V[id] = v;
        if (init) {
          d.W[id] = v;
          d.X[id] = 0.0;
        } else {
          const double w = d.W[id];
          d.X[id] = s.t1 * w + d.X[id];
          d.W[id] = s.t2 * w + v;
          const double q = s.t3 * w;
          dk = q;
        }
      } else if (init) {
        d.W[id] = 0.0; d.X[id] = 0.0;
      }
      if (!d.pc9) {  // with the block preconditioner g_pc_vp writes the operand
        const int b = (int)(j / d.pk_ne);
        const int64_t jj = j - (int64_t)b * d.pk_ne;
        d.Vp[((int64_t)b * K8 + c) * d.pk_ldp + jj] = (float)(d.q[j] * d.V[id]);
      }
    }
  }
  block_sumsq8(dk, d.part + (int64_t)blk * K8);
}

// x(:,c) = q .* X(:,c)   (zero warm start)
__global__ void g_finish(const GDesc* __restrict__ D) {
  const GDesc& d = D[blockIdx.y];
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)d.n * d.k;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t / d.n);
    const int64_t j = t % d.n;
    double v;
    if (d.pc9) {
      const int b = (int)(j / d.pk_ne);
      const int64_t i = j - (int64_t)b * d.pk_ne;
      const double* mi = d.pc9 + 9 * i + 3 * b;
      v = 0.0;
      for (int bb = 0; bb < 3; ++bb) v += mi[bb] * d.X[((int64_t)bb * d.pk_ne + i) * K8 + c];
    } else {
      v = d.q[j] * d.X[j * K8 + c];
    }
    d.x[(int64_t)c * d.n + j] = v;
  }
}

// the sweep-1 operand of the block-preconditioned LSQR, W = M^-1 V as
// [b][k][ldp] FP32, over the init tiles of the systems
__global__ void __launch_bounds__(BT) g_pc_vp(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                              const int* __restrict__ bact) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  if (!d.pc9) return;
  const int64_t t = (int64_t)(blockIdx.x - off[bi]) * BT + threadIdx.x;
  const int64_t i = t / K8;
  const int c = (int)(t % K8);
  if (i >= d.pk_ne) return;
  const double v0 = d.V[i * K8 + c], v1 = d.V[((int64_t)d.pk_ne + i) * K8 + c],
               v2 = d.V[(2 * (int64_t)d.pk_ne + i) * K8 + c];
  const double* mi = d.pc9 + 9 * i;
#pragma unroll
  for (int b = 0; b < 3; ++b)
    d.Vp[((int64_t)b * K8 + c) * d.pk_ldp + i] = (float)(mi[3 * b] * v0 + mi[3 * b + 1] * v1 + mi[3 * b + 2] * v2);
}

// inverses of every system's 3x3 self blocks (FP64 from the FP32 packed
// values); blockIdx.y = system
__global__ void g_pc_blocks(const GDesc* __restrict__ D, int* __restrict__ bad) {
  const GDesc& d = D[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (!d.pc9 || i >= d.pk_ne) return;
  double B[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) B[a][b] = (double)d.A[pk_idx(i, sym6(a, b), i, d.pk_ldp)];
  if (!inv3(B, d.pc9 + 9 * (int64_t)i)) atomicExch(bad, 1);
}

__global__ void g_fill(int* p, int n, int v) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) p[t] = v;
}

// ---------------------------------------------------------------------------
// Batched BiCGSTAB with the Jacobi preconditioner (the solver of the
// reference's LIS path; the recurrence of DenseLsqr::bicgstab, agb_bicg.cu),
// every kernel one launch over the tiles of all systems.  Element-wise kernels
// use the init tiles (mpad * 8 / 256 per system): t = 8 u + c, row u = 3i+a.
// ---------------------------------------------------------------------------
// per-CTA sums of 8 interleaved columns of v (lanes with equal c are 8 apart)
__device__ __forceinline__ void block_sum8(double v, double* __restrict__ out) {
  __shared__ double sQ[BT / 32][K8];
  v += __shfl_xor_sync(0xffffffffu, v, 8);
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();  // sQ may still be read by a previous call in this kernel
  if (lane < K8) sQ[warp][lane] = v;
  __syncthreads();
  if (threadIdx.x < K8) {
    double a = 0.0;
    for (int w = 0; w < BT / 32; ++w) a += sQ[w][threadIdx.x];
    out[threadIdx.x] = a;
  }
}

__global__ void __launch_bounds__(BT) gb_diag(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                             int* __restrict__ bad) {
  const int bi = find_body(off, nb, blockIdx.x);
  const GDesc& d = D[bi];
  const int64_t u = (int64_t)(blockIdx.x - off[bi]) * BT + threadIdx.x;
  if (u >= d.m) return;
  const int i = (int)(u / 3), a = (int)(u % 3);
  const double g = (double)d.A[pk_idx(i, sym6(a, a), i, d.pk_ldp)];
  if (g == 0.0 || !isfinite(g)) {
    atomicExch(bad, 1);
    d.dinv[u] = 0.0;
  } else {
    d.dinv[u] = 1.0 / g;
  }
}

// R = Rt = b, P = V = X = 0; partial ||b||^2
__global__ void __launch_bounds__(BT) gb_init(const GDesc* __restrict__ D, const int* __restrict__ off, int nb) {
  const int bi = find_body(off, nb, blockIdx.x);
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t u = t / K8;
  const int c = (int)(t % K8);
  double v = 0.0;
  if (u < d.m && c < d.k) v = d.b[(int64_t)c * d.m + u];
  if (u < d.mpad) {
    d.Rb[t] = v; d.Rt[t] = v; d.Pb[t] = 0.0; d.Y[t] = 0.0; d.Xb[t] = 0.0; d.Tb[t] = 0.0;
  }
  block_sum8(v * v, d.part + (int64_t)blk * K8);
}

// Scalar phases, one CTA per system: 0 start, 1 alpha, 2 the test on s, 3 omega,
// 4 end of the iteration (stopping tests, rho, activity).  Partial sums over
// the system's init tiles in a fixed order.
__global__ void __launch_bounds__(256) gb_scal(const GDesc* __restrict__ D, int phase, int* __restrict__ bact,
                                              int* nactive, double tol) {
  const int bi = blockIdx.x;
  if (phase != 0 && !bact[bi]) return;
  const GDesc& d = D[bi];
  __shared__ double sred[2][256];
  __shared__ double ssum[2][K8];
  const int two = (phase == 3 || phase == 4) ? 2 : 1;
  {
    const int t = threadIdx.x, cc = t % K8;
    for (int h = 0; h < two; ++h) {
      const double* P = h == 0 ? d.part : d.part2;
      double a = 0.0;
      for (int b = t / K8; b < d.nb_b; b += 256 / K8) a += P[(int64_t)b * K8 + cc];
      sred[h][t] = a;
    }
    __syncthreads();
    if (t < K8)
      for (int h = 0; h < two; ++h) {
        double tot = 0.0;
        for (int i = t; i < 256; i += K8) tot += sred[h][i];
        ssum[h][t] = tot;
      }
    __syncthreads();
  }
  const int c = threadIdx.x;
  if (c < K8) {
    BicgScalars& q = d.bs[c];
    const double s0 = ssum[0][c], s1 = ssum[1][c];
    if (d.tolc) tol = d.tolc[c];
    if (phase == 0) {
      bicg_start(q, s0, c < d.k);
    } else if (q.active) {
      if (phase == 1) {
        if (s0 == 0.0 || !isfinite(s0)) { q.status = 2; q.active = 0; q.alpha = 0.0; }
        else q.alpha = q.rho / s0;
      } else if (phase == 2) {
        q.snorm = sqrt(s0) / q.bnorm;
        q.half = (q.snorm <= tol) ? 1 : 0;
      } else if (phase == 3) {
        if (!q.half) {
          if (s1 == 0.0 || !isfinite(s1)) { q.status = 2; q.active = 0; q.omega = 0.0; }
          else q.omega = s0 / s1;
        }
      } else {
        bicg_end(q, s0, s1, tol, d.itnlim);
      }
    }
  }
  if (phase == 0 || phase == 4) {
    __syncthreads();
    if (threadIdx.x == 0) {
      int na = 0;
      for (int cc = 0; cc < K8; ++cc) na += d.bs[cc].active;
      bact[bi] = na > 0;
      if (phase == 4 && na) atomicAdd(nactive, na);
    }
  }
}

// p = r (first iteration) or r + beta (p - omega v); Vp[a][c][i] = fp32(p / d)
__global__ void __launch_bounds__(BT) gb_p(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                          const int* __restrict__ bact) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int64_t t = (int64_t)(blockIdx.x - off[bi]) * BT + threadIdx.x;
  const int64_t u = t / K8;
  const int c = (int)(t % K8);
  if (u >= d.m) return;
  const BicgScalars& q = d.bs[c];
  float w = 0.f;
  if (q.active) {
    const double p = (q.its > 0) ? d.Rb[t] + (q.rho / q.rho_old) * (q.alpha / q.omega) * (d.Pb[t] - q.omega * d.Y[t])
                                 : d.Rb[t];
    d.Pb[t] = p;
    w = (float)(p * d.dinv[u]);
  }
  d.Vp[((int64_t)(u % 3) * K8 + c) * d.pk_ldp + u / 3] = w;
}

// Y (which 0) or T (which 1) = A D^-1 (p or s), gamma 0
__global__ void __launch_bounds__(AVP_THREADS, 1) gb_avp(const GDesc* __restrict__ D, const int* __restrict__ off,
                                                        int nb, const int* __restrict__ bact, int* errflag,
                                                        int which) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  avp_tile(&d.tm_av, &d.tm_vp, d.pk_ne, d.pk_ldp, d.sc0, which ? d.Tb : d.Y, d.Ys, d.part, errflag,
           (int)(blockIdx.x - off[bi]));
}

// mode 0: part = r~ . v; mode 1: part = t . s, part2 = t . t
__global__ void __launch_bounds__(BT) gb_dots(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                             const int* __restrict__ bact, int mode) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const bool in = t / K8 < d.m;
  if (mode == 0) {
    block_sum8(in ? d.Rt[t] * d.Y[t] : 0.0, d.part + (int64_t)blk * K8);
  } else {
    block_sum8(in ? d.Tb[t] * d.Sb[t] : 0.0, d.part + (int64_t)blk * K8);
    block_sum8(in ? d.Tb[t] * d.Tb[t] : 0.0, d.part2 + (int64_t)blk * K8);
  }
}

// s = r - alpha v; Vp = fp32(s / d); partial ||s||^2
__global__ void __launch_bounds__(BT) gb_s(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                          const int* __restrict__ bact) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t u = t / K8;
  const int c = (int)(t % K8);
  double ss = 0.0;
  if (u < d.m) {
    const BicgScalars& q = d.bs[c];
    float w = 0.f;
    if (q.active) {
      const double sv = d.Rb[t] - q.alpha * d.Y[t];
      d.Sb[t] = sv;
      ss = sv * sv;
      w = (float)(sv * d.dinv[u]);
    }
    d.Vp[((int64_t)(u % 3) * K8 + c) * d.pk_ldp + u / 3] = w;
  }
  block_sum8(ss, d.part + (int64_t)blk * K8);
}

// x += alpha p/d + omega s/d; r = s - omega t; partials ||r||^2, r~ . r
__global__ void __launch_bounds__(BT) gb_xr(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                           const int* __restrict__ bact) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t u = t / K8;
  const int c = (int)(t % K8);
  double rr = 0.0, rtr = 0.0;
  if (u < d.m) {
    const BicgScalars& q = d.bs[c];
    if (q.active) {
      const double di = d.dinv[u];
      if (q.half) {
        d.Xb[t] += q.alpha * (d.Pb[t] * di);
      } else {
        d.Xb[t] += q.alpha * (d.Pb[t] * di) + q.omega * (d.Sb[t] * di);
        const double r = d.Sb[t] - q.omega * d.Tb[t];
        d.Rb[t] = r;
        rr = r * r;
        rtr = d.Rt[t] * r;
      }
    }
  }
  block_sum8(rr, d.part + (int64_t)blk * K8);
  block_sum8(rtr, d.part2 + (int64_t)blk * K8);
}

// x(:,c) in the unknown numbering a ne + i
__global__ void gb_finish(const GDesc* __restrict__ D) {
  const GDesc& d = D[blockIdx.y];
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)d.m * K8;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t % K8);
    if (c >= d.k) continue;
    const int64_t u = t / K8;
    d.x[(int64_t)c * d.n + (u % 3) * d.pk_ne + u / 3] = d.Xb[t];
  }
}

// ||b - A x||^2 per right-hand side with FP64 products and sums, A the body's
// FP32 packed single layer, x from gb_finish: one warp per element row i (its
// three equations), lanes over the element columns; a CTA per 8 rows of one
// body (the A*V tiles of 16 rows, two CTAs each).  rr must start at zero.
__global__ void __launch_bounds__(256) gb_resid(const GDesc* __restrict__ D, const int* __restrict__ off, int nb) {
  const int tile = blockIdx.x >> 1;
  const int bi = find_body(off, nb, tile);
  const GDesc& d = D[bi];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = (tile - off[bi]) * AVP_R + (blockIdx.x & 1) * 8 + warp;
  if (i >= d.pk_ne) return;  // a whole warp; the kernel has no block barrier
  const int ne = d.pk_ne;
  double acc[3][K8];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) acc[a][c] = 0.0;
  for (int j = lane; j < ne; j += 32) {
    double g6[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) g6[c] = (double)d.A[pk_idx(i, c, j, d.pk_ldp)];
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = 0; c < K8; ++c) {
        if (c >= d.k) break;
        const double xv = d.x[(int64_t)c * d.n + (int64_t)b * ne + j];
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[a][c] += g6[sym6(a, b)] * xv;
      }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) {
      double v = acc[a][c];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0 && c < d.k) {
        const double r = d.b[(int64_t)c * d.m + 3 * (int64_t)i + a] - v;
        atomicAdd(&d.rr[c], r * r);
      }
    }
}

// ---------------------------------------------------------------------------
// Batched restarted GMRES with the 3x3 self-block right preconditioner (the
// recurrence of DenseLsqr::gmres, agb_gmres.cu), every kernel one launch over
// the tiles of all systems.  Element-wise kernels use the init tiles
// (mpad * 8 / 256 per system, t = 8 u + c); per-system reductions are one CTA
// per system over its tiles' partial sums in a fixed order.  bact: systems
// with a column still in the current cycle; bran: systems that ran the cycle
// (their iterate is updated and their true residual formed after it).
// ---------------------------------------------------------------------------
// w = b (from_b) or the residual already in Y; partial 0: ||w||^2
__global__ void __launch_bounds__(BT) gg_load(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                             const int* __restrict__ bran, int from_b) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bran[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t u = t / K8;
  const int c = (int)(t % K8);
  double v = 0.0;
  if (from_b) {
    if (u < d.m && c < d.k) v = d.b[(int64_t)c * d.m + u];
    d.Y[t] = v;
  } else {
    v = d.Y[t];
  }
  block_sum8(v * v, d.gpart + (int64_t)blk * (d.gmr + 1) * K8);
}

// start of a cycle (DenseLsqr::gmres's k_gm_begin per system)
__global__ void __launch_bounds__(256) gg_begin(const GDesc* __restrict__ D, int* __restrict__ bact,
                                               int* __restrict__ bran, int* nactive, double tol, int first) {
  const int bi = blockIdx.x;
  if (!bran[bi]) return;
  const GDesc& d = D[bi];
  const int np = d.gmr + 1;
  __shared__ double sred[256];
  __shared__ double ssum[K8];
  const int t = threadIdx.x, cc = t % K8;
  double a = 0.0;
  for (int b = t / K8; b < d.nb_b; b += 256 / K8) a += d.gpart[((int64_t)b * np) * K8 + cc];
  sred[t] = a;
  __syncthreads();
  if (t < K8) {
    double tot = 0.0;
    for (int i = t; i < 256; i += K8) tot += sred[i];
    ssum[t] = tot;
  }
  __syncthreads();
  if (t < K8) {
    GmresScalars& q = d.gs[t];
    const double beta = sqrt(ssum[t]);
    if (first) {
      q.bnorm = beta;
      q.its = 0;
      q.cycles = 0;
      q.status = (t < d.k && beta > 0.0) ? -1 : 0;
      q.prev = 1.0;
      q.relres = (beta > 0.0) ? 1.0 : 0.0;
    }
    q.jc = 0;
    if (q.status == -1) {
      const double rel = beta / q.bnorm;
      q.relres = rel;
      if (rel <= tol) q.status = 0;
      else if (q.its >= d.itnlim) q.status = 1;
      else if (!first && rel > 0.9 * q.prev) q.status = 3;
      q.prev = rel;
    }
    q.active = (q.status == -1) ? 1 : 0;
    if (q.active) q.cycles += 1;
    q.beta = beta;
    q.hnext = beta;
    d.gg[t] = beta;
  }
  __syncthreads();
  if (t == 0) {
    int na = 0;
    for (int c = 0; c < K8; ++c) na += d.gs[c].active;
    bact[bi] = na > 0;
    bran[bi] = na > 0;
    if (na) atomicAdd(nactive, na);
  }
}

// v_j = w / h; W = fp32(M^-1 v_j) as [b][8][ldp] (zero for an inactive column)
__global__ void __launch_bounds__(BT) gg_pc(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                           const int* __restrict__ bact, int j) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int64_t t = (int64_t)(blockIdx.x - off[bi]) * BT + threadIdx.x;
  const int i = (int)(t / K8), c = (int)(t % K8);
  if (i >= d.pk_ne) return;
  const GmresScalars& q = d.gs[c];
  double* Vj = d.gV + (int64_t)j * d.mpad * K8;
  float o[3] = {0.f, 0.f, 0.f};
  if (q.active) {
    const double inv = 1.0 / q.hnext;
    double v[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int64_t id = (int64_t)(3 * i + a) * K8 + c;
      v[a] = d.Y[id] * inv;
      Vj[id] = v[a];
    }
    const double* mi = d.pc9 + 9 * (int64_t)i;
#pragma unroll
    for (int b = 0; b < 3; ++b) o[b] = (float)(mi[3 * b] * v[0] + mi[3 * b + 1] * v[1] + mi[3 * b + 2] * v[2]);
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a) Vj[(int64_t)(3 * i + a) * K8 + c] = 0.0;
  }
#pragma unroll
  for (int b = 0; b < 3; ++b) d.Vp[((int64_t)b * K8 + c) * d.pk_ldp + i] = o[b];
}

// partial l (l = 0..j): v_l . w
__global__ void __launch_bounds__(BT) gg_dots(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                             const int* __restrict__ bact, int j) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int64_t mv = d.mpad * K8;
  const double w = d.Y[t];
  for (int l = 0; l <= j; ++l)
    block_sum8(d.gV[(int64_t)l * mv + t] * w, d.gpart + ((int64_t)blk * (d.gmr + 1) + l) * K8);
}

// hc[l] = v_l . w from the tile partials (in order); H[l][j] = hc (pass 0) or += hc
__global__ void __launch_bounds__(256) gg_hred(const GDesc* __restrict__ D, const int* __restrict__ bact, int j,
                                              int pass) {
  const int bi = blockIdx.x;
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int np = d.gmr + 1;
  for (int p = threadIdx.x; p < (j + 1) * K8; p += blockDim.x) {
    const int l = p / K8, c = p % K8;
    double v = 0.0;
    for (int b = 0; b < d.nb_b; ++b) v += d.gpart[((int64_t)b * np + l) * K8 + c];
    d.ghc[p] = v;
    double* h = d.gH + ((int64_t)l * d.gmr + j) * K8 + c;
    *h = pass ? *h + v : v;
  }
}

// w -= sum_l hc[l] v_l over the active columns; partial 0: ||w||^2
__global__ void __launch_bounds__(BT) gg_orth(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                             const int* __restrict__ bact, int j) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int blk = blockIdx.x - off[bi];
  const int64_t t = (int64_t)blk * BT + threadIdx.x;
  const int c = (int)(t % K8);
  const int64_t mv = d.mpad * K8;
  double w = d.Y[t];
  if (d.gs[c].active) {
    for (int l = 0; l <= j; ++l) w -= d.ghc[l * K8 + c] * d.gV[(int64_t)l * mv + t];
    d.Y[t] = w;
  } else {
    w = 0.0;
  }
  block_sum8(w * w, d.gpart + (int64_t)blk * (d.gmr + 1) * K8);
}

// end of step j (k_gm_givens per system)
__global__ void __launch_bounds__(256) gg_givens(const GDesc* __restrict__ D, int* __restrict__ bact,
                                                int* nactive, double tol, int j) {
  const int bi = blockIdx.x;
  if (!bact[bi]) return;
  const GDesc& d = D[bi];
  const int mr = d.gmr, np = mr + 1;
  const int c = threadIdx.x;
  if (c < K8) {
    GmresScalars& q = d.gs[c];
    if (q.active) {
      double ss = 0.0;
      for (int b = 0; b < d.nb_b; ++b) ss += d.gpart[((int64_t)b * np) * K8 + c];
      const double hn = sqrt(ss);
      double* H = d.gH;
      for (int l = 0; l < j; ++l) {
        double* a0 = H + ((int64_t)l * mr + j) * K8 + c;
        double* a1 = H + ((int64_t)(l + 1) * mr + j) * K8 + c;
        const double x0 = *a0, x1 = *a1, cs = d.gcs[l * K8 + c], sn = d.gsn[l * K8 + c];
        *a0 = cs * x0 + sn * x1;
        *a1 = -sn * x0 + cs * x1;
      }
      double* hjj = H + ((int64_t)j * mr + j) * K8 + c;
      const double hd = *hjj;
      const double r = hypot(hd, hn);
      double cs = 1.0, sn = 0.0;
      if (r > 0.0) {
        cs = hd / r;
        sn = hn / r;
      }
      *hjj = r;
      d.gcs[j * K8 + c] = cs;
      d.gsn[j * K8 + c] = sn;
      const double gj = d.gg[j * K8 + c];
      d.gg[(j + 1) * K8 + c] = -sn * gj;
      d.gg[j * K8 + c] = cs * gj;
      q.its += 1;
      q.jc = j + 1;
      q.hnext = hn;
      q.relres = fabs(d.gg[(j + 1) * K8 + c]) / q.bnorm;
      if (q.relres <= tol || !(hn > 0.0) || j + 1 == mr || q.its >= d.itnlim) q.active = 0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int na = 0;
    for (int cc = 0; cc < K8; ++cc) na += d.gs[cc].active;
    bact[bi] = na > 0;
    if (na) atomicAdd(nactive, na);
  }
}

// y = R^-1 g per column over the jc steps of the cycle
__global__ void gg_solve(const GDesc* __restrict__ D, const int* __restrict__ bran) {
  const int bi = blockIdx.x;
  if (!bran[bi]) return;
  const GDesc& d = D[bi];
  const int c = threadIdx.x;
  if (c >= K8) return;
  const int jc = d.gs[c].jc, mr = d.gmr;
  for (int l = jc - 1; l >= 0; --l) {
    double v = d.gg[l * K8 + c];
    for (int p = l + 1; p < jc; ++p) v -= d.gH[((int64_t)l * mr + p) * K8 + c] * d.gy[p * K8 + c];
    const double dd = d.gH[((int64_t)l * mr + l) * K8 + c];
    d.gy[l * K8 + c] = (dd != 0.0) ? v / dd : 0.0;
  }
}

// X += M^-1 (sum_l y_l v_l), a thread per (element, column)
__global__ void __launch_bounds__(BT) gg_xupd(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                             const int* __restrict__ bran) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bran[bi]) return;
  const GDesc& d = D[bi];
  const int64_t t = (int64_t)(blockIdx.x - off[bi]) * BT + threadIdx.x;
  const int i = (int)(t / K8), c = (int)(t % K8);
  if (i >= d.pk_ne) return;
  const int jc = d.gs[c].jc;
  if (jc == 0) return;
  const int64_t mv = d.mpad * K8;
  double z[3] = {0.0, 0.0, 0.0};
  for (int l = 0; l < jc; ++l) {
    const double yl = d.gy[l * K8 + c];
#pragma unroll
    for (int a = 0; a < 3; ++a) z[a] += yl * d.gV[(int64_t)l * mv + (int64_t)(3 * i + a) * K8 + c];
  }
  const double* mi = d.pc9 + 9 * (int64_t)i;
#pragma unroll
  for (int b = 0; b < 3; ++b)
    d.gX[(int64_t)(3 * i + b) * K8 + c] += mi[3 * b] * z[0] + mi[3 * b + 1] * z[1] + mi[3 * b + 2] * z[2];
}

// X (row numbering) -> FP32 high/low parts in the unknown numbering [b ne + i][8]
__global__ void __launch_bounds__(BT) gg_split(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                              const int* __restrict__ bran) {
  const int bi = find_body(off, nb, blockIdx.x);
  if (!bran[bi]) return;
  const GDesc& d = D[bi];
  const int64_t t = (int64_t)(blockIdx.x - off[bi]) * BT + threadIdx.x;
  const int64_t u = t / K8;
  const int c = (int)(t % K8);
  if (u >= d.m) return;
  const int64_t i = u / 3, b = u % 3;
  const double x = d.gX[t];
  const float h = (float)x;
  const int64_t id = (b * d.pk_ne + i) * K8 + c;
  d.gXh[id] = h;
  d.gXl[id] = (float)(x - (double)h);
}

// Y = b - A x per system in the float-float form of k_residp_ff (one warp per
// element row; two CTAs of 8 rows per A*V tile of 16)
template <int KC>
__global__ void __launch_bounds__(256) gg_resid(const GDesc* __restrict__ D, const int* __restrict__ off, int nb,
                                               const int* __restrict__ bran) {
  const int tile = blockIdx.x >> 1;
  const int bi = find_body(off, nb, tile);
  if (!bran[bi]) return;
  const GDesc& d = D[bi];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = (tile - off[bi]) * AVP_R + (blockIdx.x & 1) * 8 + warp;
  if (i >= d.pk_ne) return;  // a whole warp; the kernel has no block barrier
  const int ne = d.pk_ne;
  float sm[3][KC], er[3][KC], lo[3][KC];
  double acc[3][KC];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < KC; ++c) {
      sm[a][c] = er[a][c] = lo[a][c] = 0.f;
      acc[a][c] = 0.0;
    }
  for (int j0 = lane; j0 < ne; j0 += 32 * kFFTerms) {
    const int j1 = min(ne, j0 + 32 * kFFTerms);
    for (int j = j0; j < j1; j += 32) {
      float g6[6];
#pragma unroll
      for (int cc = 0; cc < 6; ++cc) g6[cc] = d.A[pk_idx(i, cc, j, d.pk_ldp)];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float* xh = d.gXh + ((int64_t)b * ne + j) * K8;
        const float* xl = d.gXl + ((int64_t)b * ne + j) * K8;
#pragma unroll
        for (int c = 0; c < KC; ++c) {
          const float hv = xh[c], lv = xl[c];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float g = g6[sym6(a, b)];
            const float p = __fmul_rn(g, hv);
            const float pe = fmaf(g, hv, -p);
            const float s0 = sm[a][c];
            const float tt = __fadd_rn(s0, p);
            const float bp = __fsub_rn(tt, s0);
            const float e = __fadd_rn(__fsub_rn(s0, __fsub_rn(tt, bp)), __fsub_rn(p, bp));
            sm[a][c] = tt;
            er[a][c] = __fadd_rn(er[a][c], e);
            lo[a][c] = fmaf(g, lv, __fadd_rn(lo[a][c], pe));
          }
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < KC; ++c) {
        acc[a][c] += (double)sm[a][c] + ((double)er[a][c] + (double)lo[a][c]);
        sm[a][c] = er[a][c] = lo[a][c] = 0.f;
      }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) {
      double v = 0.0;
      if (c < KC) v = acc[a][c];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) {
        const int64_t row = 3 * (int64_t)i + a;
        d.Y[row * K8 + c] = (c < d.k) ? d.b[(int64_t)c * d.m + row] - v : 0.0;
      }
    }
}

// x (column-major [k][n], unknown b ne + i) from X
__global__ void __launch_bounds__(BT) gg_out(const GDesc* __restrict__ D, const int* __restrict__ off, int nb) {
  const int bi = find_body(off, nb, blockIdx.x);
  const GDesc& d = D[bi];
  const int64_t t = (int64_t)(blockIdx.x - off[bi]) * BT + threadIdx.x;
  const int64_t u = t / K8;
  const int c = (int)(t % K8);
  if (u >= d.m || c >= d.k) return;
  d.x[(int64_t)c * d.n + (u % 3) * d.pk_ne + u / 3] = d.gX[t];
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
template <typename K>
static cudaError_t set_smem(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

struct BatchSolver {
  int nb = 0, k = 0;
  BatchTune tune;
  cudaStream_t s = 0;
  std::vector<GDesc> hd;
  std::vector<double*> tolc_dev;  // per-column tolerance pieces of the pool (BiCGSTAB)
  std::vector<int> hoff_b, hoff_av, hoff_atu, hoff_red, hoff_upd;
  GDesc* d_desc = nullptr;
  int* d_off = nullptr;  // 5 tables of nb+1
  GOffsets off{};
  int* bact = nullptr;
  int* bran = nullptr;  // GMRES: systems that run the current cycle
  int* nactive = nullptr;
  int* h_nactive = nullptr;
  int* errflag = nullptr;
  void* pool = nullptr;
  double bytes_A = 0.0;
  std::string err;

  ~BatchSolver() { release(); }
  void release() {
    cudaFree(d_desc); cudaFree(d_off); cudaFree(bact); cudaFree(bran); cudaFree(nactive); cudaFree(errflag);
    cudaFree(pool);
    bran = nullptr;
    if (h_nactive) cudaFreeHost(h_nactive);
    d_desc = nullptr; d_off = nullptr; bact = nullptr; nactive = nullptr; errflag = nullptr; pool = nullptr;
    h_nactive = nullptr;
  }

  bool setup(const std::vector<BatchBody>& bodies, int k_, int maxit, const BatchTune& t, cudaStream_t st,
             bool bicg = false, bool bj = false, int gmr = 0) {
    release();
    nb = (int)bodies.size();
    k = k_;
    tune = t;
    s = st;
    if (nb == 0) { err = "empty batch"; return false; }
    if (k < 1 || k > K8) { err = "number of right-hand sides must be 1..8"; return false; }
    BCK(set_smem(g_avp, AVP_SMEM));
    BCK(set_smem(g_atup, ATUP_SMEM));
    hd.assign(nb, GDesc{});
    tolc_dev.assign(nb, nullptr);
    hoff_b.assign(nb + 1, 0); hoff_av.assign(nb + 1, 0); hoff_atu.assign(nb + 1, 0);
    hoff_red.assign(nb + 1, 0); hoff_upd.assign(nb + 1, 0);
    // pool layout (bytes), every piece 256-byte aligned
    size_t bytes = 0;
    auto take = [&](size_t n) { const size_t o = bytes; bytes += (n + 255) / 256 * 256; return o; };
    struct Offs { size_t Y, Ys, V, W, X, Vp, Zp, part, sc, bg, part2, bs, rr, tolc, pc9, gm, gmf, gs; };
    std::vector<Offs> po(nb);
    const size_t o_sc0 = take(K8 * sizeof(LsqrScalars));  // zero gammas of the BiCGSTAB sweeps
    bytes_A = 0.0;
    for (int i = 0; i < nb; ++i) {
      const BatchBody& B = bodies[i];
      if (B.lda % 32 != 0 || B.lda < B.n || B.pk_ne < 1 || B.m != 3 * B.pk_ne || B.n != B.m ||
          B.pk_ldp % 64 != 0 || B.pk_ldp < B.pk_ne || !B.A || !B.b || !B.q || !B.x) {
        err = "bad system " + std::to_string(i);
        return false;
      }
      GDesc& d = hd[i];
      d.lda = B.lda; d.m = B.m; d.n = B.n; d.k = k;
      d.pk_ne = B.pk_ne;
      d.pk_ldp = B.pk_ldp;
      d.mpad = ((int64_t)B.m + 255) / 256 * 256;
      d.itnlim = maxit > 0 ? maxit : (bicg ? 1000 : 10 * (B.m + B.n + 50));
      // A^T U tiles: 256 element columns x a group of block rows
      d.cblocks = (int)cdivu(B.pk_ldp, ATUP_C);
      d.zgroups = std::max(1, (int)cdivu(B.pk_ne, std::max(tune.atup_rows, ATUP_RS)));
      d.rpg = (int)((cdivu(B.pk_ne, d.zgroups) + ATUP_RS - 1) / ATUP_RS * ATUP_RS);
      d.zgroups = (int)cdivu(B.pk_ne, d.rpg);
      d.nb_av = (int)cdivu(B.pk_ne, AVP_R);
      d.nb_b = (int)cdivu(d.mpad * K8, BT);
      d.nb_red = (int)cdivu((int64_t)B.n * K8, BT);
      d.nb_upd = (int)cdivu(B.lda * K8, BT);
      const int nbmax = std::max(std::max(d.nb_b, d.nb_av), std::max(d.nb_red, d.nb_upd));
      po[i].Y = take(d.mpad * K8 * sizeof(double));
      po[i].Ys = take(d.mpad * K8 * sizeof(float));
      po[i].V = take(B.lda * K8 * sizeof(double));
      po[i].W = take(B.lda * K8 * sizeof(double));
      po[i].X = take(B.lda * K8 * sizeof(double));
      po[i].Vp = take((size_t)3 * K8 * B.pk_ldp * sizeof(float));
      po[i].Zp = take((size_t)d.zgroups * B.lda * K8 * sizeof(double));
      po[i].part = take((size_t)nbmax * K8 * sizeof(double));
      po[i].sc = take(K8 * sizeof(LsqrScalars));
      if (bicg) {
        po[i].bg = take((size_t)(6 * d.mpad * K8 + d.mpad) * sizeof(double));  // R, Rt, P, S, T, X; 1/diag
        po[i].part2 = take((size_t)nbmax * K8 * sizeof(double));
        po[i].bs = take(K8 * sizeof(BicgScalars));
        po[i].rr = take(K8 * sizeof(double));
        po[i].tolc = take(K8 * sizeof(double));
      }
      if (bj || gmr > 0) po[i].pc9 = take((size_t)9 * B.pk_ne * sizeof(double));
      if (gmr > 0) {
        const size_t mv = (size_t)d.mpad * K8;
        po[i].gm = take(((size_t)gmr * mv + (size_t)(gmr + 1) * gmr * K8 + 5 * (size_t)(gmr + 1) * K8 + mv +
                         (size_t)d.nb_b * (gmr + 1) * K8) * sizeof(double));
        po[i].gmf = take(2 * (size_t)3 * B.pk_ne * K8 * sizeof(float));
        po[i].gs = take(K8 * sizeof(GmresScalars));
      }
      hoff_b[i + 1] = hoff_b[i] + d.nb_b;
      hoff_av[i + 1] = hoff_av[i] + d.nb_av;
      hoff_atu[i + 1] = hoff_atu[i] + d.cblocks * d.zgroups;
      hoff_red[i + 1] = hoff_red[i] + d.nb_red;
      hoff_upd[i + 1] = hoff_upd[i] + d.nb_upd;
      bytes_A += 24.0 * (double)B.pk_ne * (double)B.pk_ne;
      if (!make_packed_map(&d.tm_av, B.A, B.pk_ldp, B.pk_ne, 6 * AVP_NB, AVP_R, err)) return false;
      if (!make_packed_map(&d.tm_atu, B.A, B.pk_ldp, B.pk_ne, 6 * (ATUP_C / 64), ATUP_RS, err)) return false;
      d.b = B.b; d.q = B.q; d.x = B.x;
      d.A = B.A;
    }
    BCK(cudaMalloc(&pool, bytes));
    BCK(cudaMemsetAsync(pool, 0, bytes, s));
    char* p = (char*)pool;
    for (int i = 0; i < nb; ++i) {
      GDesc& d = hd[i];
      d.Y = (double*)(p + po[i].Y); d.Ys = (float*)(p + po[i].Ys);
      d.V = (double*)(p + po[i].V); d.W = (double*)(p + po[i].W); d.X = (double*)(p + po[i].X);
      d.Vp = (float*)(p + po[i].Vp); d.Zp = (double*)(p + po[i].Zp); d.part = (double*)(p + po[i].part);
      d.sc = (LsqrScalars*)(p + po[i].sc);
      d.sc0 = (const LsqrScalars*)(p + o_sc0);
      if (bicg) {
        double* g = (double*)(p + po[i].bg);
        const int64_t mv = d.mpad * K8;
        d.Rb = g; d.Rt = g + mv; d.Pb = g + 2 * mv; d.Sb = g + 3 * mv; d.Tb = g + 4 * mv; d.Xb = g + 5 * mv;
        d.dinv = g + 6 * mv;
        d.part2 = (double*)(p + po[i].part2);
        d.bs = (BicgScalars*)(p + po[i].bs);
        d.rr = (double*)(p + po[i].rr);
        d.tolc = nullptr;  // set by batch_bicgstab_solve when it is given per-column tolerances
        tolc_dev[i] = (double*)(p + po[i].tolc);
      }
      d.pc9 = (bj || gmr > 0) ? (double*)(p + po[i].pc9) : nullptr;
      d.gmr = gmr;
      if (gmr > 0) {
        const size_t mv = (size_t)d.mpad * K8;
        double* g = (double*)(p + po[i].gm);
        d.gV = g; g += (size_t)gmr * mv;
        d.gH = g; g += (size_t)(gmr + 1) * gmr * K8;
        d.gcs = g; g += (size_t)(gmr + 1) * K8;
        d.gsn = g; g += (size_t)(gmr + 1) * K8;
        d.gg = g; g += (size_t)(gmr + 1) * K8;
        d.gy = g; g += (size_t)(gmr + 1) * K8;
        d.ghc = g; g += (size_t)(gmr + 1) * K8;
        d.gX = g; g += mv;
        d.gpart = g;
        d.gXh = (float*)(p + po[i].gmf);
        d.gXl = d.gXh + (size_t)3 * d.pk_ne * K8;
        d.gs = (GmresScalars*)(p + po[i].gs);
      }
      // the pool is zeroed: the pad columns pk_ne..pk_ldp-1 of Vp stay zero
      if (!make_tensor_map_2d(&d.tm_vp, d.Vp, d.pk_ldp, 3 * K8, AVP_BC, 3 * K8, err)) return false;
    }
    BCK(cudaMalloc(&d_desc, nb * sizeof(GDesc)));
    BCK(cudaMemcpyAsync(d_desc, hd.data(), nb * sizeof(GDesc), cudaMemcpyHostToDevice, s));
    BCK(cudaMalloc(&d_off, 5 * (size_t)(nb + 1) * sizeof(int)));
    const std::vector<int>* tabs[5] = {&hoff_b, &hoff_av, &hoff_atu, &hoff_red, &hoff_upd};
    for (int t = 0; t < 5; ++t)
      BCK(cudaMemcpyAsync(d_off + t * (nb + 1), tabs[t]->data(), (nb + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    off.b = d_off; off.av = d_off + (nb + 1); off.atu = d_off + 2 * (nb + 1); off.red = d_off + 3 * (nb + 1);
    off.upd = d_off + 4 * (nb + 1);
    BCK(cudaMalloc(&bact, nb * sizeof(int)));
    BCK(cudaMalloc(&bran, nb * sizeof(int)));
    g_fill<<<cdivu(nb, 256), 256, 0, s>>>(bran, nb, 1);
    BCK(cudaMalloc(&nactive, sizeof(int)));
    BCK(cudaMallocHost(&h_nactive, sizeof(int)));
    BCK(cudaMalloc(&errflag, sizeof(int)));
    BCK(cudaMemsetAsync(errflag, 0, sizeof(int), s));
    g_fill<<<cdivu(nb, 256), 256, 0, s>>>(bact, nb, 1);
    BCK(cudaStreamSynchronize(s));  // host tables above must outlive their copies
    return true;
  }

  void launch_av() {
    g_avp<<<hoff_av[nb], AVP_THREADS, AVP_SMEM, s>>>(d_desc, off.av, nb, bact, errflag);
  }
  void launch_atu() { g_atup<<<hoff_atu[nb], ATUP_C, ATUP_SMEM, s>>>(d_desc, off.atu, nb, bact, errflag); }
};

bool batch_lsqr_solve(const std::vector<BatchBody>& bodies, int k, double eps, int maxit, const BatchTune& tune,
                      cudaStream_t s, std::vector<int>& nit, std::vector<int>& istop, BatchStats* st,
                      std::string& err, bool bj) {
  BatchSolver S;
  if (!S.setup(bodies, k, maxit, tune, s, false, bj)) { err = S.err; return false; }
  const int nb = S.nb;
  int itmax = 0;
  for (const auto& d : S.hd) itmax = std::max(itmax, d.itnlim);
  long launches = 0;
  if (bj) {  // the inverse self blocks of every system
    int nemax = 1;
    for (const auto& d : S.hd) nemax = std::max(nemax, d.pk_ne);
    BCK(cudaMemsetAsync(S.nactive, 0, sizeof(int), s));
    g_pc_blocks<<<dim3(cdivu(nemax, 128), nb), 128, 0, s>>>(S.d_desc, S.nactive);
    int bad = 0;
    BCK(cudaMemcpyAsync(&bad, S.nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
    ++launches;
    if (bad) { err = "a singular 3x3 self block: the block preconditioner cannot be formed"; return false; }
  }
  // initial vectors: r0 = b, beta0, tolerances; A^T r0, alpha0, W = V
  g_init_b<<<S.hoff_b[nb], BT, 0, s>>>(S.d_desc, S.off.b, nb);
  g_scalars<<<nb, 256, 0, s>>>(S.d_desc, 0, S.bact, S.nactive, eps);
  S.launch_atu();
  g_reduce<<<S.hoff_red[nb], BT, 0, s>>>(S.d_desc, S.off.red, nb, S.bact, 1);
  g_scalars<<<nb, 256, 0, s>>>(S.d_desc, 1, S.bact, S.nactive, eps);
  g_update<<<S.hoff_upd[nb], BT, 0, s>>>(S.d_desc, S.off.upd, nb, S.bact, 1);
  if (bj) g_pc_vp<<<S.hoff_b[nb], BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact);
  launches += bj ? 7 : 6;
  BCK(cudaGetLastError());
  const int ce = std::max(1, std::min(tune.check_every, 32));
  std::vector<cudaEvent_t> ev(4 * ce, nullptr);
  for (auto& e : ev) BCK(cudaEventCreate(&e));
  auto iteration = [&](int i) {
    cudaEventRecordWithFlags(ev[4 * i], s, cudaEventRecordExternal);
    S.launch_av();
    cudaEventRecordWithFlags(ev[4 * i + 1], s, cudaEventRecordExternal);
    g_scalars<<<nb, 256, 0, s>>>(S.d_desc, 2, S.bact, S.nactive, eps);
    cudaEventRecordWithFlags(ev[4 * i + 2], s, cudaEventRecordExternal);
    S.launch_atu();
    cudaEventRecordWithFlags(ev[4 * i + 3], s, cudaEventRecordExternal);
    g_reduce<<<S.hoff_red[nb], BT, 0, s>>>(S.d_desc, S.off.red, nb, S.bact, 0);
    g_scalars<<<nb, 256, 0, s>>>(S.d_desc, 3, S.bact, S.nactive, eps);
    g_update<<<S.hoff_upd[nb], BT, 0, s>>>(S.d_desc, S.off.upd, nb, S.bact, 0);
    if (bj) g_pc_vp<<<S.hoff_b[nb], BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact);
    cudaMemsetAsync(S.nactive, 0, sizeof(int), s);
    g_scalars<<<nb, 256, 0, s>>>(S.d_desc, 4, S.bact, S.nactive, eps);
  };
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool ok = true;
  auto cleanup = [&]() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ev) if (e) cudaEventDestroy(e);
  };
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) ok = false;
  if (ok) {
    for (int i = 0; i < ce; ++i) iteration(i);
    if (cudaStreamEndCapture(s, &graph) != cudaSuccess) ok = false;
  }
  if (ok && cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) ok = false;
  if (!ok) {
    err = std::string("batch graph capture: ") + cudaGetErrorString(cudaGetLastError());
    cleanup();
    return false;
  }
  // initial activity
  cudaMemsetAsync(S.nactive, 0, sizeof(int), s);
  std::vector<int> hb(nb);
  if (cudaMemcpyAsync(hb.data(), S.bact, nb * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    err = "batch: initial state";
    cleanup();
    return false;
  }
  int act = 0;
  for (int v : hb) act += v;
  long iters = 0;
  double av_ms = 0.0, atu_ms = 0.0;
  long nav = 0, natu = 0;
  while (act > 0 && iters < (long)itmax + ce) {
    if (cudaGraphLaunch(gexec, s) != cudaSuccess) { ok = false; break; }
    launches += (bj ? 8L : 7L) * ce;
    cudaMemcpyAsync(S.h_nactive, S.nactive, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) { ok = false; break; }
    for (int i = 0; i < ce; ++i) {
      float a = 0.f, b = 0.f;
      if (cudaEventElapsedTime(&a, ev[4 * i], ev[4 * i + 1]) == cudaSuccess) { av_ms += a; ++nav; }
      if (cudaEventElapsedTime(&b, ev[4 * i + 2], ev[4 * i + 3]) == cudaSuccess) { atu_ms += b; ++natu; }
    }
    (void)cudaGetLastError();
    iters += ce;
    act = *S.h_nactive;
  }
  cleanup();
  if (!ok) {
    err = std::string("batch iterations: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  int nmax = 1;
  for (const auto& d : S.hd) nmax = std::max(nmax, d.n * k);
  g_finish<<<dim3(std::min<unsigned>(cdivu(nmax, 256), 1024), nb), 256, 0, s>>>(S.d_desc);
  launches += 1;
  std::vector<LsqrScalars> hs((size_t)nb * K8);
  for (int i = 0; i < nb; ++i)
    BCK(cudaMemcpyAsync(hs.data() + (size_t)i * K8, S.hd[i].sc, K8 * sizeof(LsqrScalars), cudaMemcpyDeviceToHost, s));
  int hflag = 0;
  BCK(cudaMemcpyAsync(&hflag, S.errflag, sizeof(int), cudaMemcpyDeviceToHost, s));
  BCK(cudaStreamSynchronize(s));
  BCK(cudaGetLastError());
  if (hflag) { err = "a bounded barrier wait in a batched sweep gave up"; return false; }
  nit.assign((size_t)nb * k, 0);
  istop.assign((size_t)nb * k, 0);
  for (int i = 0; i < nb; ++i)
    for (int c = 0; c < k; ++c) {
      nit[(size_t)i * k + c] = hs[(size_t)i * K8 + c].itn;
      istop[(size_t)i * k + c] = hs[(size_t)i * K8 + c].istop;
    }
  if (st) {
    st->av_ms += av_ms; st->atu_ms += atu_ms;
    st->av_launches += nav; st->atu_launches += natu;
    st->launches += launches;
    st->iterations = std::max(st->iterations, iters);
    st->av_rows = AVP_R;
    st->atu_rs = ATUP_RS;
    st->atu_rows = tune.atup_rows;
    for (int i = 0; i < nb; ++i) {
      int mx = 0;
      for (int c = 0; c < k; ++c) mx = std::max(mx, nit[(size_t)i * k + c]);
      st->bytes_av += (double)mx * 24.0 * (double)S.hd[i].pk_ne * (double)S.hd[i].pk_ne;
    }
  }
  return true;
}

bool batch_bicgstab_solve(const std::vector<BatchBody>& bodies, int k, double tol, int maxit, cudaStream_t s,
                          std::vector<int>& nit, std::vector<int>& status, BatchStats* st, std::string& err,
                          const std::vector<double>* tol_cols) {
  BatchSolver S;
  if (!S.setup(bodies, k, maxit, BatchTune(), s, true)) { err = S.err; return false; }
  BCK(set_smem(gb_avp, AVP_SMEM));
  const int nb = S.nb;
  std::vector<double> htol;
  if (tol_cols) {
    if (tol_cols->size() != (size_t)nb * k) { err = "tol_cols must hold one tolerance per right-hand side"; return false; }
    htol.assign((size_t)nb * K8, tol);
    for (int i = 0; i < nb; ++i)
      for (int c = 0; c < k; ++c) htol[(size_t)i * K8 + c] = (*tol_cols)[(size_t)i * k + c];
    for (int i = 0; i < nb; ++i) {
      BCK(cudaMemcpyAsync(S.tolc_dev[i], htol.data() + (size_t)i * K8, K8 * sizeof(double), cudaMemcpyHostToDevice, s));
      S.hd[i].tolc = S.tolc_dev[i];
    }
    BCK(cudaMemcpyAsync(S.d_desc, S.hd.data(), nb * sizeof(GDesc), cudaMemcpyHostToDevice, s));
  }
  int itmax = 0;
  for (const auto& d : S.hd) itmax = std::max(itmax, d.itnlim);
  long launches = 0;
  BCK(cudaMemsetAsync(S.nactive, 0, sizeof(int), s));
  gb_diag<<<S.hoff_b[nb], BT, 0, s>>>(S.d_desc, S.off.b, nb, S.nactive);
  int bad = 0;
  BCK(cudaMemcpyAsync(&bad, S.nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
  BCK(cudaStreamSynchronize(s));
  if (bad) {
    err = "BiCGSTAB: a zero or non-finite diagonal entry (the Jacobi preconditioner needs every diagonal)";
    return false;
  }
  gb_init<<<S.hoff_b[nb], BT, 0, s>>>(S.d_desc, S.off.b, nb);
  gb_scal<<<nb, 256, 0, s>>>(S.d_desc, 0, S.bact, S.nactive, tol);
  launches += 3;
  BCK(cudaGetLastError());
  const int ce = 8;
  std::vector<cudaEvent_t> ev(4 * ce, nullptr);
  for (auto& e : ev) BCK(cudaEventCreate(&e));
  const unsigned nbv = S.hoff_b[nb], nav = S.hoff_av[nb];
  auto iteration = [&](int i) {
    gb_p<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact);
    cudaEventRecordWithFlags(ev[4 * i], s, cudaEventRecordExternal);
    gb_avp<<<nav, AVP_THREADS, AVP_SMEM, s>>>(S.d_desc, S.off.av, nb, S.bact, S.errflag, 0);
    cudaEventRecordWithFlags(ev[4 * i + 1], s, cudaEventRecordExternal);
    gb_dots<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact, 0);
    gb_scal<<<nb, 256, 0, s>>>(S.d_desc, 1, S.bact, S.nactive, tol);
    gb_s<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact);
    gb_scal<<<nb, 256, 0, s>>>(S.d_desc, 2, S.bact, S.nactive, tol);
    cudaEventRecordWithFlags(ev[4 * i + 2], s, cudaEventRecordExternal);
    gb_avp<<<nav, AVP_THREADS, AVP_SMEM, s>>>(S.d_desc, S.off.av, nb, S.bact, S.errflag, 1);
    cudaEventRecordWithFlags(ev[4 * i + 3], s, cudaEventRecordExternal);
    gb_dots<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact, 1);
    gb_scal<<<nb, 256, 0, s>>>(S.d_desc, 3, S.bact, S.nactive, tol);
    gb_xr<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact);
    cudaMemsetAsync(S.nactive, 0, sizeof(int), s);
    gb_scal<<<nb, 256, 0, s>>>(S.d_desc, 4, S.bact, S.nactive, tol);
  };
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool ok = true;
  auto cleanup = [&]() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ev) if (e) cudaEventDestroy(e);
  };
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) ok = false;
  if (ok) {
    for (int i = 0; i < ce; ++i) iteration(i);
    if (cudaStreamEndCapture(s, &graph) != cudaSuccess) ok = false;
  }
  if (ok && cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) ok = false;
  if (!ok) {
    err = std::string("batch BiCGSTAB graph capture: ") + cudaGetErrorString(cudaGetLastError());
    cleanup();
    return false;
  }
  std::vector<int> hb(nb);
  if (cudaMemcpyAsync(hb.data(), S.bact, nb * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    err = "batch BiCGSTAB: initial state";
    cleanup();
    return false;
  }
  int act = 0;
  for (int v : hb) act += v;
  long iters = 0;
  double av_ms = 0.0;
  long nav_t = 0;
  while (act > 0 && iters < (long)itmax + ce) {
    if (cudaGraphLaunch(gexec, s) != cudaSuccess) { ok = false; break; }
    launches += 11L * ce;
    cudaMemcpyAsync(S.h_nactive, S.nactive, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) { ok = false; break; }
    for (int i = 0; i < ce; ++i) {
      float a = 0.f, b = 0.f;
      if (cudaEventElapsedTime(&a, ev[4 * i], ev[4 * i + 1]) == cudaSuccess) { av_ms += a; ++nav_t; }
      if (cudaEventElapsedTime(&b, ev[4 * i + 2], ev[4 * i + 3]) == cudaSuccess) { av_ms += b; ++nav_t; }
    }
    (void)cudaGetLastError();
    iters += ce;
    act = *S.h_nactive;
  }
  cleanup();
  if (!ok) {
    err = std::string("batch BiCGSTAB iterations: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  int mmax = 1;
  for (const auto& d : S.hd) mmax = std::max(mmax, d.m * K8);
  gb_finish<<<dim3(std::min<unsigned>(cdivu(mmax, 256), 1024), nb), 256, 0, s>>>(S.d_desc);
  // the true residual of every right-hand side, FP64 (the recursive residual
  // of the FP32 products can drift from it)
  for (int i = 0; i < nb; ++i) BCK(cudaMemsetAsync(S.hd[i].rr, 0, K8 * sizeof(double), s));
  gb_resid<<<2 * S.hoff_av[nb], 256, 0, s>>>(S.d_desc, S.off.av, nb);
  launches += 2;
  std::vector<BicgScalars> hs((size_t)nb * K8);
  std::vector<double> hrr((size_t)nb * K8);
  for (int i = 0; i < nb; ++i) {
    BCK(cudaMemcpyAsync(hs.data() + (size_t)i * K8, S.hd[i].bs, K8 * sizeof(BicgScalars), cudaMemcpyDeviceToHost, s));
    BCK(cudaMemcpyAsync(hrr.data() + (size_t)i * K8, S.hd[i].rr, K8 * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  int hflag = 0;
  BCK(cudaMemcpyAsync(&hflag, S.errflag, sizeof(int), cudaMemcpyDeviceToHost, s));
  BCK(cudaStreamSynchronize(s));
  BCK(cudaGetLastError());
  if (hflag) { err = "a bounded barrier wait in a batched sweep gave up"; return false; }
  nit.assign((size_t)nb * k, 0);
  status.assign((size_t)nb * k, 0);
  for (int i = 0; i < nb; ++i)
    for (int c = 0; c < k; ++c) {
      const BicgScalars& q = hs[(size_t)i * K8 + c];
      nit[(size_t)i * k + c] = q.its;
      int stt = q.status < 0 ? 1 : q.status;
      // converged by its recursive residual but not by the true one: 4
      const double rel = q.bnorm > 0.0 ? std::sqrt(hrr[(size_t)i * K8 + c]) / q.bnorm : 0.0;
      if (stt == 0 && !(rel <= (tol_cols ? htol[(size_t)i * K8 + c] : tol))) stt = 4;
      status[(size_t)i * k + c] = stt;
    }
  if (st) {
    st->av_ms += av_ms;
    st->av_launches += nav_t;
    st->launches += launches;
    st->iterations = std::max(st->iterations, iters);
    st->av_rows = AVP_R;
    for (int i = 0; i < nb; ++i) {
      int mx = 0;
      for (int c = 0; c < k; ++c) mx = std::max(mx, nit[(size_t)i * k + c]);
      st->bytes_av += 2.0 * (double)mx * 24.0 * (double)S.hd[i].pk_ne * (double)S.hd[i].pk_ne;
    }
  }
  return true;
}

bool batch_gmres_solve(const std::vector<BatchBody>& bodies, int k, double tol, int maxit, int restart,
                       cudaStream_t s, std::vector<int>& nit, std::vector<int>& status, BatchStats* st,
                       std::string& err) {
  if (restart < 1 || restart > 512) { err = "GMRES restart length must be 1..512"; return false; }
  const int mr = restart;
  BatchSolver S;
  if (!S.setup(bodies, k, maxit > 0 ? maxit : 1000, BatchTune(), s, false, true, mr)) { err = S.err; return false; }
  BCK(set_smem(gb_avp, AVP_SMEM));
  const int nb = S.nb;
  int itmax = 0;
  for (const auto& d : S.hd) itmax = std::max(itmax, d.itnlim);
  long launches = 0;
  {  // the inverse self blocks of every system
    int nemax = 1;
    for (const auto& d : S.hd) nemax = std::max(nemax, d.pk_ne);
    BCK(cudaMemsetAsync(S.nactive, 0, sizeof(int), s));
    g_pc_blocks<<<dim3(cdivu(nemax, 128), nb), 128, 0, s>>>(S.d_desc, S.nactive);
    int bad = 0;
    BCK(cudaMemcpyAsync(&bad, S.nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
    ++launches;
    if (bad) { err = "a singular 3x3 self block: the block preconditioner cannot be formed"; return false; }
  }
  const unsigned nbv = S.hoff_b[nb], nav = S.hoff_av[nb];
  gg_load<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bran, 1);
  BCK(cudaMemsetAsync(S.nactive, 0, sizeof(int), s));
  gg_begin<<<nb, 256, 0, s>>>(S.d_desc, S.bact, S.bran, S.nactive, tol, 1);
  launches += 2;
  BCK(cudaGetLastError());
  cudaEvent_t ev[2] = {nullptr, nullptr};
  for (auto& e : ev) BCK(cudaEventCreate(&e));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  auto cleanup = [&]() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ev) if (e) cudaEventDestroy(e);
  };
  bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    for (int j = 0; j < mr; ++j) {
      gg_pc<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact, j);
      if (j == 0) cudaEventRecordWithFlags(ev[0], s, cudaEventRecordExternal);
      gb_avp<<<nav, AVP_THREADS, AVP_SMEM, s>>>(S.d_desc, S.off.av, nb, S.bact, S.errflag, 0);
      if (j == 0) cudaEventRecordWithFlags(ev[1], s, cudaEventRecordExternal);
      for (int pass = 0; pass < 2; ++pass) {
        gg_dots<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact, j);
        gg_hred<<<nb, 256, 0, s>>>(S.d_desc, S.bact, j, pass);
        gg_orth<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bact, j);
      }
      cudaMemsetAsync(S.nactive, 0, sizeof(int), s);
      gg_givens<<<nb, 256, 0, s>>>(S.d_desc, S.bact, S.nactive, tol, j);
    }
    ok = cudaStreamEndCapture(s, &graph) == cudaSuccess;
  }
  if (ok) ok = cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess;
  if (!ok) {
    err = std::string("batch GMRES graph capture: ") + cudaGetErrorString(cudaGetLastError());
    cleanup();
    return false;
  }
  double av_ms = 0.0, timed_bytes = 0.0;
  long nav_t = 0, cycles = 0;
  std::vector<int> hbran(nb, 0);
  for (int cyc = 0; cyc < itmax + 2; ++cyc) {
    if (cudaMemcpyAsync(S.h_nactive, S.nactive, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(hbran.data(), S.bran, nb * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { ok = false; break; }
    if (*S.h_nactive == 0) break;
    // algorithmic bytes of the cycle's first (timed) sweep: the systems in it
    double cyc_bytes = 0.0;
    for (int i = 0; i < nb; ++i)
      if (hbran[i]) cyc_bytes += 24.0 * (double)S.hd[i].pk_ne * (double)S.hd[i].pk_ne;
    if (cudaGraphLaunch(gexec, s) != cudaSuccess) { ok = false; break; }
    launches += 9L * mr;
    ++cycles;
    // iterate update, float-float true residual and the start of the next cycle
    gg_solve<<<nb, 32, 0, s>>>(S.d_desc, S.bran);
    gg_xupd<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bran);
    gg_split<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bran);
    if (k <= 6) gg_resid<6><<<2 * nav, 256, 0, s>>>(S.d_desc, S.off.av, nb, S.bran);
    else gg_resid<8><<<2 * nav, 256, 0, s>>>(S.d_desc, S.off.av, nb, S.bran);
    gg_load<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb, S.bran, 0);
    cudaMemsetAsync(S.nactive, 0, sizeof(int), s);
    gg_begin<<<nb, 256, 0, s>>>(S.d_desc, S.bact, S.bran, S.nactive, tol, 0);
    launches += 6;
    float a = 0.f;
    if (cudaEventSynchronize(ev[1]) == cudaSuccess && cudaEventElapsedTime(&a, ev[0], ev[1]) == cudaSuccess) {
      av_ms += a;
      ++nav_t;
      timed_bytes += cyc_bytes;
    }
    (void)cudaGetLastError();
  }
  cleanup();
  if (!ok) {
    err = std::string("batch GMRES cycles: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  gg_out<<<nbv, BT, 0, s>>>(S.d_desc, S.off.b, nb);
  ++launches;
  std::vector<GmresScalars> hs((size_t)nb * K8);
  for (int i = 0; i < nb; ++i)
    BCK(cudaMemcpyAsync(hs.data() + (size_t)i * K8, S.hd[i].gs, K8 * sizeof(GmresScalars), cudaMemcpyDeviceToHost,
                        s));
  int hflag = 0;
  BCK(cudaMemcpyAsync(&hflag, S.errflag, sizeof(int), cudaMemcpyDeviceToHost, s));
  BCK(cudaStreamSynchronize(s));
  BCK(cudaGetLastError());
  if (hflag) { err = "a bounded barrier wait in a batched sweep gave up"; return false; }
  nit.assign((size_t)nb * k, 0);
  status.assign((size_t)nb * k, 0);
  long maxits = 0;
  for (int i = 0; i < nb; ++i)
    for (int c = 0; c < k; ++c) {
      const GmresScalars& q = hs[(size_t)i * K8 + c];
      nit[(size_t)i * k + c] = q.its;
      status[(size_t)i * k + c] = q.status < 0 ? 1 : q.status;
      maxits = std::max<long>(maxits, q.its);
    }
  if (st) {
    // the first A*V sweep of every cycle is timed (live events), with the
    // algorithmic bytes of the systems it covered
    st->av_ms += av_ms;
    st->av_launches += nav_t;
    st->launches += launches;
    st->iterations = std::max(st->iterations, maxits);
    st->av_rows = AVP_R;
    st->bytes_av += timed_bytes;
  }
  if (st) st->cycles += cycles;
  return true;
}

// ---------------------------------------------------------------------------
// True residual of many systems (FP64), for the BiCGSTAB restarts
// ---------------------------------------------------------------------------
struct RDesc {
  const float* A;
  int pk_ne, pk_ldp, m, n, k;
  const double* b;
  const double* x;
  double* r;   // [k][m] or null
  double* ss;  // [2][K8]: ||r||^2, ||b||^2 per right-hand side
};

// a warp per element row i (its three equations), lanes over the element
// columns; CTAs of 8 rows, off[] = prefix of the CTAs per system
__global__ void __launch_bounds__(256) gb_residual(const RDesc* __restrict__ D, const int* __restrict__ off, int nb) {
  const int bi = find_body(off, nb, blockIdx.x);
  const RDesc& d = D[bi];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = (blockIdx.x - off[bi]) * 8 + warp;
  if (i >= d.pk_ne) return;  // a whole warp; no block barrier in this kernel
  const int ne = d.pk_ne;
  double acc[3][K8];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) acc[a][c] = 0.0;
  for (int j = lane; j < ne; j += 32) {
    double g6[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) g6[c] = (double)d.A[pk_idx(i, c, j, d.pk_ldp)];
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = 0; c < K8; ++c) {
        if (c >= d.k) break;
        const double xv = d.x[(int64_t)c * d.n + (int64_t)b * ne + j];
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[a][c] += g6[sym6(a, b)] * xv;
      }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) {
      double v = acc[a][c];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0 && c < d.k) {
        const int64_t row = 3 * (int64_t)i + a;
        const double bv = d.b[(int64_t)c * d.m + row];
        const double r = bv - v;
        if (d.r) d.r[(int64_t)c * d.m + row] = r;
        atomicAdd(&d.ss[c], r * r);
        atomicAdd(&d.ss[K8 + c], bv * bv);
      }
    }
}

bool batch_residual(const std::vector<BatchBody>& bodies, int k, cudaStream_t s, const std::vector<double*>& r_out,
                    std::vector<double>& rel, std::string& err) {
  const int nb = (int)bodies.size();
  rel.assign((size_t)nb * k, 0.0);
  if (nb == 0) return true;
  std::vector<RDesc> hd(nb);
  std::vector<int> off(nb + 1, 0);
  RDesc* dd = nullptr;
  int* doff = nullptr;
  double* ss = nullptr;
  bool ok = false;
  std::vector<double> hss((size_t)nb * 2 * K8);
  for (int i = 0; i < nb; ++i) {
    const BatchBody& B = bodies[i];
    hd[i] = RDesc{B.A, B.pk_ne, B.pk_ldp, B.m, B.n, k, B.b, B.x, r_out.empty() ? nullptr : r_out[i], nullptr};
    off[i + 1] = off[i] + (int)cdivu(B.pk_ne, 8);
  }
#define RCK(x)                                                                   \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      goto done;                                                                 \
    }                                                                            \
  } while (0)
  RCK(cudaMallocAsync(&dd, nb * sizeof(RDesc), s));
  RCK(cudaMallocAsync(&doff, (nb + 1) * sizeof(int), s));
  RCK(cudaMallocAsync(&ss, (size_t)nb * 2 * K8 * sizeof(double), s));
  RCK(cudaMemsetAsync(ss, 0, (size_t)nb * 2 * K8 * sizeof(double), s));
  for (int i = 0; i < nb; ++i) hd[i].ss = ss + (size_t)i * 2 * K8;
  RCK(cudaMemcpyAsync(dd, hd.data(), nb * sizeof(RDesc), cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(doff, off.data(), (nb + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  gb_residual<<<off[nb], 256, 0, s>>>(dd, doff, nb);
  RCK(cudaGetLastError());
  RCK(cudaMemcpyAsync(hss.data(), ss, hss.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  RCK(cudaStreamSynchronize(s));  // the host tables above must outlive their copies
  for (int i = 0; i < nb; ++i)
    for (int c = 0; c < k; ++c) {
      const double rr = hss[(size_t)i * 2 * K8 + c], bb = hss[(size_t)i * 2 * K8 + K8 + c];
      rel[(size_t)i * k + c] = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    }
  ok = true;
done:
#undef RCK
  if (dd) cudaFreeAsync(dd, s);
  if (doff) cudaFreeAsync(doff, s);
  if (ss) cudaFreeAsync(ss, s);
  return ok;
}

__global__ void k_batch_axpy(int64_t n, const double* __restrict__ d, double* __restrict__ x) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    x[t] += d[t];
}
bool batch_axpy(const std::vector<BatchBody>& bodies, int k, const std::vector<double*>& d, cudaStream_t s,
                std::string& err) {
  for (size_t i = 0; i < bodies.size(); ++i) {
    const int64_t n = (int64_t)k * bodies[i].n;
    k_batch_axpy<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(n, d[i], bodies[i].x);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    err = std::string("batch axpy: ") + cudaGetErrorString(e);
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Autotuner: times the candidate row groups of the A^T*U sweep on the given
// systems (warm-up launch + 3 timed launches each, CUDA events), keeps the
// fastest.  The vectors are zero: the sweeps' cost does not
// depend on the values.
// ---------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::map<std::string, BatchTune> g_tune_cache;

bool batch_autotune(const std::vector<BatchBody>& bodies, cudaStream_t s, BatchTune& best, std::string& report,
                    std::string& err) {
  double tot = 0.0;
  for (const auto& b : bodies) tot += 24.0 * (double)b.pk_ne * (double)b.pk_ldp;
  int nbk = 0;
  for (size_t v = bodies.size(); v > 1; v >>= 1) ++nbk;
  int tbk = 0;
  for (double v = tot / 1e6; v > 1.0; v /= 2.0) ++tbk;
  const std::string key = std::to_string(nbk) + "/" + std::to_string(tbk);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      best = it->second;
      report = "cached " + key;
      return true;
    }
  }
  cudaEvent_t e0, e1;
  BCK(cudaEventCreate(&e0));
  BCK(cudaEventCreate(&e1));
  auto time_it = [&](BatchSolver& S, bool av) -> double {
    if (av) S.launch_av(); else S.launch_atu();
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; ++r) { if (av) S.launch_av(); else S.launch_atu(); }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / 3.0;
  };
  char line[160];
  report.clear();
  BatchTune t0 = best;
  double best_atu = 1e300;
  // block rows per A^T*U row group (the A*V tile shape is fixed)
  const int grp_rows[] = {512, 1024, 4096};
  for (int g : grp_rows) {
    BatchTune t = t0;
    t.atup_rows = g;
    BatchSolver S;
    if (!S.setup(bodies, 1, 1, t, s)) { err = S.err; cudaEventDestroy(e0); cudaEventDestroy(e1); return false; }
    const double ms = time_it(S, false);
    snprintf(line, sizeof line, "atup rows=%d: %.3f ms; ", g, ms);
    report += line;
    if (ms < best_atu) { best_atu = ms; best.atup_rows = g; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  BCK(cudaGetLastError());
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = best;
  return true;
}

}  // namespace agb
