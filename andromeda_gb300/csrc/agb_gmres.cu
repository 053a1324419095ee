// Restarted GMRES on the packed Stokes single layer: the LIS path's solver with
// the options "-i gmres -restart m" (the reference passes its LIS options string
// from the input file to lis_solver_set_option, src/mod_par.f90:288,418 and
// src/mod_plis.f90:235; LIS's default restart length is 40).  LIS is not part
// of the reference sources; the method is the published GMRES(m) of Saad and
// Schultz (SIAM J. Sci. Stat. Comput. 7, 1986) with Givens rotations, as in
// Saad, "Iterative Methods for Sparse Linear Systems", 2nd ed., Alg. 6.9, with
// a right preconditioner, so that the residual it minimises is the
// unpreconditioned ||b - A x||_2 and the stop is ||b - A x|| <= tol ||b||, LIS's
// default criterion.
//
// The preconditioner is the inverse of every element's 3x3 self block (the
// block-Jacobi preconditioner of the block LSQR, DenseLsqr::block_precon).
// Vectors are held as BiCGSTAB holds them: row numbering u = 3i+a, [m][8] FP64
// for up to 8 right-hand sides, each column its own Krylov space; the sweep
// operand W[b][c][i] = fp32((M^-1 v)[3i+b]) feeds k_avp over the FP32 blocks.
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2), FP64, with
// inner products reduced over a fixed grid in a fixed order (bitwise
// reproducible).  One restart cycle (m Arnoldi steps, 9 kernels each) is one
// CUDA graph, replayed per cycle; kernels of a step return at once when no
// right-hand side is active, so a cycle whose columns all converged early
// costs only launches.
//
// With FP32 products the Arnoldi relation holds to the FP32 rounding of A, so
// the residual estimate |g_{j+1}| can fall below the true residual: a cycle's
// steps run until the estimate is below kGmresInner x tol.  At the end of
// every cycle the iterate is updated and its true residual b - A x is formed
// over the stored matrix in float-float (or FP64) arithmetic
// (DenseLsqr::residual); a column is converged when that residual is within
// tol, and the next cycle starts from it otherwise (iterative refinement in
// extended precision around the FP32 Krylov solver).  A cycle that does not
// lower a column's true residual by 10 % stops that column with status 3.
#include "agb_lsqr.cuh"
#include "agb_sweeps.cuh"
#include <algorithm>
#include <cmath>

namespace agb {

#define GCK(x)                                                                   \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      return false;                                                              \
    }                                                                            \
  } while (0)

namespace {

constexpr int GM_THREADS = 256;  // 32 rows x 8 right-hand sides per pass of a CTA
constexpr int GM_BLOCKS = 304;   // 2 CTAs per SM on 152 SMs; fixed, so partial sums reduce in a fixed order
// A cycle's Arnoldi steps run until the residual estimate |g_{j+1}| is below
// kGmresInner * tol ||b||: with FP32 products the estimate runs ahead of the
// true residual, and the margin lets the true residual formed at the end of
// the cycle meet tol without a second cycle (and a second true residual).
constexpr double kGmresInner = 0.5;

inline unsigned gdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// CTA sum of v over the threads with equal threadIdx.x & 7 (one right-hand side)
__device__ __forceinline__ void gm_sum8(double v, double* sred, double* out) {
  v += __shfl_down_sync(0xffffffffu, v, 16);
  v += __shfl_down_sync(0xffffffffu, v, 8);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < 8) sred[warp * 8 + lane] = v;
  __syncthreads();
  if (threadIdx.x < 8) {
    double t = 0.0;
    for (int w = 0; w < GM_THREADS / 32; ++w) t += sred[w * 8 + threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// partial p of right-hand side c summed over the CTAs by one warp in a fixed
// order: lane k adds CTAs k, k+32, ..., then a butterfly over the lanes (every
// lane ends with the same bits: each level adds the same two values).  All 32
// lanes must call it.
__device__ __forceinline__ double gm_total(const double* part, int np, int p, int c) {
  const int lane = threadIdx.x & 31;
  double t = 0.0;
  for (int b = lane; b < GM_BLOCKS; b += 32) t += part[((size_t)b * np + p) * 8 + c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  return t;
}

// w = r (r column-major m x k, or b on the first cycle); partial 0: ||w||^2
__global__ void __launch_bounds__(GM_THREADS) k_gm_load(int m, int k, const double* __restrict__ r,
                                                       double* __restrict__ w, double* __restrict__ part, int np) {
  __shared__ double sred[GM_THREADS / 32 * 8];
  const int c = threadIdx.x & 7;
  double ss = 0.0;
  for (long long t = (long long)blockIdx.x * GM_THREADS + threadIdx.x; t < (long long)m * 8;
       t += (long long)GM_BLOCKS * GM_THREADS) {
    const double v = (c < k) ? r[(size_t)c * m + (t >> 3)] : 0.0;
    w[t] = v;
    ss += v * v;
  }
  gm_sum8(ss, sred, part + (size_t)blockIdx.x * np * 8);
}

// start of a cycle: beta = ||r||; the first call also takes ||b||.  A column
// still running (status -1) is converged if its true residual is within tol,
// stops at the iteration limit (1) or when the last cycle did not lower its
// true residual by 10 % (3); otherwise it runs this cycle with g = beta e1.
__global__ void k_gm_begin(const double* __restrict__ part, int np, int k, double tol, int maxit, int first,
                           GmresScalars* __restrict__ s, double* __restrict__ g, int* __restrict__ nactive) {
  const int c = threadIdx.x;
  double tot = 0.0;
  for (int cc = 0; cc < 8; ++cc) {
    const double t = gm_total(part, np, 0, cc);
    if (cc == c) tot = t;
  }
  if (c < 8) {
    GmresScalars& q = s[c];
    const double beta = sqrt(tot);
    if (first) {
      q.bnorm = beta;
      q.its = 0;
      q.cycles = 0;
      q.status = (c < k && beta > 0.0) ? -1 : 0;
      q.prev = 1.0;
      q.relres = (beta > 0.0) ? 1.0 : 0.0;
    }
    q.jc = 0;
    if (q.status == -1) {
      const double rel = beta / q.bnorm;
      q.relres = rel;
      if (rel <= tol) q.status = 0;
      else if (q.its >= maxit) q.status = 1;
      else if (!first && rel > 0.9 * q.prev) q.status = 3;
      q.prev = rel;
    }
    q.active = (q.status == -1) ? 1 : 0;
    if (q.active) q.cycles += 1;
    q.beta = beta;
    q.hnext = beta;
    g[c] = beta;
  }
  __syncwarp();
  if (c == 0) {
    int na = 0;
    for (int cc = 0; cc < 8; ++cc) na += s[cc].active;
    *nactive = na;
  }
}

// Arnoldi step j: v_j = w / h (h = beta for j = 0, else the norm of the last
// orthogonalised w); W = fp32(M^-1 v_j) in the sweep layout W[b][c][i]
// (zero for a column that is not active).  A thread per (element, column).
__global__ void __launch_bounds__(GM_THREADS) k_gm_pc(int ne, int ldp, int j, const double* __restrict__ w,
                                                     double* __restrict__ Vj, const double* __restrict__ pc9,
                                                     const GmresScalars* __restrict__ s,
                                                     float* __restrict__ W, const int* __restrict__ gate) {
  if (*gate == 0) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ne * 8) return;
  const int i = (int)(t >> 3), c = (int)(t & 7);
  const GmresScalars& q = s[c];
  float o[3] = {0.f, 0.f, 0.f};
  if (q.active) {
    const double inv = 1.0 / q.hnext;
    double v[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const size_t id = (size_t)(3 * i + a) * 8 + c;
      v[a] = w[id] * inv;
      Vj[id] = v[a];
    }
    const double* mi = pc9 + 9 * (size_t)i;
#pragma unroll
    for (int b = 0; b < 3; ++b) o[b] = (float)(mi[3 * b] * v[0] + mi[3 * b + 1] * v[1] + mi[3 * b + 2] * v[2]);
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a) Vj[(size_t)(3 * i + a) * 8 + c] = 0.0;
  }
#pragma unroll
  for (int b = 0; b < 3; ++b) W[((size_t)b * 8 + c) * ldp + i] = o[b];
}

// partial l (l = 0..j): v_l . w.  Eight basis vectors per pass over w (one
// CTA reduction per eight); each partial sums its thread's terms in index
// order, then over the warp and the CTA as gm_sum8 does.
__global__ void __launch_bounds__(GM_THREADS) k_gm_dots(int m, int j, const double* __restrict__ Vb,
                                                       size_t vstride, const double* __restrict__ w,
                                                       double* __restrict__ part, int np,
                                                       const int* __restrict__ gate) {
  if (*gate == 0) return;
  constexpr int LB = 8;
  __shared__ double sred[GM_THREADS / 32][LB][8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int l0 = 0; l0 <= j; l0 += LB) {
    const int nl = min(LB, j + 1 - l0);
    double d[LB];
#pragma unroll
    for (int u = 0; u < LB; ++u) d[u] = 0.0;
    for (long long t = (long long)blockIdx.x * GM_THREADS + threadIdx.x; t < (long long)m * 8;
         t += (long long)GM_BLOCKS * GM_THREADS) {
      const double wv = w[t];
#pragma unroll
      for (int u = 0; u < LB; ++u)
        if (u < nl) d[u] += Vb[(size_t)(l0 + u) * vstride + t] * wv;
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      double v = d[u];
      v += __shfl_down_sync(0xffffffffu, v, 16);
      v += __shfl_down_sync(0xffffffffu, v, 8);
      if (lane < 8) sred[warp][u][lane] = v;
    }
    __syncthreads();
    if (threadIdx.x < LB * 8) {
      const int u = threadIdx.x >> 3, c = threadIdx.x & 7;
      if (u < nl) {
        double tsum = 0.0;
        for (int ww = 0; ww < GM_THREADS / 32; ++ww) tsum += sred[ww][u][c];
        part[((size_t)blockIdx.x * np + l0 + u) * 8 + c] = tsum;
      }
    }
    __syncthreads();
  }
}

// hc[l] = v_l . w (l = 0..j) from the partials; H[l][j] = hc (pass 0) or += hc (pass 1).
// CTA l, warp c (8 warps).
__global__ void __launch_bounds__(256) k_gm_hred(int j, int mr, const double* __restrict__ part, int np, int pass,
                                                 double* __restrict__ hc, double* __restrict__ H,
                                                 const int* __restrict__ gate) {
  if (*gate == 0) return;
  const int l = blockIdx.x, c = threadIdx.x >> 5;
  if (l > j) return;
  const double v = gm_total(part, np, l, c);
  if ((threadIdx.x & 31) == 0) {
    hc[l * 8 + c] = v;
    double* h = H + ((size_t)l * mr + j) * 8 + c;
    *h = pass ? *h + v : v;
  }
}

// w -= sum_l hc[l] v_l over the active columns; partial 0: ||w||^2
__global__ void __launch_bounds__(GM_THREADS) k_gm_orth(int m, int j, const double* __restrict__ Vb,
                                                       size_t vstride, const double* __restrict__ hc,
                                                       const GmresScalars* __restrict__ s, double* __restrict__ w,
                                                       double* __restrict__ part, int np,
                                                       const int* __restrict__ gate) {
  if (*gate == 0) return;
  __shared__ double sred[GM_THREADS / 32 * 8];
  const int c = threadIdx.x & 7;
  const bool act = s[c].active != 0;
  double ss = 0.0;
  for (long long t = (long long)blockIdx.x * GM_THREADS + threadIdx.x; t < (long long)m * 8;
       t += (long long)GM_BLOCKS * GM_THREADS) {
    if (!act) continue;
    double v = w[t];
#pragma unroll 8
    for (int l = 0; l <= j; ++l) v -= hc[l * 8 + c] * Vb[(size_t)l * vstride + t];
    w[t] = v;
    ss += v * v;
  }
  gm_sum8(ss, sred, part + (size_t)blockIdx.x * np * 8);
}

// end of step j: h_{j+1,j} = ||w||, the previous rotations applied to column j
// of H, a new rotation that zeroes h_{j+1,j}, g updated; the column leaves the
// cycle when |g_{j+1}| <= tol ||b|| (tol: the in-cycle target kGmresInner x the solve's), on a breakdown (h_{j+1,j} = 0: the Krylov
// space is invariant), at the end of the cycle or at the iteration limit
__global__ void k_gm_givens(int j, int mr, const double* __restrict__ part, int np, double tol, int maxit,
                            double* __restrict__ H, double* __restrict__ cs, double* __restrict__ sn,
                            double* __restrict__ g, GmresScalars* __restrict__ s, int* __restrict__ nactive) {
  if (*nactive == 0) return;
  const int c = threadIdx.x;
  double tot = 0.0;
  for (int cc = 0; cc < 8; ++cc) {
    const double t = gm_total(part, np, 0, cc);
    if (cc == c) tot = t;
  }
  if (c < 8) {
    GmresScalars& q = s[c];
    if (q.active) {
      const double hn = sqrt(tot);
      for (int l = 0; l < j; ++l) {
        double* a0 = H + ((size_t)l * mr + j) * 8 + c;
        double* a1 = H + ((size_t)(l + 1) * mr + j) * 8 + c;
        const double x0 = *a0, x1 = *a1, cc = cs[l * 8 + c], ss = sn[l * 8 + c];
        *a0 = cc * x0 + ss * x1;
        *a1 = -ss * x0 + cc * x1;
      }
      double* hjj = H + ((size_t)j * mr + j) * 8 + c;
      const double hd = *hjj;
      const double r = hypot(hd, hn);
      double cc = 1.0, ss = 0.0;
      if (r > 0.0) {
        cc = hd / r;
        ss = hn / r;
      }
      *hjj = r;
      cs[j * 8 + c] = cc;
      sn[j * 8 + c] = ss;
      const double gj = g[j * 8 + c];
      g[(j + 1) * 8 + c] = -ss * gj;
      g[j * 8 + c] = cc * gj;
      q.its += 1;
      q.jc = j + 1;
      q.hnext = hn;
      q.relres = fabs(g[(j + 1) * 8 + c]) / q.bnorm;
      if (q.relres <= tol || !(hn > 0.0) || j + 1 == mr || q.its >= maxit) q.active = 0;
    }
  }
  __syncwarp();
  if (c == 0) {
    int na = 0;
    for (int cc = 0; cc < 8; ++cc) na += s[cc].active;
    *nactive = na;
  }
}

// y = R^-1 g over the jc steps of the cycle (back substitution, per column)
__global__ void k_gm_solve(int mr, const double* __restrict__ H, const double* __restrict__ g,
                           const GmresScalars* __restrict__ s, double* __restrict__ y) {
  const int c = threadIdx.x;
  if (c >= 8) return;
  const int jc = s[c].jc;
  for (int l = jc - 1; l >= 0; --l) {
    double v = g[l * 8 + c];
    for (int p = l + 1; p < jc; ++p) v -= H[((size_t)l * mr + p) * 8 + c] * y[p * 8 + c];
    const double d = H[((size_t)l * mr + l) * 8 + c];
    y[l * 8 + c] = (d != 0.0) ? v / d : 0.0;
  }
}

// X += M^-1 (sum_l y_l v_l): a thread per (element, column); X in the row
// numbering 3i+b of the unknown b ne + i
__global__ void __launch_bounds__(GM_THREADS) k_gm_xupd(int ne, const double* __restrict__ Vb, size_t vstride,
                                                       const double* __restrict__ y, const double* __restrict__ pc9,
                                                       const GmresScalars* __restrict__ s, double* __restrict__ X) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ne * 8) return;
  const int i = (int)(t >> 3), c = (int)(t & 7);
  const int jc = s[c].jc;
  if (jc == 0) return;
  double z[3] = {0.0, 0.0, 0.0};
  for (int l = 0; l < jc; ++l) {
    const double yl = y[l * 8 + c];
    const double* v = Vb + (size_t)l * vstride;
#pragma unroll
    for (int a = 0; a < 3; ++a) z[a] += yl * v[(size_t)(3 * i + a) * 8 + c];
  }
  const double* mi = pc9 + 9 * (size_t)i;
#pragma unroll
  for (int b = 0; b < 3; ++b) X[(size_t)(3 * i + b) * 8 + c] += mi[3 * b] * z[0] + mi[3 * b + 1] * z[1] + mi[3 * b + 2] * z[2];
}

// x (column-major n x k, unknown a ne + i) from X[3i+a][c]
__global__ void k_gm_out(int ne, int k, const double* __restrict__ X, double* __restrict__ x) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)3 * ne * 8) return;
  const int c = (int)(t & 7);
  if (c >= k) return;
  const long long u = t >> 3;
  const int i = (int)(u / 3), a = (int)(u % 3);
  x[(size_t)c * 3 * ne + (size_t)a * ne + i] = X[t];
}

}  // namespace

bool DenseLsqr::gmres(const double* b_dev, double* x_dev, const double* q_dev, double tol, int maxit, int restart,
                      int* nit_host, int* status_host, double* relres_host, int* cycles_host) {
  if (!packed || !A || !Vp || !fp32) {
    err = "GMRES needs the packed single layer (mixed Stokes path with velocity known on every wall)";
    return false;
  }
  if (maxit <= 0) maxit = 1000;  // the LIS default of the reference's options
  if (restart <= 0) restart = 40;
  if (restart > 512) { err = "GMRES restart length must be 1..512"; return false; }
  if (!block_precon()) return false;
  const int mr = restart, np = mr + 1;
  const size_t mv = (size_t)m * K8;
  // basis [mr+1][m][8] (v_mr is never formed: mr vectors), w, X, r [k][m]; H, cs,
  // sn, g, y, hc; partials [GM_BLOCKS][mr+1][8]
  const size_t need = (size_t)mr * mv + 2 * mv + (size_t)k * m + (size_t)(mr + 1) * mr * 8 + 5 * (size_t)(mr + 1) * 8;
  if (need > gm_cap || mr != gm_mr) {
    if (gm) cudaFree(gm);
    if (gm_part) cudaFree(gm_part);
    gm = nullptr;
    gm_part = nullptr;
    gm_cap = 0;
    GCK(cudaMalloc(&gm, need * sizeof(double)));
    GCK(cudaMalloc(&gm_part, (size_t)GM_BLOCKS * np * 8 * sizeof(double)));
    gm_cap = need;
    gm_mr = mr;
  }
  if (!gsc) GCK(cudaMalloc(&gsc, K8 * sizeof(GmresScalars)));
  if (!sc0) {
    GCK(cudaMalloc(&sc0, K8 * sizeof(LsqrScalars)));
    GCK(cudaMemsetAsync(sc0, 0, K8 * sizeof(LsqrScalars), stream));  // gamma = 0: the sweep writes A W
  }
  double* Vb = gm;
  double* w = Vb + (size_t)mr * mv;
  double* X = w + mv;
  double* r = X + mv;
  double* H = r + (size_t)k * m;
  double* cs = H + (size_t)(mr + 1) * mr * 8;
  double* sn = cs + (size_t)(mr + 1) * 8;
  double* g = sn + (size_t)(mr + 1) * 8;
  double* y = g + (size_t)(mr + 1) * 8;
  double* hc = y + (size_t)(mr + 1) * 8;
  GCK(cudaMemsetAsync(X, 0, mv * sizeof(double), stream));
  GCK(cudaMemsetAsync(H, 0, (size_t)(mr + 1) * mr * 8 * sizeof(double), stream));
  GCK(cudaMemsetAsync(errflag, 0, sizeof(int), stream));
  const unsigned nb_el = gdiv((long long)pk_ne * 8, GM_THREADS);
  k_gm_load<<<GM_BLOCKS, GM_THREADS, 0, stream>>>(m, k, b_dev, w, gm_part, np);
  k_gm_begin<<<1, 32, 0, stream>>>(gm_part, np, k, tol, maxit, 1, gsc, g, nactive);
  launches += 2;
  if (!pev_ready) {
    for (int i = 0; i < 4 * 32; ++i) GCK(cudaEventCreate(&pev[i]));
    pev_ready = true;
  }
  // one cycle: mr Arnoldi steps
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  GCK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  for (int j = 0; j < mr; ++j) {
    k_gm_pc<<<nb_el, GM_THREADS, 0, stream>>>(pk_ne, pk_ldp, j, w, Vb + (size_t)j * mv, pc9, gsc, Vp, nactive);
    if (j == 0) cudaEventRecordWithFlags(pev[0], stream, cudaEventRecordExternal);
    launch_avp(*this, sc0, w, nactive);  // w = A M^-1 v_j
    if (j == 0) cudaEventRecordWithFlags(pev[1], stream, cudaEventRecordExternal);
    for (int pass = 0; pass < 2; ++pass) {
      k_gm_dots<<<GM_BLOCKS, GM_THREADS, 0, stream>>>(m, j, Vb, mv, w, gm_part, np, nactive);
      k_gm_hred<<<j + 1, 256, 0, stream>>>(j, mr, gm_part, np, pass, hc, H, nactive);
      k_gm_orth<<<GM_BLOCKS, GM_THREADS, 0, stream>>>(m, j, Vb, mv, hc, gsc, w, gm_part, np, nactive);
    }
    k_gm_givens<<<1, 32, 0, stream>>>(j, mr, gm_part, np, tol * kGmresInner, maxit, H, cs, sn, g, gsc, nactive);
  }
  GCK(cudaStreamEndCapture(stream, &graph));
  if (cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) {
    cudaGraphDestroy(graph);
    err = "GMRES: graph instantiation failed";
    return false;
  }
  bool ok = true;
  const int max_cycles = maxit + 2;
  for (int cyc = 0; cyc < max_cycles; ++cyc) {
    if (cudaMemcpyAsync(h_nactive, nactive, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess) {
      ok = false;
      break;
    }
    if (*h_nactive == 0) break;
    if (cudaGraphLaunch(gexec, stream) != cudaSuccess) { ok = false; break; }
    launches += 10L * mr;
    // iterate update and the true residual of every column
    k_gm_solve<<<1, 32, 0, stream>>>(mr, H, g, gsc, y);
    k_gm_xupd<<<nb_el, GM_THREADS, 0, stream>>>(pk_ne, Vb, mv, y, pc9, gsc, X);
    k_gm_out<<<gdiv((long long)m * 8, 256), 256, 0, stream>>>(pk_ne, k, X, x_dev);
    launches += 3;
    if (!residual(b_dev, x_dev, q_dev, r)) { ok = false; break; }
    launches += 3;
    k_gm_load<<<GM_BLOCKS, GM_THREADS, 0, stream>>>(m, k, r, w, gm_part, np);
    k_gm_begin<<<1, 32, 0, stream>>>(gm_part, np, k, tol, maxit, 0, gsc, g, nactive);
    launches += 2;
    float a = 0.f;
    if (cudaEventSynchronize(pev[1]) == cudaSuccess && cudaEventElapsedTime(&a, pev[0], pev[1]) == cudaSuccess) {
      t_av += a;
      ++n_av;
    }
    (void)cudaGetLastError();  // a timing query must not leak into the error checks
  }
  cudaGraphExecDestroy(gexec);
  cudaGraphDestroy(graph);
  if (!ok) {
    if (err.empty()) err = std::string("GMRES cycles: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  GmresScalars hs[K8];
  int hflag = 0;
  GCK(cudaMemcpyAsync(hs, gsc, K8 * sizeof(GmresScalars), cudaMemcpyDeviceToHost, stream));
  GCK(cudaMemcpyAsync(&hflag, errflag, sizeof(int), cudaMemcpyDeviceToHost, stream));
  GCK(cudaStreamSynchronize(stream));
  if (hflag) {
    err = "a bounded barrier wait in the A*V sweep gave up";
    return false;
  }
  for (int c = 0; c < k; ++c) {
    if (nit_host) nit_host[c] = hs[c].its;
    if (status_host) status_host[c] = hs[c].status < 0 ? 1 : hs[c].status;
    if (relres_host) relres_host[c] = hs[c].relres;
    if (cycles_host) cycles_host[c] = hs[c].cycles;
  }
  return true;
}

}  // namespace agb
