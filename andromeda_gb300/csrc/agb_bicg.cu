// BiCGSTAB with the Jacobi preconditioner on the packed Stokes single layer: the
// solver of the reference's LIS path (SLET LIS; StokesBigSystemSOLVElis,
// src/lib_StokesLis.f90:4-56, with the default LIS options "-i bicgstab -p jacobi
// -tol 1.0e-8 -maxiter 1000", src/mod_par.f90:288).  LIS is not part of the
// reference sources; the recurrence is the published preconditioned BiCGSTAB
// (van der Vorst 1992, in the form of Barrett et al., "Templates for the Solution
// of Linear Systems", SIAM 1994, Fig. 2.10) with a zero initial guess and the stop
// ||b - A x||_2 <= tol ||b||_2, as LIS runs it by default.
//
// The LIS system puts the equation of every unknown in the unknown's own row
// (DivideRows, src/lib_StokesLis.f90:66-161); in the packed layout row 3i+a is
// the equation of element i, component a, and its unknown is column a ne + i,
// so the Jacobi diagonal is d[3i+a] = Ap[pk_idx(i, sym(a,a), i)].  Every vector
// is held in the row numbering u = 3i+a, [u][8] for up to 8 right-hand sides.
// The preconditioner is a column scaling: the sweep operand is
// W[a][c][i] = fp32(p[3i+a][c] / d[3i+a]), so k_avp computes A D^-1 p from the
// FP32 blocks; vectors, inner products and scalars are FP64, reduced in a fixed
// order (bitwise reproducible).  Each iteration: two k_avp sweeps and six
// vector kernels of a few MB, replayed eight at a time from a CUDA graph.  Both
// sweeps of the first iteration of every replay are timed with CUDA events into
// the A*V counters (agb_kernel_times).
#include "agb_lsqr.cuh"
#include "agb_sweeps.cuh"
#include <algorithm>

namespace agb {

#define BCK(x)                                                                   \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      return false;                                                              \
    }                                                                            \
  } while (0)

namespace {

constexpr int BG_THREADS = 256;   // 32 rows x 8 right-hand sides per pass of a CTA
constexpr int BG_BLOCKS = 304;    // 2 CTAs per SM on 152 SMs; fixed, so the partial sums reduce in a fixed order
constexpr int BG_NP = 3;          // partial sums per CTA and right-hand side

__host__ __device__ inline unsigned cdivu(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// sums v over the threads of the CTA that share threadIdx.x & 7 (one right-hand side)
// and writes the CTA's sum of right-hand side c to out[c]
__device__ __forceinline__ void cta_sum8(double v, double* sred, double* out) {
  v += __shfl_down_sync(0xffffffffu, v, 16);
  v += __shfl_down_sync(0xffffffffu, v, 8);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < 8) sred[warp * 8 + lane] = v;
  __syncthreads();
  if (threadIdx.x < 8) {
    double t = 0.0;
    for (int w = 0; w < BG_THREADS / 32; ++w) t += sred[w * 8 + threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// sum of partial p of right-hand side c over the BG_BLOCKS CTAs, in CTA order
__device__ __forceinline__ double part_total(const double* part, int p, int c) {
  double t = 0.0;
  for (int b = 0; b < BG_BLOCKS; ++b) t += part[((size_t)b * BG_NP + p) * 8 + c];
  return t;
}

__global__ void k_bg_diag(const float* __restrict__ Ap, int ne, int ldp, double* __restrict__ dinv,
                          int* __restrict__ bad) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= 3 * ne) return;
  const int i = u / 3, a = u % 3;
  const double d = (double)Ap[pk_idx(i, sym6(a, a), i, ldp)];
  if (d == 0.0 || !isfinite(d)) {
    atomicExch(bad, 1);
    dinv[u] = 0.0;
  } else {
    dinv[u] = 1.0 / d;
  }
}

// R = Rt = b (b column-major m x k), X = P = V = 0; partial 0: ||b||^2
__global__ void __launch_bounds__(BG_THREADS) k_bg_init(int m, int k, const double* __restrict__ b,
                                                       double* __restrict__ R, double* __restrict__ Rt,
                                                       double* __restrict__ P, double* __restrict__ V,
                                                       double* __restrict__ X, double* __restrict__ part) {
  __shared__ double sred[BG_THREADS / 32 * 8];
  const int c = threadIdx.x & 7;
  double ss = 0.0;
  for (long long t = (long long)blockIdx.x * BG_THREADS + threadIdx.x; t < (long long)m * 8;
       t += (long long)BG_BLOCKS * BG_THREADS) {
    const long long u = t >> 3;
    const double r = (c < k) ? b[(size_t)c * m + u] : 0.0;
    R[t] = r;
    Rt[t] = r;
    P[t] = 0.0;
    V[t] = 0.0;
    X[t] = 0.0;
    ss += r * r;
  }
  cta_sum8(ss, sred, part + (size_t)blockIdx.x * BG_NP * 8);
}

__global__ void k_bg_start(const double* __restrict__ part, int k, BicgScalars* __restrict__ s,
                           int* __restrict__ nactive) {
  if (threadIdx.x != 0) return;
  int na = 0;
  for (int c = 0; c < 8; ++c) {
    BicgScalars& q = s[c];
    bicg_start(q, part_total(part, 0, c), c < k);
    na += q.active;
  }
  *nactive = na;
}

// p = r (first iteration) or r + beta (p - omega v); W = fp32(p / d) in the
// sweep layout W[a][c][i] (zero for a finished right-hand side)
__global__ void __launch_bounds__(BG_THREADS) k_bg_p(int m, int ldp, const double* __restrict__ R,
                                                    double* __restrict__ P, const double* __restrict__ V,
                                                    const double* __restrict__ dinv,
                                                    const BicgScalars* __restrict__ s, float* __restrict__ W) {
  const int c = threadIdx.x & 7;
  const BicgScalars q = s[c];
  const double beta = (q.its > 0) ? (q.rho / q.rho_old) * (q.alpha / q.omega) : 0.0;
  for (long long t = (long long)blockIdx.x * BG_THREADS + threadIdx.x; t < (long long)m * 8;
       t += (long long)BG_BLOCKS * BG_THREADS) {
    const long long u = t >> 3;
    const int i = (int)(u / 3), a = (int)(u % 3);
    float w = 0.f;
    if (q.active) {
      const double p = (q.its > 0) ? R[t] + beta * (P[t] - q.omega * V[t]) : R[t];
      P[t] = p;
      w = (float)(p * dinv[u]);
    }
    W[((size_t)a * 8 + c) * ldp + i] = w;
  }
}

// partial 0: sum x1 . x2 (and partial 1: sum x3 . x4 when x3 != nullptr)
__global__ void __launch_bounds__(BG_THREADS) k_bg_dots(int m, const double* __restrict__ x1,
                                                       const double* __restrict__ x2, const double* __restrict__ x3,
                                                       const double* __restrict__ x4, double* __restrict__ part) {
  __shared__ double sred[BG_THREADS / 32 * 8];
  double d0 = 0.0, d1 = 0.0;
  for (long long t = (long long)blockIdx.x * BG_THREADS + threadIdx.x; t < (long long)m * 8;
       t += (long long)BG_BLOCKS * BG_THREADS) {
    d0 += x1[t] * x2[t];
    if (x3) d1 += x3[t] * x4[t];
  }
  cta_sum8(d0, sred, part + (size_t)blockIdx.x * BG_NP * 8);
  if (x3) cta_sum8(d1, sred, part + ((size_t)blockIdx.x * BG_NP + 1) * 8);
}

// alpha = rho / (r~ . v)
__global__ void k_bg_alpha(const double* __restrict__ part, BicgScalars* __restrict__ s) {
  const int c = threadIdx.x;
  if (c >= 8) return;
  BicgScalars& q = s[c];
  if (!q.active) return;
  const double rtv = part_total(part, 0, c);
  if (rtv == 0.0 || !isfinite(rtv)) {
    q.status = 2;
    q.active = 0;
    q.alpha = 0.0;
    return;
  }
  q.alpha = q.rho / rtv;
}

// s = r - alpha v; W = fp32(s / d); partial 0: ||s||^2
__global__ void __launch_bounds__(BG_THREADS) k_bg_s(int m, int ldp, const double* __restrict__ R,
                                                    const double* __restrict__ V, const double* __restrict__ dinv,
                                                    const BicgScalars* __restrict__ s, double* __restrict__ S,
                                                    float* __restrict__ W, double* __restrict__ part) {
  __shared__ double sred[BG_THREADS / 32 * 8];
  const int c = threadIdx.x & 7;
  const BicgScalars q = s[c];
  double ss = 0.0;
  for (long long t = (long long)blockIdx.x * BG_THREADS + threadIdx.x; t < (long long)m * 8;
       t += (long long)BG_BLOCKS * BG_THREADS) {
    const long long u = t >> 3;
    const int i = (int)(u / 3), a = (int)(u % 3);
    float w = 0.f;
    if (q.active) {
      const double sv = R[t] - q.alpha * V[t];
      S[t] = sv;
      ss += sv * sv;
      w = (float)(sv * dinv[u]);
    }
    W[((size_t)a * 8 + c) * ldp + i] = w;
  }
  cta_sum8(ss, sred, part + (size_t)blockIdx.x * BG_NP * 8);
}

// ||s|| <= tol ||b||: the right-hand side ends after x += alpha p^ (half step)
__global__ void k_bg_scheck(const double* __restrict__ part, double tol, BicgScalars* __restrict__ s) {
  const int c = threadIdx.x;
  if (c >= 8) return;
  BicgScalars& q = s[c];
  if (!q.active) return;
  q.snorm = sqrt(part_total(part, 0, c)) / q.bnorm;
  q.half = (q.snorm <= tol) ? 1 : 0;
}

// omega = (t . s) / (t . t)
__global__ void k_bg_omega(const double* __restrict__ part, BicgScalars* __restrict__ s) {
  const int c = threadIdx.x;
  if (c >= 8) return;
  BicgScalars& q = s[c];
  if (!q.active || q.half) return;
  const double ts = part_total(part, 0, c), tt = part_total(part, 1, c);
  if (tt == 0.0 || !isfinite(tt)) {
    q.status = 2;
    q.active = 0;
    q.omega = 0.0;
    return;
  }
  q.omega = ts / tt;
}

// x += alpha p/d + omega s/d; r = s - omega t; partial 0: ||r||^2, partial 1: r~ . r
__global__ void __launch_bounds__(BG_THREADS) k_bg_xr(int m, const double* __restrict__ P,
                                                     const double* __restrict__ S, const double* __restrict__ T,
                                                     const double* __restrict__ dinv, const double* __restrict__ Rt,
                                                     const BicgScalars* __restrict__ s, double* __restrict__ X,
                                                     double* __restrict__ R, double* __restrict__ part) {
  __shared__ double sred[BG_THREADS / 32 * 8];
  const int c = threadIdx.x & 7;
  const BicgScalars q = s[c];
  double rr = 0.0, rtr = 0.0;
  for (long long t = (long long)blockIdx.x * BG_THREADS + threadIdx.x; t < (long long)m * 8;
       t += (long long)BG_BLOCKS * BG_THREADS) {
    if (!q.active) continue;
    const double di = dinv[t >> 3];
    if (q.half) {
      X[t] += q.alpha * (P[t] * di);
    } else {
      X[t] += q.alpha * (P[t] * di) + q.omega * (S[t] * di);
      const double r = S[t] - q.omega * T[t];
      R[t] = r;
      rr += r * r;
      rtr += Rt[t] * r;
    }
  }
  cta_sum8(rr, sred, part + (size_t)blockIdx.x * BG_NP * 8);
  cta_sum8(rtr, sred, part + ((size_t)blockIdx.x * BG_NP + 1) * 8);
}

// end of an iteration: stopping tests, rho for the next one, the count of active right-hand sides
__global__ void k_bg_end(const double* __restrict__ part, double tol, int maxit, BicgScalars* __restrict__ s,
                         int* __restrict__ nactive) {
  if (threadIdx.x != 0) return;
  int na = 0;
  for (int c = 0; c < 8; ++c) {
    BicgScalars& q = s[c];
    if (q.active) bicg_end(q, part_total(part, 0, c), part_total(part, 1, c), tol, maxit);
    na += q.active;
  }
  *nactive = na;
}

// x (column-major n x k, unknown a ne + i) from X[3i+a][c]
__global__ void k_bg_out(int ne, int k, const double* __restrict__ X, double* __restrict__ x) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)3 * ne * 8) return;
  const int c = (int)(t & 7);
  if (c >= k) return;
  const long long u = t >> 3;
  const int i = (int)(u / 3), a = (int)(u % 3);
  x[(size_t)c * 3 * ne + (size_t)a * ne + i] = X[t];
}

}  // namespace

bool DenseLsqr::bicgstab(const double* b_dev, double* x_dev, double tol, int maxit, int* nit_host,
                         int* status_host, double* relres_host) {
  if (!packed || !A || !Vp) {
    err = "BiCGSTAB needs the packed single layer (mixed Stokes path with velocity known on every wall)";
    return false;
  }
  if (maxit <= 0) maxit = 1000;  // the LIS default of the reference's options
  const int64_t mv = (int64_t)m * K8;
  if (!bg) {
    BCK(cudaMalloc(&bg, (size_t)(6 * mv + m) * sizeof(double)));
    BCK(cudaMalloc(&bg_part, (size_t)BG_BLOCKS * BG_NP * K8 * sizeof(double)));
    BCK(cudaMalloc(&bsc, K8 * sizeof(BicgScalars)));
    BCK(cudaMalloc(&sc0, K8 * sizeof(LsqrScalars)));
    BCK(cudaMemsetAsync(sc0, 0, K8 * sizeof(LsqrScalars), stream));  // gamma = 0: Y = A W
    bg_diag = false;
  }
  double *R = bg, *Rt = bg + mv, *P = bg + 2 * mv, *S = bg + 3 * mv, *T = bg + 4 * mv, *X = bg + 5 * mv;
  double* dinv = bg + 6 * mv;
  double* V = Y;  // the first sweep writes the solver's Y
  if (!bg_diag) {
    BCK(cudaMemsetAsync(nactive, 0, sizeof(int), stream));
    k_bg_diag<<<cdivu(m, 256), 256, 0, stream>>>((const float*)A, pk_ne, pk_ldp, dinv, nactive);
    BCK(cudaGetLastError());
    int bad = 0;
    BCK(cudaMemcpyAsync(&bad, nactive, sizeof(int), cudaMemcpyDeviceToHost, stream));
    BCK(cudaStreamSynchronize(stream));
    ++launches;
    if (bad) {
      err = "BiCGSTAB: a zero or non-finite diagonal entry (the Jacobi preconditioner needs every diagonal)";
      return false;
    }
    bg_diag = true;
  }
  // T is a sweep output with gamma = 0: A W + 0 * T must not see NaN from old memory
  BCK(cudaMemsetAsync(T, 0, (size_t)mv * sizeof(double), stream));
  BCK(cudaMemsetAsync(errflag, 0, sizeof(int), stream));
  k_bg_init<<<BG_BLOCKS, BG_THREADS, 0, stream>>>(m, k, b_dev, R, Rt, P, V, X, bg_part);
  k_bg_start<<<1, 32, 0, stream>>>(bg_part, k, bsc, nactive);
  launches += 2;
  if (!pev_ready) {
    for (int i = 0; i < 4 * 32; ++i) BCK(cudaEventCreate(&pev[i]));
    pev_ready = true;
  }
  // eight iterations captured in one CUDA graph and replayed until no right-hand
  // side is active; both sweeps of the first iteration of each replay are timed
  // (events on the solver stream); sweeps after the last convergence read nothing
  constexpr int CE = 8;
  auto iteration = [&](bool timed) {
    k_bg_p<<<BG_BLOCKS, BG_THREADS, 0, stream>>>(m, pk_ldp, R, P, V, dinv, bsc, Vp);
    if (timed) cudaEventRecordWithFlags(pev[0], stream, cudaEventRecordExternal);
    launch_avp(*this, sc0, V, nactive);                                 // v = A D^-1 p
    if (timed) cudaEventRecordWithFlags(pev[1], stream, cudaEventRecordExternal);
    k_bg_dots<<<BG_BLOCKS, BG_THREADS, 0, stream>>>(m, Rt, V, nullptr, nullptr, bg_part);
    k_bg_alpha<<<1, 32, 0, stream>>>(bg_part, bsc);
    k_bg_s<<<BG_BLOCKS, BG_THREADS, 0, stream>>>(m, pk_ldp, R, V, dinv, bsc, S, Vp, bg_part);
    k_bg_scheck<<<1, 32, 0, stream>>>(bg_part, tol, bsc);
    if (timed) cudaEventRecordWithFlags(pev[2], stream, cudaEventRecordExternal);
    launch_avp(*this, sc0, T, nactive);                                 // t = A D^-1 s
    if (timed) cudaEventRecordWithFlags(pev[3], stream, cudaEventRecordExternal);
    k_bg_dots<<<BG_BLOCKS, BG_THREADS, 0, stream>>>(m, T, S, T, T, bg_part);
    k_bg_omega<<<1, 32, 0, stream>>>(bg_part, bsc);
    k_bg_xr<<<BG_BLOCKS, BG_THREADS, 0, stream>>>(m, P, S, T, dinv, Rt, bsc, X, R, bg_part);
    k_bg_end<<<1, 32, 0, stream>>>(bg_part, tol, maxit, bsc, nactive);
  };
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  BCK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  for (int j = 0; j < CE; ++j) iteration(j == 0);
  BCK(cudaStreamEndCapture(stream, &graph));
  if (cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) {
    cudaGraphDestroy(graph);
    err = "BiCGSTAB: graph instantiation failed";
    return false;
  }
  bool ok = true;
  for (int it = 0; it < maxit + CE; it += CE) {
    if (cudaGraphLaunch(gexec, stream) != cudaSuccess) { ok = false; break; }
    launches += 11L * CE;
    if (cudaMemcpyAsync(h_nactive, nactive, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess) {
      ok = false;
      break;
    }
    float a = 0.f, b = 0.f;
    if (cudaEventElapsedTime(&a, pev[0], pev[1]) == cudaSuccess) { t_av += a; ++n_av; }
    if (cudaEventElapsedTime(&b, pev[2], pev[3]) == cudaSuccess) { t_av += b; ++n_av; }
    (void)cudaGetLastError();  // a timing query must not leak into the error checks
    if (*h_nactive == 0) break;
  }
  cudaGraphExecDestroy(gexec);
  cudaGraphDestroy(graph);
  if (!ok) {
    err = std::string("BiCGSTAB iterations: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  k_bg_out<<<cdivu((long long)m * 8, 256), 256, 0, stream>>>(pk_ne, k, X, x_dev);
  ++launches;
  BicgScalars hs[K8];
  int hflag = 0;
  BCK(cudaMemcpyAsync(hs, bsc, K8 * sizeof(BicgScalars), cudaMemcpyDeviceToHost, stream));
  BCK(cudaMemcpyAsync(&hflag, errflag, sizeof(int), cudaMemcpyDeviceToHost, stream));
  BCK(cudaStreamSynchronize(stream));
  if (hflag) {
    err = "a bounded barrier wait in the A*V sweep gave up";
    return false;
  }
  for (int c = 0; c < k; ++c) {
    if (nit_host) nit_host[c] = hs[c].its;
    if (status_host) status_host[c] = hs[c].status < 0 ? 1 : hs[c].status;
    if (relres_host) relres_host[c] = hs[c].relres;
  }
  return true;
}

}  // namespace agb
