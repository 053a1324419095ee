// Block LSQR on the GPU: dense sweeps over an HBM-resident matrix shared by up
// to 8 right-hand sides, plus the CRS solver behind the lsqr_solve drop-in.
//
// The recurrence is Paige & Saunders' LSQR exactly as the reference runs it
// (src/lib_lsqr.f:470-1231, damp = 0, no standard errors), with the reference's
// column scaling (lsqr_precon, :131-167) and warm start (lsqr_solve, :33-127).
// Each right-hand side keeps its own scalars and stopping test; the matrix
// products of all of them are computed in one pass over A per sweep:
//   sweep 1  Y = A V + gamma Y        (one warp per 4 rows, V staged in smem)
//   sweep 2  Z = A^T Y                (one thread per 4 columns, row groups
//                                      reduced in a fixed order -> bitwise
//                                      reproducible)
// Vector norms are reduced from per-CTA partials in index order in FP64.
#include "agb_lsqr.cuh"
#include "agb_async.cuh"
#include "agb_sweeps.cuh"
#include "agb_batch.cuh"
#include "agb_mfree.cuh"
#include <cudaTypedefs.h>
#include <cstdio>
#include <cstring>
#include <algorithm>

namespace agb {

#define CK(x)                                                                    \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      return false;                                                              \
    }                                                                            \
  } while (0)

constexpr int kThreads = 256;

template <typename T> struct Vec;
template <> struct Vec<float> { using V = float4; static constexpr int N = 4; };
template <> struct Vec<double> { using V = double2; static constexpr int N = 2; };

template <typename T>
__device__ __forceinline__ void unpack(const typename Vec<T>::V& v, T* o);
template <>
__device__ __forceinline__ void unpack<float>(const float4& v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
template <>
__device__ __forceinline__ void unpack<double>(const double2& v, double* o) { o[0] = v.x; o[1] = v.y; }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Sweep 1: Y[r][c] = s1 * (A Vin)[r][c] + g_c * Yold[r][c]
//   AccT: accumulation type inside a 1024-column chunk (T), chunk sums added
//   in FP64.  VT: type of the staged V (T, or double for the FP64-accumulated
//   refinement residual).  Writes Y (FP64), Ys (T copy) and per-CTA partial
//   sums of Y^2 (part[blockIdx.x][c]).
// ---------------------------------------------------------------------------
constexpr int AV_RR = 4;                 // rows per warp
constexpr int AV_ROWS = AV_RR * (kThreads / 32);

template <typename T, typename VT>
__global__ void __launch_bounds__(kThreads) k_av(const T* __restrict__ A, int64_t lda, int m, int ncols,
                                                  const VT* __restrict__ Vin, double s1, const LsqrScalars* sc,
                                                  int use_gamma, const double* __restrict__ Yold, double* __restrict__ Y,
                                                  T* __restrict__ Ys, double* __restrict__ part) {
  using AccT = typename std::conditional<std::is_same<VT, double>::value, double, T>::type;
  constexpr int VN = Vec<T>::N;
  constexpr int CH = 4096 / sizeof(VT);  // columns per smem chunk (32 KB of V)
  __shared__ __align__(16) VT sV[CH * K8];
  __shared__ double sPart[kThreads / 32][K8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * AV_ROWS + warp * AV_RR;
  double acc[AV_RR][K8];
#pragma unroll
  for (int r = 0; r < AV_RR; ++r)
#pragma unroll
    for (int c = 0; c < K8; ++c) acc[r][c] = 0.0;

  for (int64_t j0 = 0; j0 < lda; j0 += CH) {
    const int cw = (int)((lda - j0) < (int64_t)CH ? (lda - j0) : (int64_t)CH);
    __syncthreads();
    for (int t = threadIdx.x; t < cw * K8; t += kThreads) sV[t] = Vin[j0 * K8 + t];
    __syncthreads();
    AccT part_acc[AV_RR][K8];
#pragma unroll
    for (int r = 0; r < AV_RR; ++r)
#pragma unroll
      for (int c = 0; c < K8; ++c) part_acc[r][c] = AccT(0);
    for (int jj = lane * VN; jj < cw; jj += 32 * VN) {
      T a[AV_RR][VN];
#pragma unroll
      for (int r = 0; r < AV_RR; ++r) {
        const int row = row0 + r;
        if (row < m) {
          typename Vec<T>::V v = *reinterpret_cast<const typename Vec<T>::V*>(A + (int64_t)row * lda + j0 + jj);
          unpack<T>(v, a[r]);
        } else {
#pragma unroll
          for (int q = 0; q < VN; ++q) a[r][q] = T(0);
        }
      }
#pragma unroll
      for (int q = 0; q < VN; ++q) {
        VT vv[K8];
#pragma unroll
        for (int c = 0; c < K8; ++c) vv[c] = sV[(jj + q) * K8 + c];
#pragma unroll
        for (int r = 0; r < AV_RR; ++r)
#pragma unroll
          for (int c = 0; c < K8; ++c) part_acc[r][c] += (AccT)a[r][q] * (AccT)vv[c];
      }
    }
#pragma unroll
    for (int r = 0; r < AV_RR; ++r)
#pragma unroll
      for (int c = 0; c < K8; ++c) acc[r][c] += (double)part_acc[r][c];
  }
  // lane c finalises column c of each row (no lane reads what another writes)
  double ssq = 0.0;
#pragma unroll
  for (int r = 0; r < AV_RR; ++r) {
    const int row = row0 + r;
#pragma unroll
    for (int c = 0; c < K8; ++c) {
      double s = warp_sum(acc[r][c]);
      if (row < m && lane == c) {
        double g = use_gamma ? sc[c].gamma : 1.0;
        double y = s1 * s + (Yold ? g * Yold[(int64_t)row * K8 + c] : 0.0);
        Y[(int64_t)row * K8 + c] = y;
        Ys[(int64_t)row * K8 + c] = (T)y;
        ssq += y * y;
      }
    }
  }
  if (lane < K8) sPart[warp][lane] = ssq;
  __syncthreads();
  if (threadIdx.x < K8) {
    double s = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) s += sPart[w][threadIdx.x];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = s;
  }
}

// ---------------------------------------------------------------------------
// Sweep 2: Zp[g][j][c] = sum_{r in group g} A[r][j] Us[r][c]
// Each thread owns VN consecutive columns; rows of the group are streamed with
// U staged in smem 256 rows at a time (T accumulation per chunk, FP64 across
// chunks).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads) k_atu(const T* __restrict__ A, int64_t lda, int m, const T* __restrict__ Us,
                                                   int rows_per_group, double* __restrict__ Zp) {
  constexpr int VN = Vec<T>::N;
  constexpr int RCH = 256;
  __shared__ __align__(16) T sU[RCH * K8];
  const int64_t col = ((int64_t)blockIdx.x * kThreads + threadIdx.x) * VN;
  const int g = blockIdx.y;
  const int r0 = g * rows_per_group, r1 = min(m, r0 + rows_per_group);
  double acc[VN][K8];
#pragma unroll
  for (int q = 0; q < VN; ++q)
#pragma unroll
    for (int c = 0; c < K8; ++c) acc[q][c] = 0.0;
  for (int rb = r0; rb < r1; rb += RCH) {
    const int nr = min(RCH, r1 - rb);
    __syncthreads();
    for (int t = threadIdx.x; t < nr * K8; t += kThreads) sU[t] = Us[(int64_t)rb * K8 + t];
    __syncthreads();
    if (col < lda) {
      T pa[VN][K8];
#pragma unroll
      for (int q = 0; q < VN; ++q)
#pragma unroll
        for (int c = 0; c < K8; ++c) pa[q][c] = T(0);
      const T* ap = A + (int64_t)rb * lda + col;
#pragma unroll 4
      for (int r = 0; r < nr; ++r) {
        typename Vec<T>::V v = *reinterpret_cast<const typename Vec<T>::V*>(ap + (int64_t)r * lda);
        T a[VN];
        unpack<T>(v, a);
        const T* u = sU + r * K8;
#pragma unroll
        for (int q = 0; q < VN; ++q)
#pragma unroll
          for (int c = 0; c < K8; ++c) pa[q][c] += a[q] * u[c];
      }
#pragma unroll
      for (int q = 0; q < VN; ++q)
#pragma unroll
        for (int c = 0; c < K8; ++c) acc[q][c] += (double)pa[q][c];
    }
  }
  if (col < lda) {
#pragma unroll
    for (int q = 0; q < VN; ++q)
#pragma unroll
      for (int c = 0; c < K8; ++c) Zp[((int64_t)g * lda + col + q) * K8 + c] = acc[q][c];
  }
}

// ---------------------------------------------------------------------------
// Tuned sweeps of the LSQR iteration.
//
// k_av2: Y = A V + gamma Y.  A warp owns RR rows; lanes stream 16-byte
// vectors of each row (coalesced 512 B per warp and row).  V is kept
// RHS-major ([8][lda]) and staged chunk by chunk into shared memory by 1-D
// TMA bulk copies (cp.async.bulk + mbarrier, double buffered), so a lane's
// 16-byte reads of V hit 32 consecutive banks.  FP32 path: products are
// accumulated in FP32 within a 1024-column chunk, then reduce-scattered across
// the warp (31 shuffles) so that lane l keeps the FP64 running sum of
// (row l/8, rhs l%8) -- one FP64 register per lane instead of 32.
// ---------------------------------------------------------------------------
template <typename T> struct AV2;
template <> struct AV2<float> { static constexpr int RR = 4, WARPS = 16, CH = 1024; };
template <> struct AV2<double> { static constexpr int RR = 1, WARPS = 8, CH = 512; };  // FP64-pipe bound: 8 rows per CTA
                                                                                         // spread small systems over all SMs

template <typename T>
__global__ void __launch_bounds__(AV2<T>::WARPS * 32) k_av2(const T* __restrict__ A, int64_t lda, int m,
                                                            const T* __restrict__ Vt, const LsqrScalars* sc,
                                                            double* __restrict__ Y, T* __restrict__ Ys,
                                                            double* __restrict__ part, int* errflag) {
  constexpr int RR = AV2<T>::RR, WARPS = AV2<T>::WARPS, CH = AV2<T>::CH, VN = 16 / sizeof(T);
  extern __shared__ __align__(128) unsigned char av2_smem[];
  T* sV = reinterpret_cast<T*>(av2_smem);  // [2][8][CH]
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ double sPart[WARPS][K8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * (WARPS * RR) + warp * RR;
  const int nch = (int)((lda + CH - 1) / CH);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int k) {
    const int64_t j0 = (int64_t)k * CH;
    const int cw = (int)((lda - j0) < (int64_t)CH ? (lda - j0) : (int64_t)CH);
    uint64_t* b = &bar[k & 1];
    T* dst = sV + (size_t)(k & 1) * K8 * CH;
    mbar_expect_tx(b, (uint32_t)(K8 * cw * sizeof(T)));
#pragma unroll
    for (int c = 0; c < K8; ++c) bulk_g2s(dst + c * CH, Vt + (int64_t)c * lda + j0, (uint32_t)(cw * sizeof(T)), b);
  };
  if (threadIdx.x == 0) issue(0);

  using Acc = T;
  Acc acc[RR][K8];
  double dacc = 0.0;                // float path: lane's (row, rhs) running sum
  double dfull[RR][K8];             // double path
#pragma unroll
  for (int r = 0; r < RR; ++r)
#pragma unroll
    for (int c = 0; c < K8; ++c) { acc[r][c] = Acc(0); dfull[r][c] = 0.0; }

  // software pipeline over the A stream: the vectors of step s+1 are in flight
  // while step s is multiplied (rows beyond m read row m-1; those products are
  // discarded)
  typename Vec<T>::V an[RR];
  const T* arow[RR];
#pragma unroll
  for (int r = 0; r < RR; ++r) arow[r] = A + (int64_t)min(row0 + r, m - 1) * lda;
  if (lane * VN < lda) {
#pragma unroll
    for (int r = 0; r < RR; ++r) an[r] = __ldcs(reinterpret_cast<const typename Vec<T>::V*>(arow[r] + lane * VN));
  }
  for (int k = 0; k < nch; ++k) {
    if (threadIdx.x == 0 && k + 1 < nch) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(k + 1);
    }
    mbar_wait_bounded(&bar[k & 1], (uint32_t)((k >> 1) & 1), errflag);
    const T* cv = sV + (size_t)(k & 1) * K8 * CH;
    const int64_t j0 = (int64_t)k * CH;
    const int cw = (int)((lda - j0) < (int64_t)CH ? (lda - j0) : (int64_t)CH);
    for (int jj = lane * VN; jj < cw; jj += 32 * VN) {
      T a[RR][VN];
#pragma unroll
      for (int r = 0; r < RR; ++r) unpack<T>(an[r], a[r]);
      // next step of this lane: further along the chunk, or the first step of
      // the next chunk (A does not depend on V, so it is fetched ahead of the
      // chunk barrier)
      const int64_t jn = (jj + 32 * VN < cw) ? j0 + jj + 32 * VN : j0 + cw + lane * VN;
      if (jn < lda) {
#pragma unroll
        for (int r = 0; r < RR; ++r) an[r] = __ldcs(reinterpret_cast<const typename Vec<T>::V*>(arow[r] + jn));
      }
#pragma unroll
      for (int c = 0; c < K8; ++c) {
        typename Vec<T>::V vv = *reinterpret_cast<const typename Vec<T>::V*>(cv + c * CH + jj);
        T v[VN];
        unpack<T>(vv, v);
#pragma unroll
        for (int r = 0; r < RR; ++r)
#pragma unroll
          for (int q = 0; q < VN; ++q) acc[r][c] += a[r][q] * v[q];
      }
    }
    if constexpr (sizeof(T) == 4) {
      // reduce-scatter the 32 chunk partials: lane l ends with index l = r*8+c
      float v[32];
#pragma unroll
      for (int r = 0; r < RR; ++r)
#pragma unroll
        for (int c = 0; c < K8; ++c) { v[r * K8 + c] = acc[r][c]; acc[r][c] = 0.f; }
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
          const float send = upper ? v[i] : v[i + o];
          const float keep = upper ? v[i + o] : v[i];
          v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
      }
      dacc += (double)v[0];
    } else {
#pragma unroll
      for (int r = 0; r < RR; ++r)
#pragma unroll
        for (int c = 0; c < K8; ++c) { dfull[r][c] += (double)acc[r][c]; acc[r][c] = Acc(0); }
    }
    __syncthreads();  // everyone is done with this buffer before it is refilled
  }
  if (threadIdx.x == 0) mbar_drain(bar, 2, nch, errflag);
  double ssq = 0.0;
  if constexpr (sizeof(T) == 4) {
    const int r = lane >> 3, c = lane & 7, row = row0 + r;
    if (row < m) {
      const double y = dacc + sc[c].gamma * Y[(int64_t)row * K8 + c];
      Y[(int64_t)row * K8 + c] = y;
      Ys[(int64_t)row * K8 + c] = (T)y;
      ssq = y * y;
    }
    // lanes with equal c: l, l^8, l^16, l^24
    ssq += __shfl_xor_sync(0xffffffffu, ssq, 8);
    ssq += __shfl_xor_sync(0xffffffffu, ssq, 16);
  } else {
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      const int row = row0 + r;
#pragma unroll
      for (int c = 0; c < K8; ++c) {
        const double s = warp_sum(dfull[r][c]);
        if (row < m && lane == c) {
          const double y = s + sc[c].gamma * Y[(int64_t)row * K8 + c];
          Y[(int64_t)row * K8 + c] = y;
          Ys[(int64_t)row * K8 + c] = (T)y;
          ssq += y * y;
        }
      }
    }
  }
  if (lane < K8) sPart[warp][lane] = ssq;
  __syncthreads();
  if (threadIdx.x < K8) {
    double a = 0.0;
    for (int w = 0; w < WARPS; ++w) a += sPart[w][threadIdx.x];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = a;
  }
}

// k_atu2: Zp[g][j][c] = sum_{r in group g} A[r][j] U[r][c].  A thread owns VN
// consecutive columns and streams the rows of its group 8 at a time (8
// independent 16-byte loads in flight per thread); U rows are broadcast from
// shared memory.  FP32 path: FP32 partials over 256 rows are added into FP64
// per-thread accumulators kept in shared memory.
constexpr int ATU_THREADS = 256;
template <typename T>
__global__ void __launch_bounds__(ATU_THREADS) k_atu2(const T* __restrict__ A, int64_t lda, int m,
                                                      const T* __restrict__ Us, int rows_per_group,
                                                      double* __restrict__ Zp) {
  constexpr int VN = Vec<T>::N;
  constexpr int RCH = 256;
  constexpr int UNR = 8;
  extern __shared__ __align__(16) unsigned char atu_smem[];
  T* sU = reinterpret_cast<T*>(atu_smem);                                  // [RCH][8]
  double* sD = reinterpret_cast<double*>(atu_smem + RCH * K8 * sizeof(T));  // [VN*8][threads] (FP32 path)
  const int64_t col = ((int64_t)blockIdx.x * ATU_THREADS + threadIdx.x) * VN;
  const int g = blockIdx.y;
  const int r0 = g * rows_per_group, r1 = min(m, r0 + rows_per_group);
  const bool live = col < lda;
  T acc[VN][K8];
#pragma unroll
  for (int q = 0; q < VN; ++q)
#pragma unroll
    for (int c = 0; c < K8; ++c) acc[q][c] = T(0);
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int t = 0; t < VN * K8; ++t) sD[t * ATU_THREADS + threadIdx.x] = 0.0;
  }
  for (int rb = r0; rb < r1; rb += RCH) {
    const int nr = min(RCH, r1 - rb);
    __syncthreads();
    for (int t = threadIdx.x; t < nr * K8; t += ATU_THREADS) sU[t] = Us[(int64_t)rb * K8 + t];
    __syncthreads();
    if (live) {
      const T* ap = A + (int64_t)rb * lda + col;
      int r = 0;
      for (; r + UNR <= nr; r += UNR) {
        typename Vec<T>::V v[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) v[u] = *reinterpret_cast<const typename Vec<T>::V*>(ap + (int64_t)(r + u) * lda);
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
          T a[VN];
          unpack<T>(v[u], a);
          const T* uu = sU + (r + u) * K8;
#pragma unroll
          for (int q = 0; q < VN; ++q)
#pragma unroll
            for (int c = 0; c < K8; ++c) acc[q][c] += a[q] * uu[c];
        }
      }
      for (; r < nr; ++r) {
        typename Vec<T>::V v = *reinterpret_cast<const typename Vec<T>::V*>(ap + (int64_t)r * lda);
        T a[VN];
        unpack<T>(v, a);
        const T* uu = sU + r * K8;
#pragma unroll
        for (int q = 0; q < VN; ++q)
#pragma unroll
          for (int c = 0; c < K8; ++c) acc[q][c] += a[q] * uu[c];
      }
      if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int q = 0; q < VN; ++q)
#pragma unroll
          for (int c = 0; c < K8; ++c) {
            sD[(q * K8 + c) * ATU_THREADS + threadIdx.x] += (double)acc[q][c];
            acc[q][c] = T(0);
          }
      }
    }
  }
  if (live) {
#pragma unroll
    for (int q = 0; q < VN; ++q)
#pragma unroll
      for (int c = 0; c < K8; ++c) {
        double v;
        if constexpr (sizeof(T) == 4) v = sD[(q * K8 + c) * ATU_THREADS + threadIdx.x];
        else v = (double)acc[q][c];
        Zp[((int64_t)g * lda + col + q) * K8 + c] = v;
      }
  }
}

// ---------------------------------------------------------------------------
// TMA-fed FP32 sweeps.  A is streamed through a 3-stage shared-memory ring by
// 2-D tensor-map copies (cp.async.bulk.tensor, one elected thread issues,
// mbarrier full/empty handshakes with bounded waits); the warps compute from
// shared memory, so the bytes in flight per SM (two 64 KB stages) no longer
// depend on registers.
// ---------------------------------------------------------------------------
constexpr int AV3_ROWS = 64, AV3_ST = 3, AV3_WARPS = AV3_ROWS / 4;
constexpr size_t AV3_SMEM = SweepAV<AV3_ROWS, AV3_ST>::SMEM;

__global__ void __launch_bounds__(AV3_WARPS * 32, 1) k_av3(const __grid_constant__ CUtensorMap tmA, int64_t lda, int m,
                                                           const float* __restrict__ Vt, const LsqrScalars* sc,
                                                           double* __restrict__ Y, float* __restrict__ Ys,
                                                           double* __restrict__ part, int* errflag) {
  av3_tile<AV3_ROWS, AV3_ST>(&tmA, lda, m, Vt, sc, Y, Ys, part, errflag, (int)blockIdx.x);
}

constexpr int ATU3_RS = 32, ATU3_ST = 3;
constexpr size_t ATU3_SMEM = SweepATU<ATU3_RS, ATU3_ST>::SMEM;

__global__ void __launch_bounds__(ATU3_THREADS, 1) k_atu3(const __grid_constant__ CUtensorMap tmA, int64_t lda, int m,
                                                          const float* __restrict__ Us, int rows_per_group,
                                                          double* __restrict__ Zp, int* errflag) {
  atu3_tile<ATU3_RS, ATU3_ST>(&tmA, lda, m, Us, rows_per_group, Zp, errflag, (int)blockIdx.x, (int)blockIdx.y);
}

// ---------------------------------------------------------------------------
// Sweeps over the packed single layer (tile bodies avp_tile / atup_tile).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(AVP_THREADS, 1) k_avp(const __grid_constant__ CUtensorMap tmA,
                                                       const __grid_constant__ CUtensorMap tmW, int ne, int ldp,
                                                       const LsqrScalars* sc, double* __restrict__ Y,
                                                       float* __restrict__ Ys, double* __restrict__ part,
                                                       int* errflag) {
  avp_tile(&tmA, &tmW, ne, ldp, sc, Y, Ys, part, errflag, (int)blockIdx.x);
}

__global__ void __launch_bounds__(ATUP_C, 2) k_atup(const __grid_constant__ CUtensorMap tmA, int ne, int ldp,
                                                   int64_t lda, const float* __restrict__ Us, int rows_per_group,
                                                   double* __restrict__ Zp, int* errflag) {
  atup_tile(&tmA, ne, lda, Us, rows_per_group, Zp, errflag, (int)blockIdx.x, (int)blockIdx.y);
}

// r = b - A (q.Xs) over the packed (unscaled) matrix, FP64 accumulation (warm start / refinement residual);
// one warp per row i
__global__ void __launch_bounds__(256) k_residp(const float* __restrict__ Ap, int ne, int ldp,
                                                const double* __restrict__ Xs, const double* __restrict__ qs,
                                                const double* __restrict__ Bp, double* __restrict__ Y,
                                                float* __restrict__ Ys, double* __restrict__ part) {
  __shared__ double sPart[8][K8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  double acc[3][K8];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) acc[a][c] = 0.0;
  if (i < ne) {
    for (int j = lane; j < ne; j += 32) {
      double g6[6];
      const float* pj = Ap + pk_idx(i, 0, j, ldp);
#pragma unroll
      for (int c = 0; c < 6; ++c) g6[c] = (double)pj[c * 64];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const double* x = Xs + ((int64_t)b * ne + j) * K8;
        const double qv = qs ? qs[(int64_t)b * ne + j] : 1.0;  // Xs = x / q and Ap is the unscaled matrix
#pragma unroll
        for (int c = 0; c < K8; ++c) {
          const double xv = qv * x[c];
#pragma unroll
          for (int a = 0; a < 3; ++a) acc[a][c] += g6[sym6(a, b)] * xv;
        }
      }
    }
  }
  double ssq = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) {
      const double v = warp_sum(acc[a][c]);
      if (lane == a * K8 + c && i < ne) {
        const int64_t id = (int64_t)(3 * i + a) * K8 + c;
        const double y = Bp[id] - v;
        Y[id] = y;
        Ys[id] = (float)y;
        ssq = y * y;
      }
    }
  ssq += __shfl_down_sync(0xffffffffu, ssq, 8);
  ssq += __shfl_down_sync(0xffffffffu, ssq, 16);
  if (lane < K8) sPart[warp][lane] = ssq;
  __syncthreads();
  if (threadIdx.x < K8) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += sPart[w][threadIdx.x];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = t;
  }
}

// q.Xs (Xs itself when qs is null) split into FP32 parts, x = xh + xl to about 2^-48 relative ([n][8])
__global__ void k_split_x(int64_t n8, const double* __restrict__ Xs, const double* __restrict__ qs,
                          float* __restrict__ Xh, float* __restrict__ Xl) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n8; t += (int64_t)gridDim.x * blockDim.x) {
    const double x = qs ? qs[t >> 3] * Xs[t] : Xs[t];
    const float h = (float)x;
    Xh[t] = h;
    Xl[t] = (float)(x - (double)h);
  }
}

// r = b - A x over the packed matrix as k_residp computes it, on the FP32 pipe:
// with x = xh + xl, every product g xh is split exactly into p + pe (p the
// rounded product, pe = fma(g, xh, -p)); the p are summed by TwoSum (Knuth;
// s + e holds the running sum exactly up to the rounding of the error term),
// the pe and the g xl terms into a third FP32 sum, and the three sums are
// moved into FP64 accumulators every kFFTerms = 256 terms of a lane (the FP64
// adds run at 1/64 of the FP32 rate: flushing every 64 terms cost ~15 % of the
// kernel).  The rounding left is that of the FP32 sum of the TwoSum errors and
// of the third sum: at most about n^2 u^2 / 2 of sum |a_ij x_j| for n = 256
// terms and u = 2^-24, i.e. 2^-33 in the worst case (random rounding: below
// 2^-44), where FP64 accumulation gives 2^-53: far below any tolerance
// the solvers test, on the FP32 pipe instead of the 1:64 FP64 pipe.  The adds
// and the product use the _rn intrinsics so that nothing is contracted into an
// FMA, which would break the exactness of TwoSum.  One warp per element row i.
template <int KC>
__global__ void __launch_bounds__(256) k_residp_ff(const float* __restrict__ Ap, int ne, int ldp,
                                                   const float* __restrict__ Xh, const float* __restrict__ Xl,
                                                   const double* __restrict__ Bp, double* __restrict__ Y,
                                                   float* __restrict__ Ys, double* __restrict__ part) {
  __shared__ double sPart[8][K8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  float sm[3][KC], er[3][KC], lo[3][KC];
  double acc[3][KC];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < KC; ++c) {
      sm[a][c] = er[a][c] = lo[a][c] = 0.f;
      acc[a][c] = 0.0;
    }
  if (i < ne) {
    for (int j0 = lane; j0 < ne; j0 += 32 * kFFTerms) {
    const int j1 = min(ne, j0 + 32 * kFFTerms);
    for (int j = j0; j < j1; j += 32) {
      float g6[6];
      const float* pj = Ap + pk_idx(i, 0, j, ldp);
#pragma unroll
      for (int c = 0; c < 6; ++c) g6[c] = pj[c * 64];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float* xh = Xh + ((int64_t)b * ne + j) * K8;
        const float* xl = Xl + ((int64_t)b * ne + j) * K8;
        float hv[KC], lv[KC];
#pragma unroll
        for (int c = 0; c < KC; ++c) {
          hv[c] = xh[c];
          lv[c] = xl[c];
        }
#pragma unroll
        for (int c = 0; c < KC; ++c)
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float g = g6[sym6(a, b)];
            const float p = __fmul_rn(g, hv[c]);
            const float pe = fmaf(g, hv[c], -p);
            const float s0 = sm[a][c];
            const float t = __fadd_rn(s0, p);
            const float bp = __fsub_rn(t, s0);
            const float e = __fadd_rn(__fsub_rn(s0, __fsub_rn(t, bp)), __fsub_rn(p, bp));
            sm[a][c] = t;
            er[a][c] = __fadd_rn(er[a][c], e);
            lo[a][c] = fmaf(g, lv[c], __fadd_rn(lo[a][c], pe));
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
  }
  double ssq = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < K8; ++c) {
      double v = 0.0;
      if (c < KC) v = acc[a][c];
      v = warp_sum(v);
      if (lane == a * K8 + c && i < ne) {
        const int64_t id = (int64_t)(3 * i + a) * K8 + c;
        const double y = Bp[id] - v;
        Y[id] = y;
        Ys[id] = (float)y;
        ssq = y * y;
      }
    }
  ssq += __shfl_down_sync(0xffffffffu, ssq, 8);
  ssq += __shfl_down_sync(0xffffffffu, ssq, 16);
  if (lane < K8) sPart[warp][lane] = ssq;
  __syncthreads();
  if (threadIdx.x < K8) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += sPart[w][threadIdx.x];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = t;
  }
}

// column sums of squares of the packed matrix per row group:
// P[g][b ne + j] = sum_{i in g} sum_a Ap[i][sym(a,b)][j]^2
__global__ void k_colsqp(const float* __restrict__ Ap, int ne, int ldp, int rows_per_group, double* __restrict__ P,
                         int64_t lda) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int g = blockIdx.y;
  if (j >= ne) return;
  const int r0 = g * rows_per_group, r1 = min(ne, r0 + rows_per_group);
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int i = r0; i < r1; ++i) {
    const float* pj = Ap + pk_idx(i, 0, j, ldp);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const double v = (double)pj[c * 64];
      s[c] += v * v;
    }
  }
  // b = 0: xx, xy, xz; b = 1: xy, yy, yz; b = 2: xz, yz, zz
  P[(int64_t)g * lda + j] = s[0] + s[1] + s[2];
  P[(int64_t)g * lda + ne + j] = s[1] + s[3] + s[4];
  P[(int64_t)g * lda + 2 * ne + j] = s[2] + s[4] + s[5];
}

// V <- Z/beta - beta V (Z = sum of group partials, in order); partial ||V||^2.
// On the initial call (init=1) the old V is taken as zero.
__global__ void k_atu_reduce(const double* __restrict__ Zp, int groups, int64_t lda, int n, const LsqrScalars* sc,
                             int init, double* __restrict__ V, double* __restrict__ part,
                             const double* __restrict__ qs = nullptr, const double* __restrict__ pc9 = nullptr,
                             int pk_ne = 0) {
  __shared__ double sP[kThreads / 32][K8];
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const int64_t j = t / K8;
  const int c = (int)(t % K8);
  double vn = 0.0;
  if (j < n) {
    double z = 0.0;
    if (pc9) {
      // block-Jacobi right preconditioner: (A M^-1)^T u = M^-T (A^T u) with the
      // element's symmetric 3x3 inverse self block, over its three components
      const int b = (int)(j / pk_ne);
      const int64_t i = j - (int64_t)b * pk_ne;
      const double* mi = pc9 + 9 * i + 3 * b;
      for (int bb = 0; bb < 3; ++bb) {
        double zb = 0.0;
        for (int g = 0; g < groups; ++g) zb += Zp[((int64_t)g * lda + (int64_t)bb * pk_ne + i) * K8 + c];
        z += mi[bb] * zb;
      }
    } else {
      for (int g = 0; g < groups; ++g) z += Zp[((int64_t)g * lda + j) * K8 + c];
      if (qs) z *= qs[j];  // column scaling applied on the fly (packed layout)
    }
    const double beta = sc[c].beta;
    if (sc[c].active && beta > 0.0) {
      vn = z / beta - (init ? 0.0 : beta * V[j * K8 + c]);
      V[j * K8 + c] = vn;
    } else {
      vn = V[j * K8 + c];
      if (!sc[c].active) vn = 0.0;
    }
  }
  // reduce vn^2 per c: lanes with equal c are 8 apart
  double s = vn * vn;
  s += __shfl_xor_sync(0xffffffffu, s, 8);
  s += __shfl_xor_sync(0xffffffffu, s, 16);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < K8) sP[warp][lane] = s;
  __syncthreads();
  if (threadIdx.x < K8) {
    double a = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) a += sP[w][threadIdx.x];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = a;
  }
}

// Vector update of one iteration: V <- V/alpha; X += t1 W; W <- t2 W + V;
// dknorm partial += (t3 W_old)^2; Vs = (T)V.  init=1: W <- V, X <- 0.
template <typename T>
__global__ void k_update(int n, int64_t lda, const LsqrScalars* sc, int init, double* __restrict__ V,
                         double* __restrict__ W, double* __restrict__ X, T* __restrict__ Vs, double* __restrict__ part,
                         int vs_rhs_major, float* __restrict__ Vp = nullptr, int pk_ne = 0, int pk_ldp = 0,
                         const double* __restrict__ qs = nullptr, int vp_later = 0) {
  __shared__ double sP[kThreads / 32][K8];
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const int64_t j = t / K8;
  const int c = (int)(t % K8);
  double dk = 0.0;
  if (j < lda) {
    const int64_t id = j * K8 + c;
    if (j >= n) {
      V[id] = 0.0; W[id] = 0.0; X[id] = 0.0; Vs[vs_rhs_major ? (int64_t)c * lda + j : id] = T(0);
    } else {
      if (sc[c].active) {
        double v = V[id];
        if (sc[c].alpha > 0.0) v = v / sc[c].alpha;
        V[id] = v;
        if (init) {
          W[id] = v;
          X[id] = 0.0;
        } else {
          double w = W[id];
          X[id] = sc[c].t1 * w + X[id];
          W[id] = sc[c].t2 * w + v;
          double q = sc[c].t3 * w;
          dk = q * q;
        }
      } else if (init) {
        W[id] = 0.0; X[id] = 0.0;
      }
      if (vp_later) {
        // the block-preconditioned operand is written by k_pc_vp (it mixes the
        // three components of an element, which other threads update here)
      } else if (Vp) {  // packed layout: W = q.V as [b][k][ldp]
        const int b = (int)(j / pk_ne);
        const int64_t jj = j - (int64_t)b * pk_ne;
        Vp[((int64_t)b * K8 + c) * pk_ldp + jj] = (float)(qs[j] * V[id]);
      } else {
        Vs[vs_rhs_major ? (int64_t)c * lda + j : id] = (T)V[id];
      }
    }
  }
  double s = dk;
  s += __shfl_xor_sync(0xffffffffu, s, 8);
  s += __shfl_xor_sync(0xffffffffu, s, 16);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < K8) sP[warp][lane] = s;
  __syncthreads();
  if (threadIdx.x < K8) {
    double a = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) a += sP[w][threadIdx.x];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = a;
  }
}

__device__ double sum_part(const double* part, int nb, int c) {
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += part[b * K8 + c];
  return s;
}

// Scalar phases (one thread per right-hand side).
// phase 0: beta0 = ||r||; bnorm.       phase 1: alpha0; init recurrences.
// phase 2: beta = ||Y|| after sweep 1; anorm.
// phase 3: alpha after sweep 2; plane rotations; t1,t2,t3; gamma for next sweep.
// phase 4: after the x/w update: dnorm, xnorm, residual estimates, stopping tests.
// The partial sums of the producing kernel are reduced by the whole block in
// a fixed order (thread t sums blocks t/8, t/8+128, ... of column t%8, then a
// shared-memory tree whose strides are multiples of 8 adds the 128 per-thread
// sums of each column): deterministic, and the serial part is O(nb/128)
// independent loads per thread (the kernel sits on the critical path of every
// LSQR iteration).
constexpr int SCAL_THREADS = 1024;
__global__ void __launch_bounds__(SCAL_THREADS) k_scalars(LsqrScalars* sc, int k, int phase, const double* part,
                                                          int nb, int* nactive) {
  __shared__ double sred[SCAL_THREADS];
  {
    const int t = threadIdx.x, cc = t % K8;
    double a = 0.0;
#pragma unroll 4
    for (int b = t / K8; b < nb; b += SCAL_THREADS / K8) a += part[(int64_t)b * K8 + cc];
    sred[t] = a;
    __syncthreads();
#pragma unroll
    for (int st = SCAL_THREADS / 2; st >= K8; st >>= 1) {
      if (t < st) sred[t] += sred[t + st];
      __syncthreads();
    }
  }
  const int c = threadIdx.x;
  if (phase == 3 && c == 0) *nactive = 0;  // the active count of this iteration is rebuilt by phase 4
  if (c >= K8) return;
  lsqr_phase(sc[c], c, k, phase, sred[c], nactive);
}

// ---------------------------------------------------------------------------
// Column scaling (lsqr_precon): partial column sums of squares per row group,
// then q_j = 1/sqrt(sum) and A <- A diag(q).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_colsq(const T* __restrict__ A, int64_t lda, int m, int rows_per_group, double* __restrict__ P) {
  constexpr int VN = Vec<T>::N;
  const int64_t col = ((int64_t)blockIdx.x * kThreads + threadIdx.x) * VN;
  const int g = blockIdx.y;
  const int r0 = g * rows_per_group, r1 = min(m, r0 + rows_per_group);
  if (col >= lda) return;
  double acc[VN];
#pragma unroll
  for (int q = 0; q < VN; ++q) acc[q] = 0.0;
  for (int r = r0; r < r1; ++r) {
    typename Vec<T>::V v = *reinterpret_cast<const typename Vec<T>::V*>(A + (int64_t)r * lda + col);
    T a[VN];
    unpack<T>(v, a);
#pragma unroll
    for (int q = 0; q < VN; ++q) acc[q] += (double)a[q] * (double)a[q];
  }
#pragma unroll
  for (int q = 0; q < VN; ++q) P[(int64_t)g * lda + col + q] = acc[q];
}
__global__ void k_colsq_finish(const double* __restrict__ P, int groups, int64_t lda, int n, double* __restrict__ q) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= lda) return;
  double s = 0.0;
  for (int g = 0; g < groups; ++g) s += P[(int64_t)g * lda + j];
  q[j] = (j < n) ? 1.0 / sqrt(s) : 0.0;
}
template <typename T>
__global__ void k_scale_cols(T* __restrict__ A, int64_t lda, int m, const double* __restrict__ q) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t tot = (int64_t)m * lda;
  for (int64_t i = idx; i < tot; i += (int64_t)gridDim.x * blockDim.x) A[i] = (T)((double)A[i] * q[i % lda]);
}

// Pack column-major (rows x k) into [rows_pad][8] (zero padding); optional
// element-wise divide by d (x/q warm start).
__global__ void k_pack(const double* __restrict__ src, int rows, int k, int64_t rows_pad, const double* __restrict__ d,
                       double* __restrict__ dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows_pad * K8) return;
  const int64_t r = t / K8;
  const int c = (int)(t % K8);
  double v = 0.0;
  if (r < rows && c < k) {
    v = src[(int64_t)c * rows + r];
    if (d) v = v / d[r];
  }
  dst[t] = v;
}
// x_out(:,c) = q .* X(:,c) + x0(:,c), or M^-1 X(:,c) + x0(:,c) with the block-Jacobi preconditioner
__global__ void k_finish_x(const double* __restrict__ X, const double* __restrict__ q, const double* __restrict__ X0,
                           int n, int k, const LsqrScalars* sc, double* __restrict__ xout,
                           const double* __restrict__ pc9 = nullptr, int pk_ne = 0) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * k) return;
  const int c = (int)(t / n);
  const int64_t j = t % n;
  double v;
  if (pc9) {
    const int b = (int)(j / pk_ne);
    const int64_t i = j - (int64_t)b * pk_ne;
    const double* mi = pc9 + 9 * i + 3 * b;
    v = 0.0;
    for (int bb = 0; bb < 3; ++bb) v += mi[bb] * X[((int64_t)bb * pk_ne + i) * K8 + c];
  } else {
    v = q[j] * X[j * K8 + c];
  }
  xout[(int64_t)c * n + j] = v + X0[j * K8 + c];
}
// the sweep-1 operand of the block-preconditioned packed LSQR: W = M^-1 V as
// [b][k][ldp] FP32 (M = the elements' 3x3 self blocks)
__global__ void k_pc_vp(int pk_ne, int pk_ldp, const double* __restrict__ V, const double* __restrict__ pc9,
                        float* __restrict__ Vp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)pk_ne * K8) return;
  const int64_t i = t / K8;
  const int c = (int)(t % K8);
  const double v0 = V[i * K8 + c], v1 = V[((int64_t)pk_ne + i) * K8 + c], v2 = V[(2 * (int64_t)pk_ne + i) * K8 + c];
  const double* mi = pc9 + 9 * i;
#pragma unroll
  for (int b = 0; b < 3; ++b)
    Vp[((int64_t)b * K8 + c) * pk_ldp + i] = (float)(mi[3 * b] * v0 + mi[3 * b + 1] * v1 + mi[3 * b + 2] * v2);
}
// inverses of the elements' 3x3 self blocks of the packed matrix (FP64 from the
// stored FP32 values); bad = 1 for a singular or non-finite block
__global__ void k_pc_blocks(int pk_ne, int pk_ldp, const float* __restrict__ Ap, double* __restrict__ pc9,
                            int* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pk_ne) return;
  double B[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) B[a][b] = (double)Ap[pk_idx(i, sym6(a, b), i, pk_ldp)];
  if (!inv3(B, pc9 + 9 * (int64_t)i)) atomicExch(bad, 1);
}
__global__ void k_sumsq_rows(const double* __restrict__ B, int rows, double* __restrict__ part) {
  __shared__ double sP[kThreads / 32][K8];
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  double v = (t < (int64_t)rows * K8) ? B[t] : 0.0;
  double s = v * v;
  s += __shfl_xor_sync(0xffffffffu, s, 8);
  s += __shfl_xor_sync(0xffffffffu, s, 16);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < K8) sP[warp][lane] = s;
  __syncthreads();
  if (threadIdx.x < K8) {
    double a = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) a += sP[w][threadIdx.x];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = a;
  }
}
// tolerances of lsqr_solve: atol = eps, btol = eps*||b||/||r0||, conlim 1e8
__global__ void k_setup_tol(LsqrScalars* sc, int k, const double* part_b, int nb_b, double eps, int itnlim) {
  const int c = threadIdx.x;
  if (c >= K8) return;
  LsqrScalars& s = sc[c];
  if (c >= k) { s.active = 0; return; }
  const double nrm_b = sqrt(sum_part(part_b, nb_b, c));
  s.atol = eps;
  s.btol = eps * nrm_b / s.beta;
  s.ctol = 1.0 / 1.0e8;
  s.itnlim = itnlim;
  s.active = (s.beta > 0.0) ? 1 : 0;
  s.istop = 0;
  s.itn = 0;
  s.alpha = 0.0;
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
static inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Build a 2-D tensor map of the row-major FP32 matrix (dims {lda, m}) with the
// given box, through the driver entry point (no link against libcuda).
bool make_tensor_map_2d(CUtensorMap* tm, const void* A, int64_t lda, int m, int box_cols, int box_rows,
                        std::string& err) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      err = "cuTensorMapEncodeTiled not available";
      return false;
    }
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t dims[2] = {(cuuint64_t)lda, (cuuint64_t)m};
  const cuuint64_t strides[1] = {(cuuint64_t)lda * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(A), dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
    return false;
  }
  return true;
}

// 3-D tensor map of the packed layout (pk_idx): dims {64 columns, 6 x pldp/64
// (plane, column block), rows}, box {64, box_y, box_z}.
bool make_packed_map(CUtensorMap* tm, const void* Ap, int pldp, int ne, int box_y, int box_z, std::string& err) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      err = "cuTensorMapEncodeTiled not available";
      return false;
    }
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t dims[3] = {64, (cuuint64_t)6 * (pldp / 64), (cuuint64_t)ne};
  const cuuint64_t strides[2] = {64 * sizeof(float), (cuuint64_t)6 * pldp * sizeof(float)};
  const cuuint32_t box[3] = {64, (cuuint32_t)box_y, (cuuint32_t)box_z};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(Ap), dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    err = "cuTensorMapEncodeTiled (packed) failed (" + std::to_string((int)r) + ")";
    return false;
  }
  return true;
}

template <typename T>
static void launch_resid(const DenseLsqr& L, const double* Xs, const double* Bp) {
  if (L.packed) {
    if (L.resid_fp64) {
      k_residp<<<cdiv(L.pk_ne, 8), 256, 0, L.stream>>>((const float*)L.A, L.pk_ne, L.pk_ldp, Xs, L.mf_q, Bp, L.Y,
                                                       (float*)L.Ys, L.part);
      return;
    }
    // products and sums on the FP32 pipe in float-float form (k_residp_ff)
    const int64_t n8 = (int64_t)3 * L.pk_ne * K8;
    float* Xh = L.Xff;
    float* Xl = L.Xff + L.lda * K8;
    k_split_x<<<(unsigned)std::min<int64_t>(cdiv(n8, 256), 4096), 256, 0, L.stream>>>(n8, Xs, L.mf_q, Xh, Xl);
    if (L.k <= 6)
      k_residp_ff<6><<<cdiv(L.pk_ne, 8), 256, 0, L.stream>>>((const float*)L.A, L.pk_ne, L.pk_ldp, Xh, Xl, Bp, L.Y,
                                                              (float*)L.Ys, L.part);
    else
      k_residp_ff<8><<<cdiv(L.pk_ne, 8), 256, 0, L.stream>>>((const float*)L.A, L.pk_ne, L.pk_ldp, Xh, Xl, Bp, L.Y,
                                                              (float*)L.Ys, L.part);
    return;
  }
  const unsigned nb = cdiv(L.m, AV_ROWS);
  k_av<T, double><<<nb, kThreads, 0, L.stream>>>((const T*)L.A, L.lda, L.m, L.n, Xs, -1.0, L.sc, 0, Bp, L.Y,
                                                 (T*)L.Ys, L.part);
}
template <typename T>
static unsigned av2_blocks(const DenseLsqr& L) { return cdiv(L.m, AV2<T>::WARPS * AV2<T>::RR); }
template <typename T>
static void launch_av2(const DenseLsqr& L) {
  if (L.packed) {
    k_avp<<<cdiv(L.pk_ne, AVP_R), AVP_THREADS, AVP_SMEM, L.stream>>>(L.tm_av, L.tm_vp, L.pk_ne, L.pk_ldp,
                                                                    L.sc, L.Y, (float*)L.Ys,
                                                                              L.part, L.errflag);
    return;
  }
  if (L.mf) {
    mf_av(*L.mf, (const float*)L.Vs, L.mf_q, L.lda, L.Yp, L.stream);
    mf_av_reduce(L.m, L.mf_cb, L.Yp, L.sc, L.Y, (float*)L.Ys, L.part, L.stream);
    return;
  }
  if (sizeof(T) == 4 && L.use_tma) {
    k_av3<<<cdiv(L.m, AV3_ROWS), AV3_WARPS * 32, AV3_SMEM, L.stream>>>(L.tm_av, L.lda, L.m, (const float*)L.Vs, L.sc,
                                                                       L.Y, (float*)L.Ys, L.part, L.errflag);
    return;
  }
  const size_t smem = 2 * K8 * AV2<T>::CH * sizeof(T);
  k_av2<T><<<av2_blocks<T>(L), AV2<T>::WARPS * 32, smem, L.stream>>>((const T*)L.A, L.lda, L.m, (const T*)L.Vs, L.sc,
                                                                     L.Y, (T*)L.Ys, L.part, L.errflag);
}
// k_avp that does nothing once no right-hand side is active (*gate == 0): the
// iterations replayed after the last one converged read no matrix
__global__ void __launch_bounds__(AVP_THREADS, 1) k_avp_gated(const __grid_constant__ CUtensorMap tmA,
                                                             const __grid_constant__ CUtensorMap tmW, int ne, int ldp,
                                                             const LsqrScalars* sc, double* __restrict__ Y,
                                                             float* __restrict__ Ys, double* __restrict__ part,
                                                             int* errflag, const int* __restrict__ gate) {
  if (*gate == 0) return;
  avp_tile(&tmA, &tmW, ne, ldp, sc, Y, Ys, part, errflag, (int)blockIdx.x);
}
void launch_avp(const DenseLsqr& L, const LsqrScalars* sc, double* Yout, const int* gate) {
  k_avp_gated<<<cdiv(L.pk_ne, AVP_R), AVP_THREADS, AVP_SMEM, L.stream>>>(L.tm_av, L.tm_vp, L.pk_ne, L.pk_ldp, sc, Yout,
                                                                        (float*)L.Ys, L.part, L.errflag, gate);
}
template <typename T>
static size_t atu2_smem() {
  return 256 * K8 * sizeof(T) + (sizeof(T) == 4 ? (size_t)Vec<T>::N * K8 * ATU_THREADS * sizeof(double) : 0);
}
template <typename T>
static void launch_atu(const DenseLsqr& L) {
  if (L.packed) {
    const int rpg = (int)((cdiv(L.pk_ne, L.zgroups) + ATUP_RS - 1) / ATUP_RS * ATUP_RS);
    k_atup<<<dim3(cdiv(L.pk_ldp, ATUP_C), L.zgroups), ATUP_C, ATUP_SMEM, L.stream>>>(
        L.tm_atu, L.pk_ne, L.pk_ldp, L.lda, (const float*)L.Ys, rpg, L.Zp, L.errflag);
    return;
  }
  if (L.mf) {
    mf_atu(*L.mf, (const float*)L.Ys, L.mf_q, L.lda, L.Zp, false, L.stream);
    return;
  }
  if (sizeof(T) == 4 && L.use_tma) {
    dim3 g(cdiv(L.lda, ATU3_COLS), L.zgroups);
    const int rpg = (int)((cdiv(L.m, L.zgroups) + 31) / 32 * 32);
    k_atu3<<<g, ATU3_THREADS, ATU3_SMEM, L.stream>>>(L.tm_atu, L.lda, L.m, (const float*)L.Ys, rpg, L.Zp, L.errflag);
    return;
  }
  constexpr int vn = Vec<T>::N;
  dim3 g(cdiv(L.lda, ATU_THREADS * vn), L.zgroups);
  const int rpg = (int)((cdiv(L.m, L.zgroups) + 31) / 32 * 32);
  k_atu2<T><<<g, ATU_THREADS, atu2_smem<T>(), L.stream>>>((const T*)L.A, L.lda, L.m, (const T*)L.Ys, rpg, L.Zp);
}
template <typename T>
static cudaError_t set_sweep_attrs() {
  cudaError_t e = cudaFuncSetAttribute(k_av2<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(2 * K8 * AV2<T>::CH * sizeof(T)));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_av3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AV3_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_atu3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ATU3_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_avp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AVP_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_avp_gated, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AVP_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_atup, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ATUP_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_atu2<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)atu2_smem<T>());
  return e;
}

void DenseLsqr::release() {
  if (pev_ready)
    for (int i = 0; i < 4 * 32; ++i) cudaEventDestroy(pev[i]);
  pev_ready = false;
  cudaFree(Y); cudaFree(V); cudaFree(W); cudaFree(X); cudaFree(Z); cudaFree(Ys); cudaFree(Vs);
  cudaFree(part); cudaFree(Zp); cudaFree(sc); cudaFree(nactive); cudaFree(XsD); cudaFree(errflag); cudaFree(Yp); cudaFree(Vp);
  cudaFree(bg); cudaFree(bg_part); cudaFree(bsc); cudaFree(sc0); cudaFree(pc9);
  cudaFree(gm); cudaFree(gm_part); cudaFree(gsc); cudaFree(Xff);
  Xff = nullptr;
  gm = nullptr; gm_part = nullptr; gsc = nullptr; gm_cap = 0; gm_mr = 0;
  pc9 = nullptr;
  pc9_ready = false;
  bj = false;
  bg = bg_part = nullptr;
  bsc = nullptr;
  sc0 = nullptr;
  bg_diag = false;
  Yp = nullptr;
  Vp = nullptr;
  XsD = nullptr; errflag = nullptr;
  if (h_nactive) cudaFreeHost(h_nactive);
  Y = V = W = X = Z = nullptr; Ys = Vs = nullptr; part = Zp = nullptr; sc = nullptr; nactive = nullptr;
  h_nactive = nullptr;
}
DenseLsqr::~DenseLsqr() { release(); }

bool DenseLsqr::setup(const void* A_dev, bool is_fp32, int m_, int n_, int64_t lda_, int k_, cudaStream_t s) {
  release();
  A = A_dev; fp32 = is_fp32; m = m_; n = n_; lda = lda_; k = k_; stream = s;
  if (k < 1 || k > K8) { err = "number of right-hand sides must be 1..8"; return false; }
  if (lda % 32 != 0 || lda < n) { err = "lda must be a multiple of 32 and >= n"; return false; }
  const size_t tsz = fp32 ? sizeof(float) : sizeof(double);
  const int64_t mpad = ((int64_t)m + 255) / 256 * 256;
  CK(cudaMalloc(&Y, mpad * K8 * sizeof(double)));
  CK(cudaMalloc(&Ys, mpad * K8 * tsz));
  CK(cudaMalloc(&V, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&W, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&X, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&Z, std::max<int64_t>(lda, mpad) * K8 * sizeof(double)));  // b / x0 staging
  CK(cudaMalloc(&Vs, lda * K8 * sizeof(double)));                            // T copy, or FP64 for residual
  // row groups for sweep 2: aim for >= 4 CTAs per SM
  use_tma = fp32 && getenv("AGB_NO_TMA") == nullptr && A_dev != nullptr && !packed;
  if (!A_dev && !mf) { err = "no matrix and no matrix-free operator"; return false; }
  if (packed) {
    if (!fp32 || 3 * pk_ne != m || m != n || pk_ldp % 64 != 0 || pk_ldp < pk_ne) {
      err = "packed layout: bad sizes";
      return false;
    }
    if (!make_packed_map(&tm_av, A_dev, pk_ldp, pk_ne, 6 * AVP_NB, AVP_R, err)) return false;
    if (!make_packed_map(&tm_atu, A_dev, pk_ldp, pk_ne, 6 * (ATUP_C / 64), ATUP_RS, err)) return false;
    CK(cudaMalloc(&Vp, (size_t)3 * K8 * pk_ldp * sizeof(float)));
    CK(cudaMemsetAsync(Vp, 0, (size_t)3 * K8 * pk_ldp * sizeof(float), stream));
    if (!make_tensor_map_2d(&tm_vp, Vp, pk_ldp, 3 * K8, AVP_BC, 3 * K8, err)) return false;
  }
  if (use_tma) {
    if (!make_tensor_map_2d(&tm_av, A_dev, lda, m, SWEEP_BC, AV3_ROWS, err)) return false;
    if (!make_tensor_map_2d(&tm_atu, A_dev, lda, m, 256, ATU3_RS, err)) return false;
  }
  const int vn = fp32 ? 4 : 2;
  const int colblocks = use_tma ? (int)cdiv(lda, ATU3_COLS) : (int)cdiv(lda, ATU_THREADS * vn);
  // row groups of sweep 2: fill whole waves of resident CTAs
  CK(fp32 ? set_sweep_attrs<float>() : set_sweep_attrs<double>());
  int per_sm = 1, nsm = 152;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (use_tma) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_atu3, ATU3_THREADS, ATU3_SMEM);
    else if (fp32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_atu2<float>, ATU_THREADS, atu2_smem<float>());
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_atu2<double>, ATU_THREADS, atu2_smem<double>());
    per_sm = std::max(per_sm, 1);
  }
  const int slots = nsm * per_sm;
  const int gmax = std::max(1, std::min((int)cdiv(m, use_tma ? 64 : 32), 64));
  int groups = 1;
  double best = -1.0;
  for (int G = 1; G <= gmax; ++G) {
    const int64_t items = (int64_t)colblocks * G;
    const double eff = (double)items / (double)(cdiv(items, slots) * (int64_t)slots);
    const double score = eff - 0.002 * G;  // prefer fewer partial sums at equal fill
    if (items >= slots / 2 && score > best) { best = score; groups = G; }
    if (best < 0 && G == gmax) groups = G;
  }
  zgroups = groups;
  if (packed) {  // row groups of the packed A^T U tiles: fill whole waves of resident CTAs
    int occ = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_atup, ATUP_C, ATUP_SMEM);
    const int pslots = nsm * std::max(occ, 1);
    const int cb = (int)cdiv(pk_ldp, ATUP_C);
    const int gmx = std::max(1, std::min(64, (int)cdiv(pk_ne, 64)));
    double bestp = -1.0;
    zgroups = 1;
    for (int G = 1; G <= gmx; ++G) {
      const int64_t items = (int64_t)cb * G;
      const double eff = (double)items / (double)(cdiv(items, pslots) * (int64_t)pslots);
      const double score = eff - 0.002 * G;
      if (items >= pslots && score > bestp) { bestp = score; zgroups = G; }
      if (bestp < 0 && G == gmx) zgroups = G;
    }
  }
  if (mf) {
    zgroups = mf_row_groups(*mf);
    mf_cb = mf_col_blocks(*mf);
    CK(cudaMalloc(&Yp, (size_t)mf_cb * m * K8 * sizeof(float)));
  }
  CK(cudaMalloc(&XsD, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&Xff, 2 * lda * K8 * sizeof(float)));
  CK(cudaMalloc(&errflag, sizeof(int)));
  CK(cudaMemsetAsync(errflag, 0, sizeof(int), stream));
  CK(cudaMalloc(&Zp, (int64_t)zgroups * lda * K8 * sizeof(double)));
  const int64_t nbmax = std::max<int64_t>({(int64_t)cdiv(m, 16), (int64_t)cdiv(m, AV_ROWS),
                                           (int64_t)cdiv(lda * K8, kThreads), (int64_t)cdiv(mpad * K8, kThreads)});
  part_cap = (size_t)nbmax * K8 * 2;
  CK(cudaMalloc(&part, part_cap * sizeof(double)));
  CK(cudaMalloc(&sc, K8 * sizeof(LsqrScalars)));
  CK(cudaMemsetAsync(sc, 0, K8 * sizeof(LsqrScalars), stream));
  CK(cudaMalloc(&nactive, sizeof(int)));
  CK(cudaMallocHost(&h_nactive, sizeof(int)));
  CK(cudaMemsetAsync(Vs, 0, lda * K8 * sizeof(double), stream));
  CK(cudaMemsetAsync(Y, 0, mpad * K8 * sizeof(double), stream));
  CK(cudaMemsetAsync(Ys, 0, mpad * K8 * tsz, stream));
  CK(cudaMemsetAsync(V, 0, lda * K8 * sizeof(double), stream));
  CK(cudaMemsetAsync(W, 0, lda * K8 * sizeof(double), stream));
  CK(cudaMemsetAsync(X, 0, lda * K8 * sizeof(double), stream));
  return true;
}

cudaError_t packed_colnorms(const float* Ap, int ne, int ldp, int64_t lda, double* q, double* P, int groups,
                            cudaStream_t s) {
  const int rpg = (int)cdiv(ne, groups);
  k_colsqp<<<dim3(cdiv(ne, 256), groups), 256, 0, s>>>(Ap, ne, ldp, rpg, P, lda);
  k_colsq_finish<<<cdiv(lda, 256), 256, 0, s>>>(P, groups, lda, 3 * ne, q);
  return cudaGetLastError();
}

bool DenseLsqr::precon(void* A_dev, double* q_dev) {
  if (packed) {  // q from the packed columns; the matrix stays unscaled, q is applied in the sweeps
    const int rpg = (int)cdiv(pk_ne, zgroups);
    k_colsqp<<<dim3(cdiv(pk_ne, 256), zgroups), 256, 0, stream>>>((const float*)A_dev, pk_ne, pk_ldp, rpg, Zp, lda);
    k_colsq_finish<<<cdiv(lda, 256), 256, 0, stream>>>(Zp, zgroups, lda, n, q_dev);
    launches += 2;
    CK(cudaGetLastError());
    return true;
  }
  if (mf) {  // q from the recomputed column sums of squares; A itself is never stored or scaled
    CK(mf_atu(*mf, nullptr, nullptr, lda, Zp, true, stream));
    k_colsq_finish<<<cdiv(lda, 256), 256, 0, stream>>>(Zp, zgroups, lda, n, q_dev);
    launches += 2;
    CK(cudaGetLastError());
    return true;
  }
  const int vn = fp32 ? 4 : 2;
  dim3 g(cdiv(lda, kThreads * vn), zgroups);
  const int rpg = (int)cdiv(m, zgroups);
  if (fp32) k_colsq<float><<<g, kThreads, 0, stream>>>((const float*)A_dev, lda, m, rpg, Zp);
  else k_colsq<double><<<g, kThreads, 0, stream>>>((const double*)A_dev, lda, m, rpg, Zp);
  k_colsq_finish<<<cdiv(lda, 256), 256, 0, stream>>>(Zp, zgroups, lda, n, q_dev);
  const int64_t tot = (int64_t)m * lda;
  unsigned blocks = (unsigned)std::min<int64_t>(cdiv(tot, 256), 152 * 64);
  if (fp32) k_scale_cols<float><<<blocks, 256, 0, stream>>>((float*)A_dev, lda, m, q_dev);
  else k_scale_cols<double><<<blocks, 256, 0, stream>>>((double*)A_dev, lda, m, q_dev);
  launches += 3;
  CK(cudaGetLastError());
  return true;
}

template <typename T>
__global__ void k_init_y(const double* __restrict__ Bp, int64_t count, double* __restrict__ Y, T* __restrict__ Ys) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  Y[t] = Bp[t];
  Ys[t] = (T)Bp[t];
}

bool DenseLsqr::solve(const double* b_dev, double* x_dev, const double* q_dev, double eps, int maxit, int* nit_host,
                      int* istop_host, double* rnorm_host, int check_every, bool x0_zero) {
  if (maxit == 0) maxit = 10 * (m + n + 50);
  const bool use_bj = bj && packed && fp32 && pc9 && pc9_ready;
  if (bj && !use_bj) { err = "the block preconditioner needs the packed mixed matrix"; return false; }
  const int64_t mpad = ((int64_t)m + 255) / 256 * 256;
  const unsigned nb_av = packed ? cdiv(pk_ne, 8) : cdiv(m, AV_ROWS);  // residual sweep
  const unsigned nb_av2 = packed ? cdiv(pk_ne, AVP_R) : mf ? cdiv((int64_t)m * K8, 256)
                            : fp32 ? (use_tma ? cdiv(m, AV3_ROWS) : av2_blocks<float>(*this)) : av2_blocks<double>(*this);
  mf_q = q_dev;
  if (mf && !x0_zero) { err = "the matrix-free operator needs a zero warm start"; return false; }
  CK(fp32 ? set_sweep_attrs<float>() : set_sweep_attrs<double>());
  const unsigned nb_red = cdiv((int64_t)n * K8, kThreads);
  const unsigned nb_upd = cdiv(lda * K8, kThreads);
  // stage: b -> Z (as [m][8]); x0 -> X0 buffer (as [n][8]); xs = x0/q -> Vs (FP64)
  double* Bp = Z;
  k_pack<<<cdiv(mpad * K8, 256), 256, 0, stream>>>(b_dev, m, k, mpad, nullptr, Bp);
  k_sumsq_rows<<<cdiv(mpad * K8, kThreads), kThreads, 0, stream>>>(Bp, (int)mpad, part);
  const int nb_b = (int)cdiv(mpad * K8, kThreads);
  // ||b|| partials are consumed right after the residual is known; keep them
  // in the upper half of `part`
  double* part_b = part + (part_cap / 2);
  if ((size_t)nb_b * K8 > part_cap / 2) { err = "partial buffer too small"; return false; }
  CK(cudaMemcpyAsync(part_b, part, (size_t)nb_b * K8 * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  if (x0_zero) {
    // r0 = b: no sweep over A; ||r0|| from the partials of ||b||
    if (fp32) k_init_y<float><<<cdiv((int64_t)m * K8, 256), 256, 0, stream>>>(Bp, (int64_t)m * K8, Y, (float*)Ys);
    else k_init_y<double><<<cdiv((int64_t)m * K8, 256), 256, 0, stream>>>(Bp, (int64_t)m * K8, Y, (double*)Ys);
    k_scalars<<<1, SCAL_THREADS, 0, stream>>>(sc, k, 0, part_b, nb_b, nactive);
  } else {
    k_pack<<<cdiv(lda * K8, 256), 256, 0, stream>>>(x_dev, n, k, lda, q_dev, XsD);
    // residual Y = b - A (x0/q), FP64 accumulation
    if (fp32) launch_resid<float>(*this, XsD, Bp);
    else launch_resid<double>(*this, XsD, Bp);
    k_scalars<<<1, SCAL_THREADS, 0, stream>>>(sc, k, 0, part, nb_av, nactive);
  }
  k_setup_tol<<<1, 32, 0, stream>>>(sc, k, part_b, nb_b, eps, maxit);
  // keep x0 (packed) for the final update: in X0 = W (W is rewritten by the init update,
  // so copy x0 to Bp region first: Bp is no longer needed)
  k_pack<<<cdiv(lda * K8, 256), 256, 0, stream>>>(x_dev, n, k, lda, nullptr, Bp);
  // A^T r, alpha0, w = v
  if (fp32) launch_atu<float>(*this); else launch_atu<double>(*this);
  const double* qs = packed ? q_dev : nullptr;
  k_atu_reduce<<<nb_red, kThreads, 0, stream>>>(Zp, zgroups, lda, n, sc, 1, V, part, qs, use_bj ? pc9 : nullptr,
                                               pk_ne);
  k_scalars<<<1, SCAL_THREADS, 0, stream>>>(sc, k, 1, part, nb_red, nactive);
  if (fp32) k_update<float><<<nb_upd, kThreads, 0, stream>>>(n, lda, sc, 1, V, W, X, (float*)Vs, part, 1, Vp, pk_ne,
                                                              pk_ldp, qs, use_bj ? 1 : 0);
  else k_update<double><<<nb_upd, kThreads, 0, stream>>>(n, lda, sc, 1, V, W, X, (double*)Vs, part, 1);
  if (use_bj) k_pc_vp<<<cdiv((int64_t)pk_ne * K8, 256), 256, 0, stream>>>(pk_ne, pk_ldp, V, pc9, Vp);
  launches += (x0_zero ? 10 : 11) + (use_bj ? 1 : 0);
  CK(cudaGetLastError());

  if (check_every > 32) check_every = 32;
  if (!pev_ready) {
    for (int i = 0; i < 4 * 32; ++i) CK(cudaEventCreate(&pev[i]));
    pev_ready = true;
  }
  int it_in_graph = 0;
  // the two sweeps of the first iteration of every replay are timed live (event
  // records in the graph); the other iterations carry no event nodes
  auto iteration = [&]() {
    const bool timed = it_in_graph++ == 0;
    if (timed) cudaEventRecordWithFlags(pev[0], stream, cudaEventRecordExternal);
    if (fp32) launch_av2<float>(*this);
    else launch_av2<double>(*this);
    if (timed) cudaEventRecordWithFlags(pev[1], stream, cudaEventRecordExternal);
    k_scalars<<<1, SCAL_THREADS, 0, stream>>>(sc, k, 2, part, nb_av2, nactive);
    if (timed) cudaEventRecordWithFlags(pev[2], stream, cudaEventRecordExternal);
    if (fp32) launch_atu<float>(*this); else launch_atu<double>(*this);
    if (timed) cudaEventRecordWithFlags(pev[3], stream, cudaEventRecordExternal);
    k_atu_reduce<<<nb_red, kThreads, 0, stream>>>(Zp, zgroups, lda, n, sc, 0, V, part, qs, use_bj ? pc9 : nullptr,
                                                 pk_ne);
    k_scalars<<<1, SCAL_THREADS, 0, stream>>>(sc, k, 3, part, nb_red, nactive);
    if (fp32) k_update<float><<<nb_upd, kThreads, 0, stream>>>(n, lda, sc, 0, V, W, X, (float*)Vs, part, 1, Vp, pk_ne,
                                                                pk_ldp, qs, use_bj ? 1 : 0);
    else k_update<double><<<nb_upd, kThreads, 0, stream>>>(n, lda, sc, 0, V, W, X, (double*)Vs, part, 1);
    if (use_bj) k_pc_vp<<<cdiv((int64_t)pk_ne * K8, 256), 256, 0, stream>>>(pk_ne, pk_ldp, V, pc9, Vp);
    k_scalars<<<1, SCAL_THREADS, 0, stream>>>(sc, k, 4, part, nb_upd, nactive);  // phase 3 zeroed nactive
  };
  // capture check_every iterations in one graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  for (int i = 0; i < check_every; ++i) iteration();
  CK(cudaStreamEndCapture(stream, &graph));
  CK(cudaGraphInstantiate(&gexec, graph, 0));
  // initial activity
  LsqrScalars hs[K8];
  CK(cudaMemcpyAsync(hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  int act = 0;
  for (int c = 0; c < k; ++c) act += hs[c].active;
  int iters = 0;
  while (act > 0 && iters < maxit + check_every) {
    CK(cudaGraphLaunch(gexec, stream));
    launches += (use_bj ? 8L : 7L) * check_every;
    CK(cudaMemcpyAsync(h_nactive, nactive, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    {
      float a = 0.f, b = 0.f;
      if (cudaEventElapsedTime(&a, pev[0], pev[1]) == cudaSuccess) { t_av += a; ++n_av; }
      if (cudaEventElapsedTime(&b, pev[2], pev[3]) == cudaSuccess) { t_atu += b; ++n_atu; }
    }
    (void)cudaGetLastError();  // a timing query must not leak into the error checks
    iters += check_every;
    act = *h_nactive;
  }
  cudaGraphExecDestroy(gexec);
  cudaGraphDestroy(graph);
  // x = q .* dx + x0
  k_finish_x<<<cdiv((int64_t)n * k, 256), 256, 0, stream>>>(X, q_dev, Bp, n, k, sc, x_dev, use_bj ? pc9 : nullptr,
                                                             pk_ne);
  launches += 1;
  CK(cudaMemcpyAsync(hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  CK(cudaGetLastError());
  int hflag = 0;
  CK(cudaMemcpy(&hflag, errflag, sizeof(int), cudaMemcpyDeviceToHost));
  if (hflag) { err = "a bounded barrier wait in the A*V sweep gave up"; return false; }
  for (int c = 0; c < k; ++c) {
    if (nit_host) nit_host[c] = hs[c].itn;
    if (istop_host) istop_host[c] = hs[c].istop;
    if (rnorm_host) rnorm_host[c] = hs[c].rnorm;
  }
  return true;
}

bool DenseLsqr::block_precon() {
  if (!packed || !A) { err = "the block preconditioner needs the packed mixed matrix"; return false; }
  if (pc9_ready) return true;
  if (!pc9) CK(cudaMalloc(&pc9, (size_t)pk_ne * 9 * sizeof(double)));
  CK(cudaMemsetAsync(nactive, 0, sizeof(int), stream));
  k_pc_blocks<<<cdiv(pk_ne, 128), 128, 0, stream>>>(pk_ne, pk_ldp, (const float*)A, pc9, nactive);
  CK(cudaGetLastError());
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, nactive, sizeof(int), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  ++launches;
  if (bad) { err = "a singular 3x3 self block: the block preconditioner cannot be formed"; return false; }
  pc9_ready = true;
  return true;
}

bool DenseLsqr::residual(const double* b_dev, const double* x_dev, const double* q_dev, double* r_dev) {
  mf_q = q_dev;
  const int64_t mpad = ((int64_t)m + 255) / 256 * 256;
  k_pack<<<cdiv(mpad * K8, 256), 256, 0, stream>>>(b_dev, m, k, mpad, nullptr, Z);
  k_pack<<<cdiv(lda * K8, 256), 256, 0, stream>>>(x_dev, n, k, lda, q_dev, XsD);
  if (fp32) launch_resid<float>(*this, XsD, Z);
  else launch_resid<double>(*this, XsD, Z);
  // unpack Y -> r (column-major)
  for (int c = 0; c < k; ++c)
    CK(cudaMemcpy2DAsync(r_dev + (int64_t)c * m, sizeof(double), Y + c, K8 * sizeof(double), sizeof(double), m,
                         cudaMemcpyDeviceToDevice, stream));
  CK(cudaGetLastError());
  return true;
}


// ---------------------------------------------------------------------------
// CRS LSQR (the lsqr_precon / lsqr_solve drop-ins).  1-based CRS as the
// reference passes it.  The transpose is built on the device by a stable sort
// of the column indices, so both products -- and the column norms of the
// preconditioner -- sum their terms in the reference's order.
// ---------------------------------------------------------------------------
}  // namespace agb
#include <cub/device/device_radix_sort.cuh>
namespace agb {

__global__ void k_iota_cols(int64_t nnz, const int* __restrict__ ja, int* __restrict__ key, int64_t* __restrict__ val) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnz) return;
  key[t] = ja[t] - 1;
  val[t] = t;
}
__global__ void k_row_of(int m, const int64_t* __restrict__ ia, int* __restrict__ rowof) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  for (int64_t t = ia[r] - 1; t < ia[r + 1] - 1; ++t) rowof[t] = r;
}
__global__ void k_colptr(int64_t nnz, int n, const int* __restrict__ skey, int64_t* __restrict__ cp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t > nnz) return;
  const int prev = (t == 0) ? -1 : skey[t - 1];
  const int cur = (t == nnz) ? n : skey[t];
  for (int c = prev + 1; c <= cur; ++c) cp[c] = t;
}
// y = s1 * A x + g y_old (warp per row); x, y in the [.][8] layout, column 0
__global__ void k_csr_av(int m, const int64_t* __restrict__ ia, const int* __restrict__ ja, const double* __restrict__ a,
                         const double* __restrict__ x, double s1, const LsqrScalars* sc, int use_gamma,
                         const double* __restrict__ yold, double* __restrict__ Y, double* __restrict__ Ys,
                         double* __restrict__ part) {
  __shared__ double sP[kThreads / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * (kThreads / 32) + warp;
  double ssq = 0.0;
  if (r < m) {
    double s = 0.0;
    for (int64_t t = ia[r] - 1 + lane; t < ia[r + 1] - 1; t += 32) s += a[t] * x[(int64_t)(ja[t] - 1) * K8];
    s = warp_sum(s);
    const double g = use_gamma ? sc[0].gamma : 1.0;
    const double y = s1 * s + (yold ? g * yold[(int64_t)r * K8] : 0.0);
    if (lane == 0) {
      Y[(int64_t)r * K8] = y;
      Ys[(int64_t)r * K8] = y;
    }
    ssq = y * y;
  }
  if (lane == 0) sP[warp] = ssq;
  __syncthreads();
  if (threadIdx.x < K8) {
    double acc = 0.0;
    if (threadIdx.x == 0)
      for (int w = 0; w < kThreads / 32; ++w) acc += sP[w];
    part[(int64_t)blockIdx.x * K8 + threadIdx.x] = acc;
  }
}
// Z(:,0) = A^T y via the transpose (CSC, rows ascending)
__global__ void k_csc_atu(int n, const int64_t* __restrict__ cp, const int* __restrict__ rows,
                          const double* __restrict__ av, const double* __restrict__ Ys, double* __restrict__ Zp) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  double s = 0.0;
  for (int64_t t = cp[warp] + lane; t < cp[warp + 1]; t += 32) s += av[t] * Ys[(int64_t)rows[t] * K8];
  s = warp_sum(s);
  if (lane < K8) Zp[(int64_t)warp * K8 + lane] = (lane == 0) ? s : 0.0;
}
// column sums of squares in row order, q = 1/sqrt
__global__ void k_csc_colnorm(int n, const int64_t* __restrict__ cp, const double* __restrict__ av,
                              double* __restrict__ q) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double s = 0.0;
  for (int64_t t = cp[j]; t < cp[j + 1]; ++t) s += av[t] * av[t];
  q[j] = 1.0 / sqrt(s);
}
__global__ void k_crs_scale(int64_t nnz, const int* __restrict__ ja, const double* __restrict__ q, double* __restrict__ a) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nnz) a[t] *= q[ja[t] - 1];
}
__global__ void k_gather(int64_t nnz, const int64_t* __restrict__ perm, const double* __restrict__ a,
                         const int* __restrict__ rowof, double* __restrict__ av, int* __restrict__ rows) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnz) return;
  av[t] = a[perm[t]];
  rows[t] = rowof[perm[t]];
}

struct CrsDev {
  int m = 0, n = 0;
  int64_t nnz = 0;
  int64_t* ia = nullptr;
  int* ja = nullptr;
  double* a = nullptr;
  int64_t* cp = nullptr;   // n+1
  int64_t* perm = nullptr;
  int* rows = nullptr;     // CSC row index per entry
  double* av = nullptr;    // CSC values
  std::string err;
  ~CrsDev() {
    cudaFree(ia); cudaFree(ja); cudaFree(a); cudaFree(cp); cudaFree(perm); cudaFree(rows); cudaFree(av);
  }
  bool upload(int m_, int n_, int64_t nnz_, const int64_t* ia_h, const int* ja_h, const double* a_h, cudaStream_t s) {
    m = m_; n = n_; nnz = nnz_;
    CK(cudaMalloc(&ia, (m + 1) * sizeof(int64_t)));
    CK(cudaMalloc(&ja, std::max<int64_t>(nnz, 1) * sizeof(int)));
    CK(cudaMalloc(&a, std::max<int64_t>(nnz, 1) * sizeof(double)));
    CK(cudaMemcpyAsync(ia, ia_h, (m + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ja, ja_h, nnz * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(a, a_h, nnz * sizeof(double), cudaMemcpyHostToDevice, s));
    return true;
  }
  // build the CSC structure (values gathered from the current a)
  bool transpose(cudaStream_t s) {
    int *key = nullptr, *skey = nullptr, *rowof = nullptr;
    int64_t* val = nullptr;
    CK(cudaMalloc(&key, std::max<int64_t>(nnz, 1) * sizeof(int)));
    CK(cudaMalloc(&skey, std::max<int64_t>(nnz, 1) * sizeof(int)));
    CK(cudaMalloc(&val, std::max<int64_t>(nnz, 1) * sizeof(int64_t)));
    CK(cudaMalloc(&perm, std::max<int64_t>(nnz, 1) * sizeof(int64_t)));
    CK(cudaMalloc(&rowof, std::max<int64_t>(nnz, 1) * sizeof(int)));
    CK(cudaMalloc(&rows, std::max<int64_t>(nnz, 1) * sizeof(int)));
    CK(cudaMalloc(&av, std::max<int64_t>(nnz, 1) * sizeof(double)));
    CK(cudaMalloc(&cp, (n + 1) * sizeof(int64_t)));
    k_iota_cols<<<cdiv(nnz, 256), 256, 0, s>>>(nnz, ja, key, val);
    k_row_of<<<cdiv(m, 256), 256, 0, s>>>(m, ia, rowof);
    size_t tmpb = 0;
    int bits = 1;
    while ((1 << bits) <= n && bits < 31) ++bits;
    cub::DeviceRadixSort::SortPairs(nullptr, tmpb, key, skey, val, perm, nnz, 0, bits, s);
    void* tmp = nullptr;
    CK(cudaMalloc(&tmp, std::max<size_t>(tmpb, 1)));
    CK(cub::DeviceRadixSort::SortPairs(tmp, tmpb, key, skey, val, perm, nnz, 0, bits, s));
    k_colptr<<<cdiv(nnz + 1, 256), 256, 0, s>>>(nnz, n, skey, cp);
    k_gather<<<cdiv(nnz, 256), 256, 0, s>>>(nnz, perm, a, rowof, av, rows);
    CK(cudaStreamSynchronize(s));
    cudaFree(tmp); cudaFree(key); cudaFree(skey); cudaFree(val); cudaFree(rowof);
    CK(cudaGetLastError());
    return true;
  }
};

bool crs_lsqr_precon(int m, int n, int64_t nnz, double* q_h, const int64_t* ia_h, const int* ja_h, double* a_h,
                     std::string& err) {
  cudaStream_t s;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  {
    CrsDev D;
    if (!D.upload(m, n, nnz, ia_h, ja_h, a_h, s) || !D.transpose(s)) { err = D.err; cudaStreamDestroy(s); return false; }
    double* q = nullptr;
    CK(cudaMalloc(&q, std::max(n, 1) * sizeof(double)));
    k_csc_colnorm<<<cdiv(n, 256), 256, 0, s>>>(n, D.cp, D.av, q);
    k_crs_scale<<<cdiv(nnz, 256), 256, 0, s>>>(nnz, D.ja, q, D.a);
    CK(cudaMemcpyAsync(q_h, q, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(a_h, D.a, nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    cudaFree(q);
  }
  cudaStreamDestroy(s);
  return true;
}

bool crs_lsqr_solve(int m, int n, int64_t nnz, int& maxit, double eps, int& nit, int& ierr, const double* q_h,
                    const int64_t* ia_h, const int* ja_h, const double* a_h, const double* b_h, double* x_h,
                    std::string& err) {
  if (maxit == 0) maxit = 10 * (m + n + 50);
  cudaStream_t s;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  CrsDev D;
  if (!D.upload(m, n, nnz, ia_h, ja_h, a_h, s) || !D.transpose(s)) { err = D.err; cudaStreamDestroy(s); return false; }
  const int64_t lda = ((int64_t)n + 31) / 32 * 32;
  const int64_t mpad = ((int64_t)m + 255) / 256 * 256;
  double *q, *b, *x, *Y, *Ys, *V, *W, *X, *Vs, *Bp, *X0, *Zp, *part;
  LsqrScalars* sc;
  int* nact;
  CK(cudaMalloc(&q, lda * sizeof(double)));
  CK(cudaMalloc(&b, std::max(m, 1) * sizeof(double)));
  CK(cudaMalloc(&x, lda * sizeof(double)));
  CK(cudaMalloc(&Y, mpad * K8 * sizeof(double)));
  CK(cudaMalloc(&Ys, mpad * K8 * sizeof(double)));
  CK(cudaMalloc(&Bp, mpad * K8 * sizeof(double)));
  CK(cudaMalloc(&V, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&W, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&X, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&X0, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&Vs, lda * K8 * sizeof(double)));
  CK(cudaMalloc(&Zp, lda * K8 * sizeof(double)));
  const int64_t nbmax = std::max<int64_t>({(int64_t)cdiv(m, kThreads / 32), (int64_t)cdiv(lda * K8, kThreads),
                                           (int64_t)cdiv(mpad * K8, kThreads)});
  CK(cudaMalloc(&part, 2 * nbmax * K8 * sizeof(double)));
  CK(cudaMalloc(&sc, K8 * sizeof(LsqrScalars)));
  CK(cudaMalloc(&nact, sizeof(int)));
  CK(cudaMemsetAsync(sc, 0, K8 * sizeof(LsqrScalars), s));
  CK(cudaMemsetAsync(q, 0, lda * sizeof(double), s));
  CK(cudaMemsetAsync(x, 0, lda * sizeof(double), s));
  CK(cudaMemsetAsync(Ys, 0, mpad * K8 * sizeof(double), s));
  CK(cudaMemsetAsync(Y, 0, mpad * K8 * sizeof(double), s));
  CK(cudaMemsetAsync(V, 0, lda * K8 * sizeof(double), s));
  CK(cudaMemsetAsync(W, 0, lda * K8 * sizeof(double), s));
  CK(cudaMemsetAsync(X, 0, lda * K8 * sizeof(double), s));
  CK(cudaMemcpyAsync(q, q_h, n * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(b, b_h, m * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(x, x_h, n * sizeof(double), cudaMemcpyHostToDevice, s));
  const unsigned nb_av = cdiv(m, kThreads / 32);
  const unsigned nb_red = cdiv((int64_t)n * K8, kThreads);
  const unsigned nb_upd = cdiv(lda * K8, kThreads);
  const int nb_b = (int)cdiv(mpad * K8, kThreads);
  double* part_b = part + nbmax * K8;
  k_pack<<<cdiv(mpad * K8, 256), 256, 0, s>>>(b, m, 1, mpad, nullptr, Bp);
  k_sumsq_rows<<<nb_b, kThreads, 0, s>>>(Bp, (int)mpad, part_b);
  k_pack<<<cdiv(lda * K8, 256), 256, 0, s>>>(x, n, 1, lda, q, Vs);
  k_pack<<<cdiv(lda * K8, 256), 256, 0, s>>>(x, n, 1, lda, nullptr, X0);
  k_csr_av<<<nb_av, kThreads, 0, s>>>(m, D.ia, D.ja, D.a, Vs, -1.0, sc, 0, Bp, Y, Ys, part);
  k_scalars<<<1, SCAL_THREADS, 0, s>>>(sc, 1, 0, part, nb_av, nact);
  k_setup_tol<<<1, 32, 0, s>>>(sc, 1, part_b, nb_b, eps, maxit);
  k_csc_atu<<<cdiv((int64_t)n * 32, kThreads), kThreads, 0, s>>>(n, D.cp, D.rows, D.av, Ys, Zp);
  k_atu_reduce<<<nb_red, kThreads, 0, s>>>(Zp, 1, lda, n, sc, 1, V, part);
  k_scalars<<<1, SCAL_THREADS, 0, s>>>(sc, 1, 1, part, nb_red, nact);
  k_update<double><<<nb_upd, kThreads, 0, s>>>(n, lda, sc, 1, V, W, X, Vs, part, 0);
  CK(cudaGetLastError());
  LsqrScalars hs;
  int act = 1;
  CK(cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  act = hs.active;
  const int chunk = 16;
  cudaGraph_t graph;
  cudaGraphExec_t gexec;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int it = 0; it < chunk; ++it) {
    k_csr_av<<<nb_av, kThreads, 0, s>>>(m, D.ia, D.ja, D.a, Vs, 1.0, sc, 1, Y, Y, Ys, part);
    k_scalars<<<1, SCAL_THREADS, 0, s>>>(sc, 1, 2, part, nb_av, nact);
    k_csc_atu<<<cdiv((int64_t)n * 32, kThreads), kThreads, 0, s>>>(n, D.cp, D.rows, D.av, Ys, Zp);
    k_atu_reduce<<<nb_red, kThreads, 0, s>>>(Zp, 1, lda, n, sc, 0, V, part);
    k_scalars<<<1, SCAL_THREADS, 0, s>>>(sc, 1, 3, part, nb_red, nact);
    k_update<double><<<nb_upd, kThreads, 0, s>>>(n, lda, sc, 0, V, W, X, Vs, part, 0);
    cudaMemsetAsync(nact, 0, sizeof(int), s);
    k_scalars<<<1, SCAL_THREADS, 0, s>>>(sc, 1, 4, part, nb_upd, nact);
  }
  CK(cudaStreamEndCapture(s, &graph));
  CK(cudaGraphInstantiate(&gexec, graph, 0));
  int iters = 0;
  while (act > 0 && iters < maxit + chunk) {
    CK(cudaGraphLaunch(gexec, s));
    CK(cudaMemcpyAsync(&act, nact, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    iters += chunk;
  }
  cudaGraphExecDestroy(gexec);
  cudaGraphDestroy(graph);
  k_finish_x<<<cdiv(n, 256), 256, 0, s>>>(X, q, X0, n, 1, sc, x);
  CK(cudaMemcpyAsync(x_h, x, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  nit = hs.itn;
  ierr = (hs.istop > 3) ? hs.istop : 0;
  cudaFree(q); cudaFree(b); cudaFree(x); cudaFree(Y); cudaFree(Ys); cudaFree(Bp); cudaFree(V); cudaFree(W);
  cudaFree(X); cudaFree(X0); cudaFree(Vs); cudaFree(Zp); cudaFree(part); cudaFree(sc); cudaFree(nact);
  cudaStreamDestroy(s);
  return true;
}

}  // namespace agb
