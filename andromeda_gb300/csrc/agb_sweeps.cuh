// TMA-fed FP32 LSQR sweeps as tile bodies: over a row-major matrix (av3_tile /
// atu3_tile, used by k_av3 / k_atu3) and over the packed symmetric 3x3 blocks
// of a Stokes single layer (avp_tile / atup_tile, used by the single-system
// kernels k_avp / k_atup and by the batched kernels g_avp / g_atup that run
// many systems in one launch).
//
// Sweep 1 (av3_tile): Y = A V + gamma Y for ROWS rows of A and 8 right-hand
// sides.  A arrives in stages of ROWS x 256 columns by 2-D tensor-map copies,
// the matching 8 x 256 slice of V (RHS-major) by 1-D bulk copies; ST stages
// ring through shared memory with full/empty mbarriers (bounded waits).  A warp
// owns 4 rows; lanes hold 4 x 8 FP32 accumulators, reduce-scattered every 1024
// columns into one FP64 running sum per lane.
//
// Sweep 2 (atu3_tile): Zp[g] = A(rows of group g)^T Y for 512 columns; stages
// of RS rows (two 256-column boxes) plus RS rows of Y; a thread owns 2 columns
// x 8 right-hand sides, FP32 partials flushed into FP64 registers every 256
// rows.
#pragma once
#include "agb_async.cuh"

namespace agb {

constexpr int SWEEP_BC = 256;       // columns per tensor-map box
constexpr int ATU3_COLS = 512;      // columns per sweep-2 CTA
constexpr int ATU3_THREADS = 256;

template <int ROWS, int ST>
struct SweepAV {
  static constexpr int WARPS = ROWS / 4;
  static constexpr size_t STAGE_A = (size_t)ROWS * SWEEP_BC * sizeof(float);
  static constexpr size_t STAGE_V = (size_t)K8 * SWEEP_BC * sizeof(float);
  static constexpr size_t SMEM = ST * (STAGE_A + STAGE_V);
};
template <int RS, int ST>
struct SweepATU {
  static constexpr size_t STAGE_A = (size_t)RS * ATU3_COLS * sizeof(float);
  static constexpr size_t STAGE_U = (size_t)RS * K8 * sizeof(float);
  static constexpr size_t SMEM = ST * (STAGE_A + STAGE_U);
};

template <int ROWS, int ST>
__device__ __forceinline__ void av3_tile(const CUtensorMap* tmA, int64_t lda, int m, const float* __restrict__ Vt,
                                         const LsqrScalars* sc, double* __restrict__ Y, float* __restrict__ Ys,
                                         double* __restrict__ part, int* errflag, int blk) {
  using P = SweepAV<ROWS, ST>;
  constexpr int WARPS = P::WARPS;
  extern __shared__ __align__(1024) unsigned char sweep_smem[];
  float* sA = reinterpret_cast<float*>(sweep_smem);
  float* sV = reinterpret_cast<float*>(sweep_smem + ST * P::STAGE_A);
  __shared__ __align__(8) uint64_t full[ST], empty[ST];
  __shared__ double sPart[WARPS][K8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row_base = blk * ROWS;
  const int nst = (int)((lda + SWEEP_BC - 1) / SWEEP_BC);
  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], WARPS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int k) {
    const int s = k % ST;
    if (k >= ST) mbar_wait_bounded(&empty[s], (uint32_t)(((k / ST) - 1) & 1), errflag);
    const int64_t j0 = (int64_t)k * SWEEP_BC;
    const int cw = (int)((lda - j0) < (int64_t)SWEEP_BC ? (lda - j0) : (int64_t)SWEEP_BC);
    mbar_expect_tx(&full[s], (uint32_t)(P::STAGE_A + K8 * cw * sizeof(float)));
    tma_load_2d(sA + (size_t)s * ROWS * SWEEP_BC, tmA, (int)j0, row_base, &full[s]);
#pragma unroll
    for (int c = 0; c < K8; ++c)
      bulk_g2s(sV + (size_t)s * K8 * SWEEP_BC + c * SWEEP_BC, Vt + (int64_t)c * lda + j0,
               (uint32_t)(cw * sizeof(float)), &full[s]);
  };
  if (threadIdx.x == 0)
    for (int k = 0; k < ST && k < nst; ++k) issue(k);
  float acc[4][K8];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < K8; ++c) acc[r][c] = 0.f;
  double dacc = 0.0;
  for (int k = 0; k < nst; ++k) {
    const int s = k % ST;
    mbar_wait_bounded(&full[s], (uint32_t)((k / ST) & 1), errflag);
    const float* tA = sA + (size_t)s * ROWS * SWEEP_BC + (warp * 4) * SWEEP_BC;
    const float* tV = sV + (size_t)s * K8 * SWEEP_BC;
    const int64_t j0 = (int64_t)k * SWEEP_BC;
    const int cw = (int)((lda - j0) < (int64_t)SWEEP_BC ? (lda - j0) : (int64_t)SWEEP_BC);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int col = half * 128 + lane * 4;
      if (col < cw) {
        float a[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float4 v = *reinterpret_cast<const float4*>(tA + r * SWEEP_BC + col);
          a[r][0] = v.x; a[r][1] = v.y; a[r][2] = v.z; a[r][3] = v.w;
        }
#pragma unroll
        for (int c = 0; c < K8; ++c) {
          const float4 vv = *reinterpret_cast<const float4*>(tV + c * SWEEP_BC + col);
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            acc[r][c] = fmaf(a[r][0], vv.x, acc[r][c]);
            acc[r][c] = fmaf(a[r][1], vv.y, acc[r][c]);
            acc[r][c] = fmaf(a[r][2], vv.z, acc[r][c]);
            acc[r][c] = fmaf(a[r][3], vv.w, acc[r][c]);
          }
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    if (threadIdx.x == 0 && k + ST < nst) issue(k + ST);
    if ((k & 3) == 3 || k == nst - 1) {
      // reduce-scatter the 32 FP32 partials of 1024 columns into one FP64 sum per lane
      float v[32];
#pragma unroll
      for (int r = 0; r < 4; ++r)
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
    }
  }
  if (threadIdx.x == 0) mbar_drain(full, ST, nst, errflag);
  double ssq = 0.0;
  {
    const int r = lane >> 3, c = lane & 7, row = row_base + warp * 4 + r;
    if (row < m) {
      const double y = dacc + sc[c].gamma * Y[(int64_t)row * K8 + c];
      Y[(int64_t)row * K8 + c] = y;
      Ys[(int64_t)row * K8 + c] = (float)y;
      ssq = y * y;
    }
    ssq += __shfl_xor_sync(0xffffffffu, ssq, 8);
    ssq += __shfl_xor_sync(0xffffffffu, ssq, 16);
  }
  if (lane < K8) sPart[warp][lane] = ssq;
  __syncthreads();
  if (threadIdx.x < K8) {
    double a = 0.0;
    for (int w = 0; w < WARPS; ++w) a += sPart[w][threadIdx.x];
    part[(int64_t)blk * K8 + threadIdx.x] = a;
  }
}

template <int RS, int ST>
__device__ __forceinline__ void atu3_tile(const CUtensorMap* tmA, int64_t lda, int m, const float* __restrict__ Us,
                                          int rows_per_group, double* __restrict__ Zp, int* errflag, int cblk,
                                          int g) {
  using P = SweepATU<RS, ST>;
  constexpr int FLUSH = 256 / RS;  // stages per FP64 flush
  extern __shared__ __align__(1024) unsigned char sweep_smem[];
  float* sA = reinterpret_cast<float*>(sweep_smem);
  float* sU = reinterpret_cast<float*>(sweep_smem + ST * P::STAGE_A);
  __shared__ __align__(8) uint64_t full[ST], empty[ST];
  const int c0 = cblk * ATU3_COLS;
  const int r0 = g * rows_per_group, r1 = min(m, r0 + rows_per_group);
  const int nst = (r1 > r0) ? (r1 - r0 + RS - 1) / RS : 0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], ATU3_THREADS / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int k) {
    const int s = k % ST;
    if (k >= ST) mbar_wait_bounded(&empty[s], (uint32_t)(((k / ST) - 1) & 1), errflag);
    const int rb = r0 + k * RS;
    const int nr = min(RS, r1 - rb);
    mbar_expect_tx(&full[s], (uint32_t)(P::STAGE_A + (size_t)nr * K8 * sizeof(float)));
    float* dA = sA + (size_t)s * RS * ATU3_COLS;
    tma_load_2d(dA, tmA, c0, rb, &full[s]);
    tma_load_2d(dA + RS * SWEEP_BC, tmA, c0 + SWEEP_BC, rb, &full[s]);
    bulk_g2s(sU + (size_t)s * RS * K8, Us + (int64_t)rb * K8, (uint32_t)(nr * K8 * sizeof(float)), &full[s]);
  };
  if (threadIdx.x == 0)
    for (int k = 0; k < ST && k < nst; ++k) issue(k);
  const int tc = threadIdx.x * 2;          // the thread's two columns within the CTA block
  const int box = tc >> 8, off = tc & 255;  // tile and column within the tile
  float acc[2][K8];
  double dacc[2][K8];
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int c = 0; c < K8; ++c) { acc[q][c] = 0.f; dacc[q][c] = 0.0; }
  for (int k = 0; k < nst; ++k) {
    const int s = k % ST;
    mbar_wait_bounded(&full[s], (uint32_t)((k / ST) & 1), errflag);
    const int rb = r0 + k * RS;
    const int nr = min(RS, r1 - rb);
    const float* tA = sA + (size_t)s * RS * ATU3_COLS + box * RS * SWEEP_BC + off;
    const float* tU = sU + (size_t)s * RS * K8;
#pragma unroll 4
    for (int r = 0; r < nr; ++r) {
      const float2 a = *reinterpret_cast<const float2*>(tA + r * SWEEP_BC);
      const float4 u0 = *reinterpret_cast<const float4*>(tU + r * K8);
      const float4 u1 = *reinterpret_cast<const float4*>(tU + r * K8 + 4);
      const float uu[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
      for (int c = 0; c < K8; ++c) {
        acc[0][c] += a.x * uu[c];
        acc[1][c] += a.y * uu[c];
      }
    }
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[s]);
    if (threadIdx.x == 0 && k + ST < nst) issue(k + ST);
    if ((k % FLUSH) == FLUSH - 1 || k == nst - 1) {
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int c = 0; c < K8; ++c) { dacc[q][c] += (double)acc[q][c]; acc[q][c] = 0.f; }
    }
  }
  if (threadIdx.x == 0) mbar_drain(full, ST, nst, errflag);
  const int64_t col = (int64_t)c0 + tc;
#pragma unroll
  for (int q = 0; q < 2; ++q)
    if (col + q < lda)
#pragma unroll
      for (int c = 0; c < K8; ++c) Zp[((int64_t)g * lda + col + q) * K8 + c] = dacc[q][c];
}

// ---------------------------------------------------------------------------
// Tile bodies of the sweeps over the packed single layer (symmetric 3x3 blocks stored once, in
// the layout of pk_idx): A[3i+a][b ne + j] = Ap[pk_idx(i, sym(a,b), j)].
// The column scaling of lsqr_precon is applied on the fly: sweep 1 reads
// W = q.V (written by the vector update into Vp[b][k][ldp]), sweep 2's
// partials are scaled by q in the reduction of the row-group partials.
// ---------------------------------------------------------------------------
// A CTA owns AVP_R = 16 rows (two per compute warp, plus one producer warp) and
// streams them in stages of 3 column blocks (192 columns: 4.5 KB contiguous per
// row), two stages in flight.  Timed on GB300 against 12..30 rows per CTA and
// 64..256 columns per stage (random packed matrices of 5 440..20 800 rows):
// this shape was the fastest or within 2 % of it at every size, 0.92 of the
// copy bandwidth at 12 000..20 800 rows.
constexpr int AVP_R = 16, AVP_NB = 3, AVP_BC = 64 * AVP_NB, AVP_ST = 2, AVP_WARPS = AVP_R / 2;
constexpr int AVP_THREADS = (AVP_WARPS + 1) * 32;
constexpr size_t AVP_STAGE_A = 6 * (size_t)AVP_R * AVP_BC * sizeof(float);   // 72 KB
constexpr size_t AVP_STAGE_W = 3 * (size_t)K8 * AVP_BC * sizeof(float);      // 18 KB
constexpr size_t AVP_SMEM = AVP_ST * (AVP_STAGE_A + AVP_STAGE_W);

__device__ __forceinline__ int sym6(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}

// reduce-scatter of 32 per-lane FP32 slots: afterwards lane l holds the warp
// sum of slot l in v[0]
__device__ __forceinline__ void reduce_scatter32(float (&v)[32], int lane) {
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
}

// Y[3i+a][k] = sum_j sum_b Ap[i][sym(a,b)][j] W[b][k][j] + gamma_k Y; a warp owns two rows i,
// a lane two columns of each 64-column block; every 960 columns the 24 FP32 sums of a
// row are reduce-scattered over the warp into one FP64 running sum per lane.
__device__ __forceinline__ void avp_tile(const CUtensorMap* tmA, const CUtensorMap* tmW, int ne, int ldp,
                                         const LsqrScalars* sc, double* __restrict__ Y, float* __restrict__ Ys,
                                         double* __restrict__ part, int* errflag, int blk) {
  constexpr int FLUSH = 1024 / AVP_BC;  // stages per FP64 flush
  extern __shared__ __align__(1024) unsigned char avp_smem[];
  float* sA = reinterpret_cast<float*>(avp_smem);
  float* sW = reinterpret_cast<float*>(avp_smem + AVP_ST * AVP_STAGE_A);
  __shared__ __align__(8) uint64_t full[AVP_ST], empty[AVP_ST];
  __shared__ double sPart[AVP_WARPS][K8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row_base = blk * AVP_R;
  constexpr int nwarps = AVP_WARPS;
  constexpr uint32_t stage_bytes = (uint32_t)(AVP_STAGE_A + AVP_STAGE_W);
  const int nst = (ldp + AVP_BC - 1) / AVP_BC;
  if (threadIdx.x == 0) {
    for (int s = 0; s < AVP_ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], nwarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int k) {
    const int s = k % AVP_ST;
    if (k >= AVP_ST) mbar_wait_bounded(&empty[s], (uint32_t)(((k / AVP_ST) - 1) & 1), errflag);
    const int j0 = k * AVP_BC;
    mbar_expect_tx(&full[s], stage_bytes);
    // one 3-D box: 16 rows x (3 column blocks x 6 planes x 64 columns), 4.5 KB contiguous per row
    tma_load_3d(sA + (size_t)s * 6 * AVP_R * AVP_BC, tmA, 0, 6 * AVP_NB * k, row_base, &full[s]);
    tma_load_2d(sW + (size_t)s * 3 * K8 * AVP_BC, tmW, j0, 0, &full[s]);
  };
  // warp nwarps is the producer: it only issues the stages (waiting for their
  // slots to be released), so no compute warp ever blocks on a refill
  double ssq = 0.0;
  if (warp == nwarps) {
    if (lane == 0) {
      for (int k = 0; k < nst; ++k) issue(k);
      mbar_drain(full, AVP_ST, nst, errflag);
    }
    __syncwarp();
  } else {
  float acc[2][3][K8];
  double dacc[2] = {0.0, 0.0};
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < K8; ++c) acc[r][a][c] = 0.f;
  for (int k = 0; k < nst; ++k) {
    const int s = k % AVP_ST;
    mbar_wait_bounded(&full[s], (uint32_t)((k / AVP_ST) & 1), errflag);
#pragma unroll
    for (int h = 0; h < AVP_NB; ++h) {
      // [row][column block][c][64]
      const float* tA = sA + (size_t)s * 6 * AVP_R * AVP_BC + (2 * warp) * 6 * AVP_BC + h * 384 + lane * 2;
      const float* tW = sW + (size_t)s * 3 * K8 * AVP_BC + h * 64 + lane * 2;
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        float2 w[K8];
#pragma unroll
        for (int c = 0; c < K8; ++c) w[c] = *reinterpret_cast<const float2*>(tW + (size_t)(b * K8 + c) * AVP_BC);
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float2 g = *reinterpret_cast<const float2*>(tA + r * 6 * AVP_BC + sym6(a, b) * 64);
#pragma unroll
            for (int c = 0; c < K8; ++c) acc[r][a][c] = fmaf(g.y, w[c].y, fmaf(g.x, w[c].x, acc[r][a][c]));
          }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    if ((k % FLUSH) == FLUSH - 1 || k == nst - 1) {
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        float v[32];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int c = 0; c < K8; ++c) { v[a * K8 + c] = acc[r][a][c]; acc[r][a][c] = 0.f; }
#pragma unroll
        for (int t = 24; t < 32; ++t) v[t] = 0.f;
        reduce_scatter32(v, lane);
        dacc[r] += (double)v[0];
      }
    }
  }
  // lane a*8+c holds row 3i+a, right-hand side c of each of the warp's two rows
  if (lane < 3 * K8) {
    const int a = lane / K8, c = lane % K8;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int i = row_base + 2 * warp + r;
      if (i < ne) {
        const int64_t id = (int64_t)(3 * i + a) * K8 + c;
        const double y = dacc[r] + sc[c].gamma * Y[id];
        Y[id] = y;
        Ys[id] = (float)y;
        ssq += y * y;
      }
    }
  }
  // per-c partial sums: lanes c, c+8, c+16
  ssq += __shfl_down_sync(0xffffffffu, ssq, 8);
  ssq += __shfl_down_sync(0xffffffffu, ssq, 16);
  if (lane < K8) sPart[warp][lane] = ssq;
  }
  __syncthreads();
  if (threadIdx.x < K8) {
    double t = 0.0;
    for (int w = 0; w < nwarps; ++w) t += sPart[w][threadIdx.x];
    part[(int64_t)blk * K8 + threadIdx.x] = t;
  }
}

// Zp[g][b ne + j][k] = sum_{i in group g} sum_a Ap[i][sym(a,b)][j] U[3i+a][k]; one thread per column j.
constexpr int ATUP_C = 256, ATUP_RS = 8, ATUP_ST = 2;  // 97.5 KB: two CTAs (16 warps) per SM
constexpr size_t ATUP_STAGE_A = 6 * (size_t)ATUP_RS * ATUP_C * sizeof(float);  // 48 KB
constexpr size_t ATUP_STAGE_U = 3 * (size_t)ATUP_RS * K8 * sizeof(float);      // 768 B
constexpr size_t ATUP_SMEM = ATUP_ST * (ATUP_STAGE_A + ATUP_STAGE_U);

__device__ __forceinline__ void atup_tile(const CUtensorMap* tmA, int ne, int64_t lda, const float* __restrict__ Us,
                                          int rows_per_group, double* __restrict__ Zp, int* errflag, int cblk, int g) {
  extern __shared__ __align__(1024) unsigned char atup_smem[];
  float* sA = reinterpret_cast<float*>(atup_smem);
  float* sU = reinterpret_cast<float*>(atup_smem + ATUP_ST * ATUP_STAGE_A);
  __shared__ __align__(8) uint64_t full[ATUP_ST], empty[ATUP_ST];
  const int j0 = cblk * ATUP_C;
  const int r0 = g * rows_per_group, r1 = min(ne, r0 + rows_per_group);
  const int nst = (r1 > r0) ? (r1 - r0 + ATUP_RS - 1) / ATUP_RS : 0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ATUP_ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], ATUP_C / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int k) {
    const int s = k % ATUP_ST;
    if (k >= ATUP_ST) mbar_wait_bounded(&empty[s], (uint32_t)(((k / ATUP_ST) - 1) & 1), errflag);
    const int rb = r0 + k * ATUP_RS;
    const int nr = min(ATUP_RS, r1 - rb);
    mbar_expect_tx(&full[s], (uint32_t)(ATUP_STAGE_A + (size_t)3 * nr * K8 * sizeof(float)));
    // one 3-D box: 8 rows x (4 column blocks x 6 planes x 64 columns), 6 KB contiguous per row
    tma_load_3d(sA + (size_t)s * 6 * ATUP_RS * ATUP_C, tmA, 0, 6 * (j0 / 64), rb, &full[s]);
    bulk_g2s(sU + (size_t)s * 3 * ATUP_RS * K8, Us + (int64_t)3 * rb * K8, (uint32_t)(3 * nr * K8 * sizeof(float)),
             &full[s]);
  };
  if (threadIdx.x == 0)
    for (int k = 0; k < ATUP_ST && k < nst; ++k) issue(k);
  float acc[3][K8];
  double dacc[3][K8];
#pragma unroll
  for (int b = 0; b < 3; ++b)
#pragma unroll
    for (int c = 0; c < K8; ++c) { acc[b][c] = 0.f; dacc[b][c] = 0.0; }
  for (int k = 0; k < nst; ++k) {
    const int s = k % ATUP_ST;
    mbar_wait_bounded(&full[s], (uint32_t)((k / ATUP_ST) & 1), errflag);
    const int rb = r0 + k * ATUP_RS;
    const int nr = min(ATUP_RS, r1 - rb);
    // [row][column block][c][64]: the thread's column is (t / 64, t % 64)
    const float* tA = sA + (size_t)s * 6 * ATUP_RS * ATUP_C + (threadIdx.x >> 6) * 384 + (threadIdx.x & 63);
    const float* tU = sU + (size_t)s * 3 * ATUP_RS * K8;
    for (int r = 0; r < nr; ++r) {
      float g6[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) g6[c] = tA[r * 6 * ATUP_C + c * 64];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float4 u0 = *reinterpret_cast<const float4*>(tU + (3 * r + a) * K8);
        const float4 u1 = *reinterpret_cast<const float4*>(tU + (3 * r + a) * K8 + 4);
        const float uu[K8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const float gv = g6[sym6(a, b)];
#pragma unroll
          for (int c = 0; c < K8; ++c) acc[b][c] = fmaf(gv, uu[c], acc[b][c]);
        }
      }
    }
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[s]);
    if (threadIdx.x == 0 && k + ATUP_ST < nst) issue(k + ATUP_ST);
    if ((k & 31) == 31 || k == nst - 1) {
#pragma unroll
      for (int b = 0; b < 3; ++b)
#pragma unroll
        for (int c = 0; c < K8; ++c) { dacc[b][c] += (double)acc[b][c]; acc[b][c] = 0.f; }
    }
  }
  if (threadIdx.x == 0) mbar_drain(full, ATUP_ST, nst, errflag);
  const int j = j0 + threadIdx.x;
  if (j < ne)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = 0; c < K8; ++c) Zp[((int64_t)g * lda + (int64_t)b * ne + j) * K8 + c] = dacc[b][c];
}

}  // namespace agb
