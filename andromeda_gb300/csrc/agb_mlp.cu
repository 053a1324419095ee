// MLP surrogate of the resistance tensor: 5 -> 256 -> 256 -> 256 -> 21 with
// SiLU, FP32 master weights, BF16 tensor-core GEMMs (mma.sync m16n8k16, FP32
// accumulation), hand-written forward, backward, Adam and inference.
//
// Every layer product is one GEMM C[M][N] = sum_k A(m,k) B(n,k) whose operands
// are read from FP32 global memory in either orientation (so the backward
// products dH = dZ W and dW = dZ^T H need no transposed copies), converted to
// BF16 while the 128 x 64 x 32 tile is staged in shared memory, and multiplied
// by 8 warps (32 x 32 each).  The epilogue is fused: bias + SiLU (storing the
// pre-activation for the backward pass), bias only, plain store, or the SiLU
// derivative.  Optional split-BF16 mode (x = hi + lo, three products
// hi*hi + hi*lo + lo*hi) gives FP32-level accuracy on the same tensor cores;
// inference uses it.
#include "agb_mlp.cuh"

#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

namespace agb {

enum { EPI_STORE = 0, EPI_BIAS_SILU = 1, EPI_BIAS = 2, EPI_DSILU = 3 };

struct GemmEpi {
  float* C;          // [M][N]
  const float* bias; // [N] (EPI_BIAS*)
  float* Z;          // EPI_BIAS_SILU: pre-activation out [M][N]
  const float* Zin;  // EPI_DSILU: pre-activation in [M][N]
};

constexpr int GBM = 128, GBN = 64, GBK = 32, GPAD = 8;

// fast exponential and division (__expf, __fdividef: a few ulp; exp(-z) = inf
// for z < -88 gives z * 0 = -0, the limit of SiLU) -- the activations are
// BF16-split downstream, and the same functions serve training and inference
__device__ __forceinline__ float silu_f(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = __fdividef(1.0f, 1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t smem_u32_mlp(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// not volatile: the only effect is the accumulator update, so the compiler may
// interleave independent products (the three split products of one
// accumulator stay in order through their data dependence)
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A(m,k) = A_K ? A[m*lda + k] : A[k*lda + m];  B(n,k) = B_K ? B[n*ldb + k] : B[k*ldb + n]
template <bool A_K, bool B_K, bool SPLIT, int EPI>
__global__ void __launch_bounds__(256) k_mlp_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                                  const float* __restrict__ B, int ldb, GemmEpi e) {
  __shared__ __align__(16) __nv_bfloat16 As[2][GBM][GBK + GPAD];
  __shared__ __align__(16) __nv_bfloat16 Bs[2][GBN][GBK + GPAD];
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = warp & 3, wn = warp >> 2;
  const int gid = lane >> 2, tig = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  for (int k0 = 0; k0 < K; k0 += GBK) {
    // stage A (128 x 32) and B (64 x 32) as BF16 (hi, and lo = x - hi in split mode)
#pragma unroll 4
    for (int t = threadIdx.x; t < GBM * GBK; t += 256) {
      int m, k;
      if (A_K) { m = t / GBK; k = t % GBK; } else { m = t % GBM; k = t / GBM; }
      const int gm = m0 + m, gk = k0 + k;
      float v = 0.f;
      if (gm < M && gk < K) v = A_K ? A[(int64_t)gm * lda + gk] : A[(int64_t)gk * lda + gm];
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      As[0][m][k] = hi;
      if (SPLIT) As[1][m][k] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
#pragma unroll 4
    for (int t = threadIdx.x; t < GBN * GBK; t += 256) {
      int n, k;
      if (B_K) { n = t / GBK; k = t % GBK; } else { n = t % GBN; k = t / GBN; }
      const int gn = n0 + n, gk = k0 + k;
      float v = 0.f;
      if (gn < N && gk < K) v = B_K ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      Bs[0][n][k] = hi;
      if (SPLIT) Bs[1][n][k] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < GBK; ks += 16) {
      uint32_t af[2][2][4], bf[2][4][2];  // [hi/lo][tile][reg]
#pragma unroll
      for (int p = 0; p < (SPLIT ? 2 : 1); ++p) {
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
          const int r = wm * 32 + mi * 16 + gid;
          af[p][mi][0] = *reinterpret_cast<const uint32_t*>(&As[p][r][ks + tig * 2]);
          af[p][mi][1] = *reinterpret_cast<const uint32_t*>(&As[p][r + 8][ks + tig * 2]);
          af[p][mi][2] = *reinterpret_cast<const uint32_t*>(&As[p][r][ks + 8 + tig * 2]);
          af[p][mi][3] = *reinterpret_cast<const uint32_t*>(&As[p][r + 8][ks + 8 + tig * 2]);
        }
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
          const int c = wn * 32 + ni * 8 + gid;
          bf[p][ni][0] = *reinterpret_cast<const uint32_t*>(&Bs[p][c][ks + tig * 2]);
          bf[p][ni][1] = *reinterpret_cast<const uint32_t*>(&Bs[p][c][ks + 8 + tig * 2]);
        }
      }
#pragma unroll
      for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
          mma_bf16(acc[mi][ni], af[0][mi], bf[0][ni]);
          if (SPLIT) {
            mma_bf16(acc[mi][ni], af[0][mi], bf[1][ni]);
            mma_bf16(acc[mi][ni], af[1][mi], bf[0][ni]);
          }
        }
    }
    __syncthreads();
  }
  // fused epilogue
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm * 32 + mi * 16 + gid + ((r >= 2) ? 8 : 0);
        const int n = n0 + wn * 32 + ni * 8 + tig * 2 + (r & 1);
        if (m >= M || n >= N) continue;
        const int64_t o = (int64_t)m * N + n;
        float v = acc[mi][ni][r];
        if (EPI == EPI_STORE) {
          e.C[o] = v;
        } else if (EPI == EPI_BIAS_SILU) {
          v += e.bias[n];
          if (e.Z) e.Z[o] = v;
          e.C[o] = silu_f(v);
        } else if (EPI == EPI_BIAS) {
          e.C[o] = v + e.bias[n];
        } else {
          e.C[o] = v * dsilu_f(e.Zin[o]);
        }
      }
}

// Xn = (X - xm) / xs
__global__ void k_mlp_norm_in(int n, int nin, const float* __restrict__ X, const float* __restrict__ xm,
                              const float* __restrict__ xs, float* __restrict__ Xn) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nin) return;
  const int j = (int)(t % nin);
  Xn[t] = (X[t] - xm[j]) / xs[j];
}
// Y = Yn * ys + ym
__global__ void k_mlp_denorm_out(int n, int nout, const float* __restrict__ Yn, const float* __restrict__ ym,
                                 const float* __restrict__ ys, float* __restrict__ Y) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nout) return;
  const int j = (int)(t % nout);
  Y[t] = Yn[t] * ys[j] + ym[j];
}
// dY = 2 (Y - (T - ym)/ys) / (n * nout); per-block partial sums of the squared error
__global__ void k_mlp_loss(int n, int nout, const float* __restrict__ Y, const float* __restrict__ T,
                           const float* __restrict__ ym, const float* __restrict__ ys, float* __restrict__ dY,
                           double* __restrict__ part) {
  __shared__ double sh[256];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double se = 0.0;
  if (t < (int64_t)n * nout) {
    const int j = (int)(t % nout);
    const float d = Y[t] - (T[t] - ym[j]) / ys[j];
    dY[t] = 2.0f * d / (float)((int64_t)n * nout);
    se = (double)d * d;
  }
  sh[threadIdx.x] = se;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
// db[j] = sum_rows dZ[row][j]
__global__ void k_mlp_colsum(int n, int ncol, const float* __restrict__ dZ, float* __restrict__ db) {
  const int j = blockIdx.x;
  __shared__ float sh[256];
  float s = 0.f;
  for (int r = threadIdx.x; r < n; r += blockDim.x) s += dZ[(int64_t)r * ncol + j];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[j] = sh[0];
}
// Adam (Kingma & Ba), FP32 master weights
__global__ void k_mlp_adam(int64_t np, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const float gi = g[t];
  const float mi = b1 * m[t] + (1.f - b1) * gi;
  const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
  m[t] = mi;
  v[t] = vi;
  w[t] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

static inline unsigned cdv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

template <bool A_K, bool B_K, int EPI>
static void gemm(bool split, int M, int N, int K, const float* A, int lda, const float* B, int ldb, GemmEpi e,
                 cudaStream_t s) {
  dim3 g(cdv(N, GBN), cdv(M, GBM));
  if (split) k_mlp_gemm<A_K, B_K, true, EPI><<<g, 256, 0, s>>>(M, N, K, A, lda, B, ldb, e);
  else k_mlp_gemm<A_K, B_K, false, EPI><<<g, 256, 0, s>>>(M, N, K, A, lda, B, ldb, e);
}

// ---------------------------------------------------------------------------
// Fused inference (split-BF16): one CTA runs 128 queries through all four
// layers.  The activations stay in shared memory as BF16 hi/lo pairs
// ([128][256+8] each); 16 warps: two warps share 16 query rows, each owning
// half of a layer's output columns (16 n-tiles x 4 FP32 accumulators per
// lane); a block barrier separates the last reads of a layer's input rows from
// the writes of its outputs into the same rows.  The weights, pre-split into
// BF16 hi/lo ([layer][hi/lo][N][K], k contiguous), stream
// through two 40 KB shared-memory buffers in chunks of 32 k (cp.async, all
// threads).  Input normalisation and output de-normalisation are fused.  The
// accumulation order (k16 steps in order; hi*hi, hi*lo, lo*hi per step) and
// the FP32 epilogues are those of k_mlp_gemm, so the outputs equal the
// unfused forward's.
// ---------------------------------------------------------------------------
constexpr int FI_M = 128, FI_H = 256, FI_HP = FI_H + 8, FI_KC = 32, FI_WP = FI_KC + 8;
constexpr int FI_NIN = 16, FI_NOUT = 32;  // padded K of layer 1, padded N of layer 4
constexpr size_t FI_SMEM_H = 2ull * FI_M * FI_HP * sizeof(__nv_bfloat16);         // 132 KB
constexpr size_t FI_SMEM_W = 2ull * 2 * FI_H * FI_WP * sizeof(__nv_bfloat16);     // 80 KB
constexpr size_t FI_SMEM = FI_SMEM_H + FI_SMEM_W;
// packed weight offsets (elements): L1 [2][256][16], L2 [2][256][256], L3 [2][256][256], L4 [2][32][256]
constexpr int64_t FI_O1 = 0, FI_O2 = FI_O1 + 2 * FI_H * FI_NIN, FI_O3 = FI_O2 + 2 * FI_H * FI_H,
                  FI_O4 = FI_O3 + 2 * FI_H * FI_H, FI_WTOT = FI_O4 + 2 * FI_NOUT * FI_H;
constexpr int FI_CHUNKS = 1 + 3 * (FI_H / FI_KC);  // layer 1: one chunk of 16 k; layers 2-4: 8 each

__global__ void k_mlp_pack_infer(const float* __restrict__ P, int nin, int nh, int nout, int64_t o0, int64_t o2,
                                 int64_t o4, int64_t o6, __nv_bfloat16* __restrict__ wb) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= FI_WTOT) return;
  int64_t r;
  int K, N, k, n, hl;
  const float* W;
  int kin, nreal;
  if (t < FI_O2) { r = t - FI_O1; K = FI_NIN; N = FI_H; W = P + o0; kin = nin; nreal = nh; }
  else if (t < FI_O3) { r = t - FI_O2; K = FI_H; N = FI_H; W = P + o2; kin = nh; nreal = nh; }
  else if (t < FI_O4) { r = t - FI_O3; K = FI_H; N = FI_H; W = P + o4; kin = nh; nreal = nh; }
  else { r = t - FI_O4; K = FI_H; N = FI_NOUT; W = P + o6; kin = nh; nreal = nout; }
  hl = (int)(r / ((int64_t)N * K));
  const int64_t q = r % ((int64_t)N * K);
  n = (int)(q / K);
  k = (int)(q % K);
  const float v = (n < nreal && k < kin) ? W[(int64_t)n * kin + k] : 0.f;
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  wb[t] = hl == 0 ? hi : __float2bfloat16_rn(v - __bfloat162float(hi));
}

// four 8x8 BF16 matrices from shared memory (lane l gives the address of row l%8 of matrix l/8)
__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32_mlp(p)));
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32_mlp(dst)), "l"(src) : "memory");
}

// stage chunk c of the packed weights into buffer `buf` ([2 hl][256][FI_WP])
__device__ __forceinline__ void fi_stage(const __nv_bfloat16* __restrict__ wb, __nv_bfloat16* Ws, int c) {
  int64_t base;
  int N, K, k0, kw;
  if (c == 0) { base = FI_O1; N = FI_H; K = FI_NIN; k0 = 0; kw = FI_NIN; }
  else {
    const int l = (c - 1) / (FI_H / FI_KC);  // 0: layer 2, 1: layer 3, 2: layer 4
    base = l == 0 ? FI_O2 : l == 1 ? FI_O3 : FI_O4;
    N = l == 2 ? FI_NOUT : FI_H;
    K = FI_H;
    k0 = ((c - 1) % (FI_H / FI_KC)) * FI_KC;
    kw = FI_KC;
  }
  const int per_row = kw / 8;  // 16-byte pieces per row
  const int total = 2 * N * per_row;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int hl = i / (N * per_row);
    const int rem = i % (N * per_row);
    const int n = rem / per_row, pc = rem % per_row;
    cp_async16(Ws + ((size_t)hl * FI_H + n) * FI_WP + pc * 8, wb + base + ((int64_t)hl * N + n) * K + k0 + pc * 8);
  }
}

// one chunk of KS k16 steps for NT n-tiles (B rows nbase*8 ...): A = the warp's 16 rows of H
// (cols kH ...), B = the staged chunk; three passes (hi*hi, hi*lo, lo*hi) so
// that consecutive products go to different accumulators (NT even)
template <int NT, int KS>
__device__ __forceinline__ void fi_chunk(float (&acc)[16][4], const __nv_bfloat16* Hh, const __nv_bfloat16* Hl,
                                         int kH, const __nv_bfloat16* Wh, const __nv_bfloat16* Wl, int nbase, int gid,
                                         int tig) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int ks = 0; ks < KS; ++ks) {
    // A fragments by ldmatrix.x4: matrices (rows 0-7, k 0-7), (rows 8-15, k 0-7),
    // (rows 0-7, k 8-15), (rows 8-15, k 8-15) of the warp's 16 rows
    uint32_t ah[4], al[4];
    {
      const int arow = (lane & 7) + 8 * ((lane >> 3) & 1);
      const int acol = kH + ks * 16 + 8 * (lane >> 4);
      ldsm_x4(ah[0], ah[1], ah[2], ah[3], Hh + arow * FI_HP + acol);
      ldsm_x4(al[0], al[1], al[2], al[3], Hl + arow * FI_HP + acol);
    }
    // B fragments of two n-tiles per ldmatrix.x4: matrices (nt, k 0-7), (nt, k 8-15),
    // (nt+1, k 0-7), (nt+1, k 8-15); lane l addresses row l%8 of matrix l/8
    const int lr = lane & 7, lm = lane >> 3;
    const int koff = ks * 16 + (lm & 1) * 8;
    const int nrow = (nbase + (lm >> 1)) * 8 + lr;
#pragma unroll
    for (int nt = 0; nt < NT; nt += 2) {
      uint32_t b0[2], b1[2];
      ldsm_x4(b0[0], b0[1], b1[0], b1[1], Wh + (nrow + nt * 8) * FI_WP + koff);
      mma_bf16(acc[nt], ah, b0);
      mma_bf16(acc[nt + 1], ah, b1);
    }
#pragma unroll
    for (int nt = 0; nt < NT; nt += 2) {
      uint32_t b0[2], b1[2];
      ldsm_x4(b0[0], b0[1], b1[0], b1[1], Wl + (nrow + nt * 8) * FI_WP + koff);
      mma_bf16(acc[nt], ah, b0);
      mma_bf16(acc[nt + 1], ah, b1);
    }
#pragma unroll
    for (int nt = 0; nt < NT; nt += 2) {
      uint32_t b0[2], b1[2];
      ldsm_x4(b0[0], b0[1], b1[0], b1[1], Wh + (nrow + nt * 8) * FI_WP + koff);
      mma_bf16(acc[nt], al, b0);
      mma_bf16(acc[nt + 1], al, b1);
    }
  }
}

// 16 warps: warp w owns query rows 16*(w/2) ... and output columns
// 128*(w%2) ... of layers 1-3 (16 n-tiles), 16*(w%2) ... of layer 4 (2 n-tiles)
constexpr int FI_THREADS = 512;
__global__ void __launch_bounds__(FI_THREADS, 1) k_mlp_infer(int n, int nin, int nout, const float* __restrict__ X,
                                                             const float* __restrict__ P, int64_t ob1, int64_t ob2,
                                                             int64_t ob3, int64_t ob4, const float* __restrict__ norm,
                                                             const __nv_bfloat16* __restrict__ wb,
                                                             float* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char fi_smem[];
  __nv_bfloat16* H = reinterpret_cast<__nv_bfloat16*>(fi_smem);                // [2 hl][128][FI_HP]
  __nv_bfloat16* Wb = reinterpret_cast<__nv_bfloat16*>(fi_smem + FI_SMEM_H);   // [2 buf][2 hl][256][FI_WP]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int rg = warp >> 1, ch = warp & 1;         // row group, column half
  const int row0 = blockIdx.x * FI_M + rg * 16;    // the warp's first query
  __nv_bfloat16* Hh = H + (size_t)(rg * 16) * FI_HP;
  __nv_bfloat16* Hl = H + (size_t)(FI_M + rg * 16) * FI_HP;
  const float* xm = norm;
  const float* xs = norm + nin;
  const float* ym = norm + 2 * nin;
  const float* ys = norm + 2 * nin + nout;
  fi_stage(wb, Wb, 0);
  asm volatile("cp.async.commit_group;" ::: "memory");
  // normalised inputs of the row group's 16 queries into H columns 0..15
  if (ch == 0)
    for (int i = lane; i < 16 * FI_NIN; i += 32) {
      const int r = i / FI_NIN, k = i % FI_NIN;
      const int g = row0 + r;
      float v = 0.f;
      if (k < nin && g < n) v = (X[(int64_t)g * nin + k] - xm[k]) / xs[k];
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      Hh[r * FI_HP + k] = hi;
      Hl[r * FI_HP + k] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
  float acc[16][4];
#pragma unroll
  for (int nt = 0; nt < 16; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
  for (int c = 0; c < FI_CHUNKS; ++c) {
    if (c + 1 < FI_CHUNKS) {
      fi_stage(wb, Wb + (size_t)((c + 1) & 1) * 2 * FI_H * FI_WP, c + 1);
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();  // chunk c staged; the previous layer's outputs (or the inputs) written
    const __nv_bfloat16* Wh = Wb + (size_t)(c & 1) * 2 * FI_H * FI_WP;
    const __nv_bfloat16* Wl = Wh + (size_t)FI_H * FI_WP;
    const int layer = c == 0 ? 1 : 2 + (c - 1) / (FI_H / FI_KC);
    const int kH = c == 0 ? 0 : ((c - 1) % (FI_H / FI_KC)) * FI_KC;
    const bool last = c == 0 || ((c - 1) % (FI_H / FI_KC)) == FI_H / FI_KC - 1;
    if (layer == 1) fi_chunk<16, 1>(acc, Hh, Hl, kH, Wh, Wl, 16 * ch, gid, tig);
    else if (layer < 4) fi_chunk<16, 2>(acc, Hh, Hl, kH, Wh, Wl, 16 * ch, gid, tig);
    else fi_chunk<FI_NOUT / 16, 2>(acc, Hh, Hl, kH, Wh, Wl, (FI_NOUT / 16) * ch, gid, tig);
    if (last && layer < 4) {
      __syncthreads();  // both warps of a row group have read all of its input columns
      // bias + SiLU, split into hi/lo
      const float* bias = P + (layer == 1 ? ob1 : layer == 2 ? ob2 : ob3);
#pragma unroll
      for (int nt = 0; nt < 16; ++nt) {
        const int col = (16 * ch + nt) * 8 + tig * 2;
        const float b0 = bias[col], b1 = bias[col + 1];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float v0 = silu_f(acc[nt][2 * h] + b0), v1 = silu_f(acc[nt][2 * h + 1] + b1);
          const __nv_bfloat16 h0 = __float2bfloat16_rn(v0), h1 = __float2bfloat16_rn(v1);
          __nv_bfloat162 hh, ll;
          hh.x = h0; hh.y = h1;
          ll.x = __float2bfloat16_rn(v0 - __bfloat162float(h0));
          ll.y = __float2bfloat16_rn(v1 - __bfloat162float(h1));
          const int r = gid + 8 * h;
          *reinterpret_cast<__nv_bfloat162*>(Hh + r * FI_HP + col) = hh;
          *reinterpret_cast<__nv_bfloat162*>(Hl + r * FI_HP + col) = ll;
          acc[nt][2 * h] = 0.f;
          acc[nt][2 * h + 1] = 0.f;
        }
      }
    } else if (last) {
      // bias, de-normalisation, store
      const float* bias = P + ob4;
#pragma unroll
      for (int nt = 0; nt < FI_NOUT / 16; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int col = ((FI_NOUT / 16) * ch + nt) * 8 + tig * 2 + (q & 1);
          const int g = row0 + gid + ((q >= 2) ? 8 : 0);
          if (col < nout && g < n) {
            const float v = acc[nt][q] + bias[col];
            Y[(int64_t)g * nout + col] = v * ys[col] + ym[col];
          }
        }
    }
    __syncthreads();  // the buffer of chunk c is refilled by the stage of chunk c + 2
  }
}

// ---------------------------------------------------------------------------
// Host object
// ---------------------------------------------------------------------------
Mlp::~Mlp() { release(); }

void Mlp::release() {
  cudaFree(params); cudaFree(grads); cudaFree(adam_m); cudaFree(adam_v); cudaFree(norm); cudaFree(ws);
  cudaFree(part);
  cudaFree(wb);
  params = grads = adam_m = adam_v = norm = ws = nullptr;
  part = nullptr;
  wb = nullptr;
  ws_rows = 0;
}

int64_t Mlp::nparams() const { return (int64_t)nh * nin + nh + 2 * ((int64_t)nh * nh + nh) + (int64_t)nout * nh + nout; }

void Mlp::offsets(int64_t o[8]) const {
  o[0] = 0;                                 // W1 [nh][nin]
  o[1] = o[0] + (int64_t)nh * nin;          // b1
  o[2] = o[1] + nh;                         // W2 [nh][nh]
  o[3] = o[2] + (int64_t)nh * nh;           // b2
  o[4] = o[3] + nh;                         // W3
  o[5] = o[4] + (int64_t)nh * nh;           // b3
  o[6] = o[5] + nh;                         // W4 [nout][nh]
  o[7] = o[6] + (int64_t)nout * nh;         // b4
}

bool Mlp::init(int dev, uint64_t seed, cudaStream_t st) {
  device = dev;
  s = st;
  const int64_t P = nparams();
  if (cudaMalloc(&params, P * sizeof(float)) != cudaSuccess || cudaMalloc(&grads, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&adam_m, P * sizeof(float)) != cudaSuccess || cudaMalloc(&adam_v, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&norm, 2 * (nin + nout) * sizeof(float)) != cudaSuccess) {
    err = "mlp: out of device memory";
    return false;
  }
  // He-uniform weights for SiLU layers, zero biases (host-side, seeded)
  std::vector<float> h(P, 0.f);
  std::mt19937_64 rng(seed);
  int64_t o[8];
  offsets(o);
  auto fill = [&](int64_t off, int fan_out, int fan_in) {
    const float lim = std::sqrt(6.0f / (float)fan_in);
    std::uniform_real_distribution<float> u(-lim, lim);
    for (int64_t i = 0; i < (int64_t)fan_out * fan_in; ++i) h[off + i] = u(rng);
  };
  fill(o[0], nh, nin);
  fill(o[2], nh, nh);
  fill(o[4], nh, nh);
  fill(o[6], nout, nh);
  for (int64_t i = o[6]; i < o[7]; ++i) h[i] *= 0.1f;
  if (cudaMemcpy(params, h.data(), P * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
    err = "mlp: upload";
    return false;
  }
  cudaMemset(adam_m, 0, P * sizeof(float));
  cudaMemset(adam_v, 0, P * sizeof(float));
  std::vector<float> nrm(2 * (nin + nout));
  for (int i = 0; i < nin; ++i) { nrm[i] = 0.f; nrm[nin + i] = 1.f; }
  for (int i = 0; i < nout; ++i) { nrm[2 * nin + i] = 0.f; nrm[2 * nin + nout + i] = 1.f; }
  cudaMemcpy(norm, nrm.data(), nrm.size() * sizeof(float), cudaMemcpyHostToDevice);
  step = 0;
  return cudaGetLastError() == cudaSuccess;
}

bool Mlp::ensure_ws(int rows) {
  if (rows <= ws_rows) return true;
  cudaFree(ws);
  cudaFree(part);
  ws = nullptr;
  part = nullptr;
  // Xn, Z1, H1, Z2, H2, Z3, H3, Y, dY, dA, dB
  const size_t per = (size_t)nin + 6 * (size_t)nh + 2 * (size_t)nout + 2 * (size_t)nh;
  if (cudaMalloc(&ws, per * rows * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&part, (size_t)cdv((int64_t)rows * nout, 256) * sizeof(double)) != cudaSuccess) {
    err = "mlp: workspace";
    ws_rows = 0;
    return false;
  }
  ws_rows = rows;
  return true;
}

// forward of `rows` normalised inputs Xn (already in the workspace); keeps the
// pre-activations when `train`
void Mlp::forward(int rows, bool train, bool split) {
  int64_t o[8];
  offsets(o);
  float* Xn = ws;
  float* Z1 = Xn + (size_t)ws_rows * nin;
  float* H1 = Z1 + (size_t)ws_rows * nh;
  float* Z2 = H1 + (size_t)ws_rows * nh;
  float* H2 = Z2 + (size_t)ws_rows * nh;
  float* Z3 = H2 + (size_t)ws_rows * nh;
  float* H3 = Z3 + (size_t)ws_rows * nh;
  float* Y = H3 + (size_t)ws_rows * nh;
  const float* P = params;
  gemm<true, true, EPI_BIAS_SILU>(split, rows, nh, nin, Xn, nin, P + o[0], nin, GemmEpi{H1, P + o[1], train ? Z1 : nullptr, nullptr}, s);
  gemm<true, true, EPI_BIAS_SILU>(split, rows, nh, nh, H1, nh, P + o[2], nh, GemmEpi{H2, P + o[3], train ? Z2 : nullptr, nullptr}, s);
  gemm<true, true, EPI_BIAS_SILU>(split, rows, nh, nh, H2, nh, P + o[4], nh, GemmEpi{H3, P + o[5], train ? Z3 : nullptr, nullptr}, s);
  gemm<true, true, EPI_BIAS>(split, rows, nout, nh, H3, nh, P + o[6], nh, GemmEpi{Y, P + o[7], nullptr, nullptr}, s);
  launches += 4;
}

// loss and gradients of one batch (targets T in physical units); loss to part
void Mlp::backward(int rows, const float* T, bool split) {
  int64_t o[8];
  offsets(o);
  float* Xn = ws;
  float* Z1 = Xn + (size_t)ws_rows * nin;
  float* H1 = Z1 + (size_t)ws_rows * nh;
  float* Z2 = H1 + (size_t)ws_rows * nh;
  float* H2 = Z2 + (size_t)ws_rows * nh;
  float* Z3 = H2 + (size_t)ws_rows * nh;
  float* H3 = Z3 + (size_t)ws_rows * nh;
  float* Y = H3 + (size_t)ws_rows * nh;
  float* dY = Y + (size_t)ws_rows * nout;
  float* dA = dY + (size_t)ws_rows * nout;
  float* dB = dA + (size_t)ws_rows * nh;
  const float* P = params;
  float* G = grads;
  const float* ym = norm + 2 * nin;
  const float* ys = norm + 2 * nin + nout;
  k_mlp_loss<<<cdv((int64_t)rows * nout, 256), 256, 0, s>>>(rows, nout, Y, T, ym, ys, dY, part);
  // layer 4
  gemm<false, false, EPI_STORE>(split, nout, nh, rows, dY, nout, H3, nh, GemmEpi{G + o[6], nullptr, nullptr, nullptr}, s);
  k_mlp_colsum<<<nout, 256, 0, s>>>(rows, nout, dY, G + o[7]);
  gemm<true, false, EPI_DSILU>(split, rows, nh, nout, dY, nout, P + o[6], nh, GemmEpi{dA, nullptr, nullptr, Z3}, s);
  // layer 3 (dA = dZ3)
  gemm<false, false, EPI_STORE>(split, nh, nh, rows, dA, nh, H2, nh, GemmEpi{G + o[4], nullptr, nullptr, nullptr}, s);
  k_mlp_colsum<<<nh, 256, 0, s>>>(rows, nh, dA, G + o[5]);
  gemm<true, false, EPI_DSILU>(split, rows, nh, nh, dA, nh, P + o[4], nh, GemmEpi{dB, nullptr, nullptr, Z2}, s);
  // layer 2 (dB = dZ2)
  gemm<false, false, EPI_STORE>(split, nh, nh, rows, dB, nh, H1, nh, GemmEpi{G + o[2], nullptr, nullptr, nullptr}, s);
  k_mlp_colsum<<<nh, 256, 0, s>>>(rows, nh, dB, G + o[3]);
  gemm<true, false, EPI_DSILU>(split, rows, nh, nh, dB, nh, P + o[2], nh, GemmEpi{dA, nullptr, nullptr, Z1}, s);
  // layer 1 (dA = dZ1)
  gemm<false, false, EPI_STORE>(split, nh, nin, rows, dA, nh, Xn, nin, GemmEpi{G + o[0], nullptr, nullptr, nullptr}, s);
  k_mlp_colsum<<<nh, 256, 0, s>>>(rows, nh, dA, G + o[1]);
  launches += 13;
}

void Mlp::load_inputs(int rows, const float* X_dev) {
  k_mlp_norm_in<<<cdv((int64_t)rows * nin, 256), 256, 0, s>>>(rows, nin, X_dev, norm, norm + nin, ws);
  launches += 1;
}

void Mlp::adam(float lr) {
  ++step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  const int64_t P = nparams();
  k_mlp_adam<<<cdv(P, 256), 256, 0, s>>>(P, params, grads, adam_m, adam_v, lr, b1, b2, 1e-8f, c1, c2);
  launches += 1;
}

void Mlp::output(int rows, float* Y_dev) {
  float* Y = ws + (size_t)ws_rows * (nin + 6 * nh);
  k_mlp_denorm_out<<<cdv((int64_t)rows * nout, 256), 256, 0, s>>>(rows, nout, Y, norm + 2 * nin,
                                                                   norm + 2 * nin + nout, Y_dev);
  launches += 1;
}

bool Mlp::infer(int rows, const float* X_dev, float* Y_dev) {
  if (nh != FI_H || nin > FI_NIN || nout > FI_NOUT || nin < 1 || nout < 1) {
    err = "fused inference needs nh = 256, nin <= 16, nout <= 32";
    return false;
  }
  if (!wb && cudaMalloc(&wb, FI_WTOT * sizeof(__nv_bfloat16)) != cudaSuccess) {
    wb = nullptr;
    err = "mlp: inference weights";
    return false;
  }
  if (cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FI_SMEM) != cudaSuccess) {
    err = "mlp: fused inference shared memory";
    return false;
  }
  int64_t o[8];
  offsets(o);
  __nv_bfloat16* w = static_cast<__nv_bfloat16*>(wb);
  k_mlp_pack_infer<<<cdv(FI_WTOT, 256), 256, 0, s>>>(params, nin, nh, nout, o[0], o[2], o[4], o[6], w);
  if (rows > 0)
    k_mlp_infer<<<cdv(rows, FI_M), FI_THREADS, FI_SMEM, s>>>(rows, nin, nout, X_dev, params, o[1], o[3], o[5], o[7],
                                                            norm, w, Y_dev);
  launches += rows > 0 ? 2 : 1;
  if (cudaGetLastError() != cudaSuccess) {
    err = "mlp: fused inference launch";
    return false;
  }
  return true;
}

double Mlp::loss_sum(int rows) {
  const int nb = (int)cdv((int64_t)rows * nout, 256);
  std::vector<double> h(nb);
  cudaMemcpyAsync(h.data(), part, nb * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  double t = 0.0;
  for (double v : h) t += v;
  return t;
}

}  // namespace agb
