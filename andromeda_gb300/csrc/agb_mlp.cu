// MLP surrogate of the resistance tensor: 5 -> 256 -> 256 -> 256 -> 21 with
// SiLU, FP32 master weights, hand-written forward, backward, Adam and
// inference.  Training runs on BF16 tensor-core GEMMs (mma.sync m16n8k16, FP32
// accumulation; batches of 512 rows); inference of large query batches runs in
// one fused kernel on the 5th-generation tensor cores (tcgen05, accumulators
// in tensor memory; k_mlp_infer_tc below).
//
// Every layer product is one GEMM C[M][N] = sum_k A(m,k) B(n,k) whose operands
// are read from FP32 global memory in either orientation (so the backward
// products dH = dZ W and dW = dZ^T H need no transposed copies), converted to
// BF16 while the 128 x 64 x 32 tile is staged in shared memory, and multiplied
// by 8 warps (32 x 32 each).  The epilogue is fused: bias + SiLU (storing the
// pre-activation for the backward pass), bias only, plain store, or the SiLU
// derivative.  Optional split-BF16 mode (x = hi + lo, three products
// hi*hi + hi*lo + lo*hi) gives FP32-level accuracy on the same tensor cores.
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
// Fused inference on the 5th-generation tensor cores (tcgen05, split-BF16).
// One CTA runs 128 queries (the tcgen05 M) through the four layers:
//   * the activations live in shared memory as BF16 hi and lo halves, K-major
//     with the 128-byte swizzle (tc_hoff), 64 KB each;
//   * the weights, pre-split and pre-packed in the same layout chunk by chunk
//     (16 k per chunk, one tcgen05 K step; [layer chunk][hi/lo][n/8][k/8][8][8]),
//     stream from L2 through a five-slot ring of 16 KB slots, one bulk copy per
//     chunk (the copy warp); a slot is released by tcgen05.commit of the
//     products that read it.  Four chunks in flight hide the L2 latency behind
//     the products of the chunk in use;
//   * one thread of the issuing warp issues tcgen05.mma (M = 128, N = 256 or 32,
//     K = 16; the three split products hi*hi, hi*lo, lo*hi per chunk) into one
//     of two 128 x 256 FP32 accumulators in tensor memory (layer l into (l-1)&1);
//     the two chunks of a 32-column activation block wait only for that block,
//     so a layer's products follow the previous layer's epilogue block by block;
//   * 16 epilogue warps read the accumulator block by block, all of them on the
//     same 32-column block at a time (warp w: tensor-memory lanes 32 (w%4) ...,
//     columns 8 (w/4) ... of the block), the load of the next block in flight
//     while the current one is processed: bias, SiLU and the hi/lo split of the
//     next layer's activations; layer 4 adds the bias, de-normalises and stores.
// Every wait is bounded (error flag); the tensor memory is freed on every path.
// ---------------------------------------------------------------------------
constexpr int TC_M = 128, TC_H = 256, TC_NOUT = 32, TC_KC = 16, TC_AB = 32;
constexpr int TC_NSLOT = 5;                   // weight ring depth
constexpr int TC_EPI = 16;                    // epilogue warps: 4 per TMEM lane group, 8 columns of a block each
constexpr int TC_THREADS = (TC_EPI + 2) * 32;  // + 1 copy warp + 1 issuing warp
constexpr size_t TC_H_BYTES = (size_t)TC_M * TC_H * 2;             // one half (hi or lo) of the activations
constexpr size_t TC_SLOT = 2ull * TC_H * TC_KC * 2;                  // largest chunk: N 256 x K 16, hi + lo
// + 1 KB so that the activations can start on a 1024-byte boundary (the 128-byte
// swizzle repeats every 8 rows x 128 B)
constexpr size_t TC_SMEM = 2 * TC_H_BYTES + TC_NSLOT * TC_SLOT + 1024;  // 209 KB (+ 4 KB static)
// packed weights (bytes): layer 1 one chunk (N 256, K 16), layers 2-3 sixteen chunks (N 256, K 16),
// layer 4 sixteen chunks (N 32, K 16); hi then lo inside a chunk
constexpr int TC_LCH = TC_H / TC_KC;  // chunks of layers 2-4
constexpr int64_t TC_C1 = 2ll * TC_H * TC_KC * 2, TC_C23 = 2ll * TC_H * TC_KC * 2, TC_C4 = 2ll * TC_NOUT * TC_KC * 2;
constexpr int64_t TC_L2 = TC_C1, TC_L3 = TC_L2 + TC_LCH * TC_C23, TC_L4 = TC_L3 + TC_LCH * TC_C23,
                  TC_WBYTES = TC_L4 + TC_LCH * TC_C4;
constexpr int TC_CHUNKS = 1 + 3 * TC_LCH;

__device__ __forceinline__ int64_t tc_chunk_off(int c) {
  return c == 0 ? 0
         : c <= TC_LCH     ? TC_L2 + (c - 1) * TC_C23
         : c <= 2 * TC_LCH ? TC_L3 + (c - 1 - TC_LCH) * TC_C23
                           : TC_L4 + (c - 1 - 2 * TC_LCH) * TC_C4;
}
__device__ __forceinline__ int64_t tc_chunk_bytes(int c) { return c == 0 ? TC_C1 : c <= 2 * TC_LCH ? TC_C23 : TC_C4; }

// one packed element per thread: (layer, hi/lo, n, k) -> chunk, core matrix, row, column
__global__ void k_mlp_pack_tc(const float* __restrict__ P, int nin, int nh, int nout, int64_t o0, int64_t o2,
                              int64_t o4, int64_t o6, __nv_bfloat16* __restrict__ wt) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= TC_WBYTES / 2) return;
  const int64_t b = 2 * t;  // byte offset of the element
  int layer, c;
  int64_t cb;
  if (b < TC_L2) { layer = 1; c = 0; cb = b; }
  else if (b < TC_L3) { layer = 2; c = (int)((b - TC_L2) / TC_C23); cb = (b - TC_L2) % TC_C23; }
  else if (b < TC_L4) { layer = 3; c = (int)((b - TC_L3) / TC_C23); cb = (b - TC_L3) % TC_C23; }
  else { layer = 4; c = (int)((b - TC_L4) / TC_C4); cb = (b - TC_L4) % TC_C4; }
  const int N = layer == 4 ? TC_NOUT : TC_H;
  const int64_t half = (int64_t)N * TC_KC * 2;
  const int hl = (int)(cb / half);
  const int64_t e = (cb % half) / 2;  // element within the half: [n/8][k/8][8][8]
  const int core = (int)(e / 64), within = (int)(e % 64);
  const int ng = core / (TC_KC / 8), kc = core % (TC_KC / 8);
  const int n = ng * 8 + within / 8, k = c * TC_KC + kc * 8 + within % 8;
  const float* W = P + (layer == 1 ? o0 : layer == 2 ? o2 : layer == 3 ? o4 : o6);
  const int kin = layer == 1 ? nin : nh, nreal = layer == 4 ? nout : nh;
  const float v = (n < nreal && k < kin) ? W[(int64_t)n * kin + k] : 0.f;
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  wt[t] = hl == 0 ? hi : __float2bfloat16_rn(v - __bfloat162float(hi));
}

__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t sbo) {
  // no-swizzle K-major: start >> 4, leading byte offset (next core matrix along K) 128 B,
  // stride byte offset (next 8-row group) sbo, descriptor version 1 (bit 46)
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) |
         ((uint64_t)1 << 46);
}
__device__ __forceinline__ uint32_t tc_idesc(int n) {
  // D F32 (bit 4), A and B BF16 (bits 7, 10), K-major, N >> 3 at bit 17, M >> 4 at bit 24
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32_mlp(bar))
               : "memory");
}
__device__ __forceinline__ bool tc_wait_once(uint64_t* bar, uint32_t parity) {
  uint32_t ok = 0;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(ok)
               : "r"(smem_u32_mlp(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, int* errflag) {
  uint32_t ok = 0, tries = 0;
  while (true) {
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_u32_mlp(bar)), "r"(parity)
                 : "memory");
    if (ok) return true;
    if ((++tries & 1023u) == 0 && *(volatile int*)errflag) return false;
    if (tries > (1u << 22)) {
      atomicExch(errflag, 1);
      return false;
    }
  }
}
// 8 accumulator columns of this warp's 32 lanes: issue the load; tc_ld8_wait makes
// the registers valid (they are operands of the wait, so no use moves above it)
__device__ __forceinline__ void tc_ld8_issue(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tc_ld8_wait(uint32_t (&r)[8]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])
               :
               : "memory");
}
// byte offset of (row, k) in one BF16 half of the activations, K-major with the
// 128-byte swizzle: four column blocks of 64 k (16 KB each: 128 rows x 128 B),
// 8-row groups of 1 KB, and within a row the 16-byte chunk k/8 stored at chunk
// (k/8) xor (row % 8) -- the layout tcgen05 reads through a SWIZZLE_128B descriptor
__device__ __forceinline__ uint32_t tc_hoff(int row, int k) {
  return (uint32_t)((k >> 6) * (TC_M * 128) + (row >> 3) * 1024 + (row & 7) * 128 +
                    ((((k >> 3) & 7) ^ (row & 7)) << 4) + (k & 7) * 2);
}
// descriptor of the A operand at activation column k0 (a multiple of 16): the
// column block's start advanced by k0 % 64 elements inside the swizzle atom,
// stride 1 KB between 8-row groups, swizzle mode 2 (128 B) in bits 61-63
__device__ __forceinline__ uint64_t tc_adesc(uint32_t half, int k0) {
  const uint32_t addr = half + (uint32_t)((k0 >> 6) * (TC_M * 128) + (k0 & 63) * 2);
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// bias + SiLU of 8 accumulator values, split into BF16 hi and lo, stored as one
// 16-byte core-matrix row each
__device__ __forceinline__ void tc_act8(const uint32_t (&r)[8], const float* bias, unsigned char* hh, unsigned char* hl) {
  __align__(16) __nv_bfloat162 hv[4], lv[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float z0 = silu_f(__uint_as_float(r[2 * j]) + bias[2 * j]);
    const float z1 = silu_f(__uint_as_float(r[2 * j + 1]) + bias[2 * j + 1]);
    hv[j] = __floats2bfloat162_rn(z0, z1);
    const float2 h = __bfloat1622float2(hv[j]);
    lv[j] = __floats2bfloat162_rn(z0 - h.x, z1 - h.y);
  }
  *reinterpret_cast<uint4*>(hh) = *reinterpret_cast<const uint4*>(hv);
  *reinterpret_cast<uint4*>(hl) = *reinterpret_cast<const uint4*>(lv);
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_infer_tc(int n, int nin, int nout, const float* __restrict__ X,
                                                                const float* __restrict__ P, int64_t ob1, int64_t ob2,
                                                                int64_t ob3, int64_t ob4,
                                                                const float* __restrict__ norm,
                                                                const unsigned char* __restrict__ wt,
                                                                float* __restrict__ Y, int* errflag) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  // the activations on a 1024-byte boundary of the shared address space
  unsigned char* Hh = tc_smem + ((1024u - (smem_u32_mlp(tc_smem) & 1023u)) & 1023u);
  unsigned char* Hl = Hh + TC_H_BYTES;
  unsigned char* Wslot = Hh + 2 * TC_H_BYTES;
  // full/empty: the weight ring; accb[b]: accumulator b complete; hready[j]: the 32
  // activation columns of block j written by the epilogue (all 16 warps arrive)
  __shared__ __align__(8) uint64_t full[TC_NSLOT], empty[TC_NSLOT], accb[2], hready[TC_H / TC_AB];
  __shared__ uint32_t tmem_base;
  __shared__ float sbias[3][TC_H], sout[3][TC_NOUT];  // biases of layers 1-3; layer-4 bias, y_std, y_mean
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q0 = blockIdx.x * TC_M;
  const float* xm = norm;
  const float* xs = norm + nin;
  if (threadIdx.x == 0) {
    for (int i = 0; i < TC_NSLOT; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32_mlp(&full[i])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32_mlp(&empty[i])) : "memory");
    }
    for (int i = 0; i < 2; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32_mlp(&accb[i])) : "memory");
    for (int i = 0; i < TC_H / TC_AB; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32_mlp(&hready[i])), "r"(TC_EPI) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // all 512 columns of tensor memory: two 128 x 256 FP32 accumulators
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32_mlp(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (warp < TC_EPI) {  // biases and output scales into shared memory
    for (int i = threadIdx.x; i < 3 * TC_H; i += TC_EPI * 32)
      sbias[i / TC_H][i % TC_H] = P[(i < TC_H ? ob1 : i < 2 * TC_H ? ob2 : ob3) + i % TC_H];
    if (threadIdx.x < TC_NOUT) {
      const int j = threadIdx.x;
      sout[0][j] = j < nout ? P[ob4 + j] : 0.f;
      sout[1][j] = j < nout ? norm[2 * nin + nout + j] : 0.f;
      sout[2][j] = j < nout ? norm[2 * nin + j] : 0.f;
    }
    // normalised inputs into activation columns 0..15 (zeros beyond nin)
    for (int i = threadIdx.x; i < TC_M * 16; i += TC_EPI * 32) {
      const int r = i >> 4, k = i & 15;
      const int g = q0 + r;
      float v = 0.f;
      if (k < nin && g < n) v = (X[(int64_t)g * nin + k] - xm[k]) / xs[k];
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      *reinterpret_cast<__nv_bfloat16*>(Hh + tc_hoff(r, k)) = hi;
      *reinterpret_cast<__nv_bfloat16*>(Hl + tc_hoff(r, k)) = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  if (warp == TC_EPI) {  // weight chunks: one bulk copy each into the ring
    if (lane == 0) {
      int issued = 0;
      for (int c = 0; c < TC_CHUNKS; ++c) {
        const int s = c % TC_NSLOT;
        if (c >= TC_NSLOT && !tc_wait(&empty[s], ((c / TC_NSLOT) - 1) & 1, errflag)) break;
        ++issued;
        const uint32_t bytes = (uint32_t)tc_chunk_bytes(c);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32_mlp(&full[s])), "r"(bytes)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32_mlp(Wslot + s * TC_SLOT)),
                     "l"(wt + tc_chunk_off(c)), "r"(bytes), "r"(smem_u32_mlp(&full[s]))
                     : "memory");
      }
      // the last copy into each slot has landed before the CTA may exit (on the normal
      // path the MMA issuer already waited for all of them; after a wait that gave up
      // this keeps the CTA alive until its own copies are done)
      for (int c = issued > TC_NSLOT ? issued - TC_NSLOT : 0; c < issued; ++c) {
        uint32_t tries = 0;
        while (!tc_wait_once(&full[c % TC_NSLOT], (c / TC_NSLOT) & 1))
          if (++tries > (1u << 22)) {
            atomicExch(errflag, 1);
            break;
          }
      }
    }
  } else if (warp == TC_EPI + 1) {  // products: layer l accumulates into buffer (l-1)&1; chunk j of a layer
                                    // waits for activation block j/2 from the previous epilogue
    if (lane == 0) {
      bool ok = true;
      for (int layer = 1, c = 0; layer <= 4 && ok; ++layer) {
        const int nchunks = layer == 1 ? 1 : TC_LCH;
        const int N = layer == 4 ? TC_NOUT : TC_H;
        const uint32_t idesc = tc_idesc(N);
        const uint32_t tacc = tmem + (uint32_t)(((layer - 1) & 1) * TC_H);
        for (int j = 0; j < nchunks; ++j, ++c) {
          const int s = c % TC_NSLOT;
          if (layer > 1 && (j & 1) == 0 && !tc_wait(&hready[j >> 1], (layer - 2) & 1, errflag)) { ok = false; break; }
          if (!tc_wait(&full[s], (c / TC_NSLOT) & 1, errflag)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t bh = smem_u32_mlp(Wslot + s * TC_SLOT);
          const uint32_t bl = bh + (uint32_t)N * TC_KC * 2;
          const uint32_t sbo_b = (uint32_t)(TC_KC / 8) * 128;
          const int k0 = j * TC_KC;  // activation column of this chunk
          const uint64_t ah = tc_adesc(smem_u32_mlp(Hh), k0);
          const uint64_t al = tc_adesc(smem_u32_mlp(Hl), k0);
          const uint64_t dbh = tc_sdesc(bh, sbo_b), dbl = tc_sdesc(bl, sbo_b);
          tc_mma(tacc, ah, dbh, idesc, j != 0);
          tc_mma(tacc, ah, dbl, idesc, 1);
          tc_mma(tacc, al, dbh, idesc, 1);
          tc_commit(&empty[s]);  // the slot is free once these products are done
        }
        tc_commit(&accb[(layer - 1) & 1]);  // also on a failed wait, so the epilogue warps never wait for nothing
      }
    }
  } else {  // epilogue warps: warp w reads TMEM lanes 32 (w%4) ... and columns 8 (w/4) ... of each block
    const int lg = warp & 3, sub = warp >> 2;
    const int row = lg * 32 + lane;
    for (int layer = 1; layer <= 4; ++layer) {
      const int b = (layer - 1) & 1;
      if (!tc_wait(&accb[b], ((layer - 1) >> 1) & 1, errflag)) break;
      __syncwarp();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tl = tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * TC_H) + (uint32_t)(sub * 8);
      if (layer < 4) {
        const float* bias = sbias[layer - 1] + sub * 8;
        uint32_t ra[8], rb[8];
        tc_ld8_issue(tl, ra);
        tc_ld8_wait(ra);
#pragma unroll 1
        for (int jb = 0; jb < TC_H / TC_AB; jb += 2) {  // two blocks per trip: ra holds block jb, rb block jb+1
          tc_ld8_issue(tl + (uint32_t)((jb + 1) * TC_AB), rb);
          tc_act8(ra, bias + jb * TC_AB, Hh + tc_hoff(row, jb * TC_AB + sub * 8), Hl + tc_hoff(row, jb * TC_AB + sub * 8));
          // block jb is written by all 16 warps: publish it to the next layer's products
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32_mlp(&hready[jb])) : "memory");
          tc_ld8_wait(rb);
          if (jb + 2 < TC_H / TC_AB) tc_ld8_issue(tl + (uint32_t)((jb + 2) * TC_AB), ra);
          tc_act8(rb, bias + (jb + 1) * TC_AB, Hh + tc_hoff(row, (jb + 1) * TC_AB + sub * 8),
                  Hl + tc_hoff(row, (jb + 1) * TC_AB + sub * 8));
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32_mlp(&hready[jb + 1])) : "memory");
          if (jb + 2 < TC_H / TC_AB) tc_ld8_wait(ra);
        }
      } else {
        uint32_t r[8];
        tc_ld8_issue(tl, r);
        tc_ld8_wait(r);
        const int g = q0 + row;
        if (g < n) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int col = sub * 8 + j;
            if (col < nout) Y[(int64_t)g * nout + col] = (__uint_as_float(r[j]) + sout[0][col]) * sout[1][col] + sout[2][col];
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();  // every product and every tensor-memory read is done
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Host object
// ---------------------------------------------------------------------------
Mlp::~Mlp() { release(); }

void Mlp::release() {
  cudaFree(params); cudaFree(grads); cudaFree(adam_m); cudaFree(adam_v); cudaFree(norm); cudaFree(ws);
  cudaFree(part);
  cudaFree(wt);
  cudaFree(tc_err);
  params = grads = adam_m = adam_v = norm = ws = nullptr;
  part = nullptr;
  wt = nullptr;
  tc_err = nullptr;
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
  if (nh != TC_H || nin > 16 || nout > TC_NOUT || nin < 1 || nout < 1) {
    err = "tcgen05 inference needs nh = 256, nin <= 16, nout <= 32";
    return false;
  }
  if (!wt && cudaMalloc(&wt, TC_WBYTES) != cudaSuccess) {
    wt = nullptr;
    err = "mlp: inference weights";
    return false;
  }
  if (!tc_err && cudaMalloc(&tc_err, sizeof(int)) != cudaSuccess) {
    tc_err = nullptr;
    err = "mlp: inference flag";
    return false;
  }
  if (cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM) != cudaSuccess) {
    err = "mlp: tcgen05 inference shared memory";
    return false;
  }
  int64_t o[8];
  offsets(o);
  cudaMemsetAsync(tc_err, 0, sizeof(int), s);
  k_mlp_pack_tc<<<cdv(TC_WBYTES / 2, 256), 256, 0, s>>>(params, nin, nh, nout, o[0], o[2], o[4], o[6],
                                                        static_cast<__nv_bfloat16*>(wt));
  if (rows > 0)
    k_mlp_infer_tc<<<cdv(rows, TC_M), TC_THREADS, TC_SMEM, s>>>(rows, nin, nout, X_dev, params, o[1], o[3], o[5], o[7],
                                                               norm, static_cast<const unsigned char*>(wt), Y_dev,
                                                               tc_err);
  launches += rows > 0 ? 2 : 1;
  int h = 0;
  if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&h, tc_err, sizeof(int), cudaMemcpyDeviceToHost, s) !=
                                               cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    err = "mlp: tcgen05 inference launch";
    return false;
  }
  if (h) {
    err = "mlp: a bounded barrier wait in the tcgen05 inference gave up";
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
