// Column scaling of a dense, caller-owned device matrix that allocates nothing.
//
// Some callers of this library cannot call cudaMalloc: a Fortran or C host
// program that manages all device memory through its own pool (or an OpenACC
// runtime) and forbids other allocators, code running inside an allocation-free
// phase of a larger application, or an embedding whose device memory is
// already fully reserved.  For them agb_lsqr_precon_dense_noalloc performs the
// lsqr_precon column scaling (q_j = 1/||A(:,j)||, A <- A diag(q)) on a matrix
// they already hold on the GPU, using as scratch only the fixed array below.
//
// The scratch array (AGB_NOALLOC_SCRATCH_DOUBLES doubles = 8 MiB) lives in the
// library's device image: every GPU that loads the library holds it until the
// process exits.  Host code cannot use the array's name as a device address,
// so the first call in each CUDA context looks the address up with
// cudaGetSymbolAddress (with that context's device current) and caches it under
// the context's unique id; make that first call before any stream capture.  A
// new context -- another device, a context that is not the primary one (as some
// OpenACC or driver-API hosts make current), or the primary context re-created
// after cudaDeviceReset -- has a new id, so its first call looks the address up
// again instead of reusing an address of a module image that no longer exists.  Every call on a device shares the one
// array and leaves its contents behind: calls whose kernels overlap on the GPU
// (different streams or host threads) race on it and must be serialised by
// the caller.  Nothing in the scratch needs to start at zero: each call writes
// every entry it later reads.
#include "../../include/andromeda_gb300.h"

#include <cuda.h>
#include <cuda_runtime.h>
#include <mutex>
#include <string>

// the context-free error text returned by agb_last_error(NULL) (agb_api.cu)
__attribute__((visibility("hidden"))) void agb_set_free_error(const std::string& msg);

// The scratch: file-scope device array of a fixed size (8 MiB).
static __device__ __align__(256) double g_noalloc_scratch[AGB_NOALLOC_SCRATCH_DOUBLES];

namespace {

// scratch addresses by context id (cuCtxGetId: unique over the life of the
// process, never reused); a full table starts over
constexpr int kMaxContexts = 64;
struct ScratchEntry {
  unsigned long long ctx_id;
  double* ptr;
};
ScratchEntry g_scratch[kMaxContexts];
int g_nscratch = 0;
std::mutex g_scratch_mu;

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// unique id of the calling thread's current context (made current by the
// runtime if there is none yet)
cudaError_t current_context_id(unsigned long long* id) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  if (!get_current || !get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    cudaError_t e = cudaGetDriverEntryPoint("cuCtxGetCurrent", &f1, cudaEnableDefault, &q1);
    if (e == cudaSuccess) e = cudaGetDriverEntryPoint("cuCtxGetId", &f2, cudaEnableDefault, &q2);
    if (e != cudaSuccess) return e;
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return cudaErrorNotSupported;
    get_current = reinterpret_cast<PfnCtxGetCurrent>(f1);
    get_id = reinterpret_cast<PfnCtxGetId>(f2);
  }
  cudaError_t e = cudaFree(nullptr);  // makes the device's primary context current if none is
  if (e != cudaSuccess) return e;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
  if (get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  return cudaSuccess;
}

// Per-row-group column sums of squares: P[g][j] = sum_{r in group g} A(r,j)^2
// (one thread per column, rows of the group in order -> coalesced row reads).
__global__ void k_noalloc_colsq(const double* __restrict__ A, int64_t lda, int m, int n, int rows_per_group,
                                double* __restrict__ P) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int g = blockIdx.y;
  if (j >= n) return;
  const int r0 = g * rows_per_group;
  const int r1 = min(m, r0 + rows_per_group);
  double s = 0.0;
  for (int r = r0; r < r1; ++r) {
    const double a = A[(int64_t)r * lda + j];
    s += a * a;
  }
  P[(int64_t)g * n + j] = s;
}

__global__ void k_noalloc_q(const double* __restrict__ P, int groups, int n, double* __restrict__ q) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double s = 0.0;
  for (int g = 0; g < groups; ++g) s += P[(int64_t)g * n + j];
  q[j] = 1.0 / sqrt(s);
}

__global__ void k_noalloc_scale(double* __restrict__ A, int64_t lda, int m, int n, const double* __restrict__ q) {
  const int64_t total = (int64_t)m * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / n;
    const int j = (int)(t % n);
    A[r * lda + j] *= q[j];
  }
}

int fail(int code, const char* what, cudaError_t e = cudaSuccess) {
  std::string msg = what;
  if (e != cudaSuccess) {
    msg += ": ";
    msg += cudaGetErrorString(e);
  }
  agb_set_free_error(msg);
  return code;
}

}  // namespace

extern "C" int agb_lsqr_precon_dense_noalloc(int m, int n, int64_t lda, double* A, double* q) {
  agb_set_free_error("");
  if (m <= 0 || n <= 0 || lda < n || !A || !q) return fail(AGB_ERR_ARG, "agb_lsqr_precon_dense_noalloc: bad sizes or NULL pointer");
  if ((int64_t)n > (int64_t)AGB_NOALLOC_SCRATCH_DOUBLES)
    return fail(AGB_ERR_ARG, "agb_lsqr_precon_dense_noalloc: n exceeds AGB_NOALLOC_MAX_COLUMNS (1048576)");
  unsigned long long ctx_id = 0;
  cudaError_t e = current_context_id(&ctx_id);
  if (e != cudaSuccess) return fail(AGB_ERR_CUDA, "agb_lsqr_precon_dense_noalloc: current CUDA context", e);
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    for (int i = 0; i < g_nscratch; ++i)
      if (g_scratch[i].ctx_id == ctx_id) scratch = g_scratch[i].ptr;
    if (!scratch) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return fail(AGB_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch)", e);
      scratch = static_cast<double*>(p);
      if (g_nscratch == kMaxContexts) g_nscratch = 0;
      g_scratch[g_nscratch++] = {ctx_id, scratch};
    }
  }
  // row groups: as many as the scratch holds, at most 64
  int groups = (int)(AGB_NOALLOC_SCRATCH_DOUBLES / n);
  if (groups > 64) groups = 64;
  if (groups > m) groups = m;
  if (groups < 1) groups = 1;
  const int rpg = (m + groups - 1) / groups;
  groups = (m + rpg - 1) / rpg;
  const int threads = 256;
  k_noalloc_colsq<<<dim3((n + threads - 1) / threads, groups), threads>>>(A, lda, m, n, rpg, scratch);
  k_noalloc_q<<<(n + threads - 1) / threads, threads>>>(scratch, groups, n, q);
  const int64_t total = (int64_t)m * n;
  int64_t blocks = (total + threads - 1) / threads;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_noalloc_scale<<<(unsigned)blocks, threads>>>(A, lda, m, n, q);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(AGB_ERR_CUDA, "agb_lsqr_precon_dense_noalloc launch", e);
  e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) return fail(AGB_ERR_CUDA, "agb_lsqr_precon_dense_noalloc", e);
  return AGB_OK;
}
