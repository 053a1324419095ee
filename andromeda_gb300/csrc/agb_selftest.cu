// Self-test of the bounded barrier wait that every TMA-fed kernel of the
// library uses (mbar_wait_ok, agb_async.cuh): one CTA initialises an mbarrier
// and waits on its first phase with the same wait function the sweeps use,
// under a caller-given poll limit.  With arrive = 0 nothing ever arrives and
// no copy is issued, so the wait must give up, raise the launch's error word
// and return; the host then reports it the way the solvers report a wait that
// gave up (AGB_ERR_CUDA, "a bounded barrier wait ... gave up").  With
// arrive = 1 one thread arrives first and the wait must succeed.  The GPU
// context stays usable either way: nothing faults, traps or hangs.
#include "../../include/andromeda_gb300.h"
#include "agb_async.cuh"

#include <cuda_runtime.h>
#include <string>

__attribute__((visibility("hidden"))) void agb_set_free_error(const std::string& msg);

namespace {

__global__ void k_selftest_wait(uint32_t limit, int arrive, int* __restrict__ errflag, int* __restrict__ done) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    agb::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0)
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(agb::smem_u32(&bar)) : "memory");
  const bool ok = agb::mbar_wait_ok(&bar, 0u, errflag, limit);
  if (ok) atomicAdd(done, 1);
}

}  // namespace

extern "C" int agb_selftest_bounded_wait(int device, unsigned polls, int arrive, int* waits_completed) {
  agb_set_free_error("");
  if (polls == 0 || polls > (1u << 22) || !waits_completed) {
    agb_set_free_error("agb_selftest_bounded_wait: polls must be in 1..2^22 and waits_completed non-NULL");
    return AGB_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(device);
  int* d = nullptr;  // [0] error word, [1] completed waits
  if (e == cudaSuccess) e = cudaMalloc(&d, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(d, 0, 2 * sizeof(int));
  if (e == cudaSuccess) {
    k_selftest_wait<<<1, 32>>>(polls, arrive ? 1 : 0, d, d + 1);
    e = cudaGetLastError();
  }
  int h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    agb_set_free_error(std::string("agb_selftest_bounded_wait: ") + cudaGetErrorString(e));
    return AGB_ERR_CUDA;
  }
  *waits_completed = h[1];
  if (h[0]) {
    agb_set_free_error("a bounded barrier wait gave up (" + std::to_string(polls) +
                       " polls, nothing arrived); the kernel returned and the context is usable");
    return AGB_ERR_CUDA;
  }
  return AGB_OK;
}
