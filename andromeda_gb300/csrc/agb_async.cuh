// Device helpers shared by the LSQR kernels: shared-memory barriers and bulk
// copies (mbarrier, cp.async.bulk, 2-D tensor-map loads) with bounded waits,
// the reference BLAS-style d2norm, and the scalar phases of the LSQR
// recurrence (lib_lsqr.f:900-1231) for one right-hand side.
#pragma once
#include "agb_lsqr.cuh"

namespace agb {

constexpr int K8 = AGB_MAX_RHS;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: after ~2^22 failed tries the barrier is reported through
// errflag and the wait gives up (the copies are in bounds by construction, so
// this only guards against a hang); once any wait has given up (errflag set),
// later long waits give up after ~1024 tries, so a launch whose barrier broke
// ends quickly.  Returns whether the barrier phase completed.
// (limit: the number of failed tries before giving up; the kernels use 2^22,
// the self-test entry point agb_selftest_bounded_wait a caller-given one)
__device__ __forceinline__ bool mbar_wait_ok(uint64_t* bar, uint32_t parity, int* errflag,
                                             uint32_t limit = (1u << 22)) {
  uint32_t tries = 0;
  while (!mbar_try_wait(bar, parity)) {
    ++tries;
    if ((tries & 1023u) == 0 && errflag && *(volatile int*)errflag) return false;
    if (tries > limit) {
      if (errflag) atomicExch(errflag, 1);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* errflag) {
  (void)mbar_wait_ok(bar, parity, errflag);
}
// Before a CTA exits: wait, bounded but without the early exit on the error
// flag, for the copies of the last stages of a ring of nslot slots (stage k
// lands on full[k % nslot], phase parity (k / nslot) & 1).  On the normal path
// the consumers already waited for every one of these phases, so each wait
// returns at once; after a wait that gave up, it keeps the CTA alive until its
// own copies have landed in its shared memory.
__device__ __forceinline__ void mbar_drain(uint64_t* full, int nslot, int nst, int* errflag) {
  for (int k = nst > nslot ? nst - nslot : 0; k < nst; ++k) {
    uint32_t tries = 0;
    while (!mbar_try_wait(&full[k % nslot], (uint32_t)((k / nslot) & 1))) {
      if (++tries > (1u << 22)) {
        if (errflag) atomicExch(errflag, 1);
        break;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ double d2norm(double a, double b) {
  double scale = fabs(a) + fabs(b);
  if (scale == 0.0) return 0.0;
  return scale * sqrt((a / scale) * (a / scale) + (b / scale) * (b / scale));
}

// Scalar phase of one right-hand side c of k right-hand sides; ssum is the
// reduced sum of squares that the phase consumes.
// phase 0: beta0 = ||r||; bnorm.       phase 1: alpha0; init recurrences.
// phase 2: beta = ||Y|| after sweep 1; anorm.
// phase 3: alpha after sweep 2; plane rotations; t1,t2,t3; gamma for next sweep.
// phase 4: after the x/w update: dnorm, xnorm, residual estimates, stopping tests.
__device__ __forceinline__ void lsqr_phase(LsqrScalars& s, int c, int k, int phase, double ssum, int* nactive) {
  if (c >= k) { s.active = 0; return; }
  if (phase == 0) {
    s.beta = sqrt(ssum);
    return;
  }
  if (!s.active) return;
  if (phase == 1) {
    s.alpha = sqrt(ssum);
    if (s.beta <= 0.0) s.alpha = 0.0;
    s.rhobar = s.alpha;
    s.phibar = s.beta;
    s.bnorm = s.beta;
    s.rnorm = s.beta;
    s.arnorm = s.alpha * s.beta;
    s.anorm = s.acond = s.dnorm = s.dxmax = s.res2 = s.xnorm = s.xnorm1 = s.z = s.sn2 = 0.0;
    s.cs2 = -1.0;
    s.itn = 0;
    s.istop = 0;
    s.gamma = (s.beta > 0.0) ? -s.alpha / s.beta : 0.0;
    if (s.arnorm == 0.0) s.active = 0;  // lsqr: GOTO 800 with istop = 0
    return;
  }
  if (phase == 2) {
    s.itn += 1;
    s.beta = sqrt(ssum);
    double temp = d2norm(s.alpha, s.beta);
    temp = d2norm(temp, 0.0);
    s.anorm = d2norm(s.anorm, temp);
    return;
  }
  if (phase == 3) {
    if (s.beta > 0.0) {
      s.alpha = sqrt(ssum);
    }
    double rhbar1 = s.rhobar;
    double rho = d2norm(rhbar1, s.beta);
    double cs = rhbar1 / rho, sn = s.beta / rho;
    double theta = sn * s.alpha;
    s.rhobar = -cs * s.alpha;
    double phi = cs * s.phibar;
    s.phibar = sn * s.phibar;
    double tau = sn * phi;
    s.t1 = phi / rho;
    s.t2 = -theta / rho;
    s.t3 = 1.0 / rho;
    // second rotation and norm estimates (depend only on scalars)
    double delta = s.sn2 * rho, gambar = -s.cs2 * rho;
    double rhs = phi - delta * s.z;
    double zbar = rhs / gambar;
    s.xnorm = d2norm(s.xnorm1, zbar);
    double gamma = d2norm(gambar, theta);
    s.cs2 = gambar / gamma;
    s.sn2 = theta / gamma;
    s.z = rhs / gamma;
    s.xnorm1 = d2norm(s.xnorm1, s.z);
    s.res2 = d2norm(s.res2, 0.0);
    s.rnorm = d2norm(s.res2, s.phibar);
    s.arnorm = s.alpha * fabs(tau);
    // stash phi for the dxk monitor
    s.dxmax = fmax(s.dxmax, 0.0);
    s.acond = phi;  // temporary (phi), replaced in phase 4
    return;
  }
  if (phase == 4) {
    const double phi = s.acond;
    double dknorm = sqrt(ssum);
    s.dnorm = d2norm(s.dnorm, dknorm);
    double dxk = fabs(phi * dknorm);
    if (s.dxmax < dxk) s.dxmax = dxk;
    s.acond = s.anorm * s.dnorm;
    const double one = 1.0, zero = 0.0;
    double test1 = s.rnorm / s.bnorm;
    double test2 = zero;
    if (s.rnorm > zero) test2 = s.arnorm / (s.anorm * s.rnorm);
    double test3 = one / s.acond;
    double t1 = test1 / (one + s.anorm * s.xnorm / s.bnorm);
    double rtol = s.btol + s.atol * s.anorm * s.xnorm / s.bnorm;
    double t3 = one + test3, t2 = one + test2;
    t1 = one + t1;
    int istop = 0;
    if (s.itn >= s.itnlim) istop = 5;
    if (t3 <= one) istop = 4;
    if (t2 <= one) istop = 2;
    if (t1 <= one) istop = 1;
    if (test3 <= s.ctol) istop = 4;
    if (test2 <= s.atol) istop = 2;
    if (test1 <= rtol) istop = 1;
    s.istop = istop;
    if (istop != 0) s.active = 0;
    s.gamma = (s.beta > 0.0) ? -s.alpha / s.beta : 0.0;
    if (s.beta <= 0.0) s.active = 0;
    if (s.active) atomicAdd(nactive, 1);
  }
}

// BiCGSTAB state of one right-hand side at the start (||b||^2 = bb) and at the
// end of an iteration (rr = ||r||^2, rho = r~ . r); shared by the single-system
// and the batched solvers.
__device__ __forceinline__ void bicg_start(BicgScalars& q, double bb, bool used) {
  q.bnorm = sqrt(bb);
  q.rho = bb;  // r~ = r0 = b
  q.rho_old = q.alpha = q.omega = 1.0;
  q.relres = (q.bnorm > 0.0) ? 1.0 : 0.0;
  q.snorm = q.relres;
  q.best = q.relres;
  q.its = 0;
  q.half = 0;
  q.since = 0;
  q.active = (used && q.bnorm > 0.0) ? 1 : 0;
  q.status = q.active ? -1 : 0;
}
__device__ __forceinline__ void bicg_end(BicgScalars& q, double rr, double rho, double tol, int maxit) {
  q.its += 1;
  if (q.half) {
    q.relres = q.snorm;
    q.status = 0;
    q.active = 0;
    return;
  }
  q.relres = sqrt(rr) / q.bnorm;
  if (q.relres <= tol) {
    q.status = 0;
    q.active = 0;
  } else if (q.its >= maxit) {
    q.status = 1;
    q.active = 0;
  } else if (rho == 0.0 || q.omega == 0.0 || !isfinite(q.relres)) {
    q.status = 2;
    q.active = 0;
  } else if (q.relres > BICG_DIVERGE * q.best || (q.relres >= 0.9 * q.best && q.since + 1 >= BICG_STALL)) {
    q.status = 3;
    q.active = 0;
  } else {
    if (q.relres < 0.9 * q.best) {
      q.best = q.relres;
      q.since = 0;
    } else {
      q.since += 1;
    }
    q.rho_old = q.rho;
    q.rho = rho;
  }
}

// inverse of a 3x3 block B (FP64) into o[9], row-major, by cofactors; false
// (and zeros) if it is singular or not finite
__device__ __forceinline__ bool inv3(const double (&B)[3][3], double* o) {
  const double c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1], c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2],
               c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
  const double det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
  if (!(det != 0.0) || !isfinite(det)) {
    for (int k = 0; k < 9; ++k) o[k] = 0.0;
    return false;
  }
  const double id = 1.0 / det;
  o[0] = c00 * id;
  o[1] = (B[0][2] * B[2][1] - B[0][1] * B[2][2]) * id;
  o[2] = (B[0][1] * B[1][2] - B[0][2] * B[1][1]) * id;
  o[3] = c01 * id;
  o[4] = (B[0][0] * B[2][2] - B[0][2] * B[2][0]) * id;
  o[5] = (B[0][2] * B[1][0] - B[0][0] * B[1][2]) * id;
  o[6] = c02 * id;
  o[7] = (B[0][1] * B[2][0] - B[0][0] * B[2][1]) * id;
  o[8] = (B[0][0] * B[1][1] - B[0][1] * B[1][0]) * id;
  return true;
}

}  // namespace agb
