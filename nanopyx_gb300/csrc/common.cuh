// Shared device/host helpers for the eSRRF/SRRF engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "nanopyx_gb300.h"

namespace nx {

// ---------------------------------------------------------------------------
// status words written by kernels (device) and returned by the C-ABI (host)
// ---------------------------------------------------------------------------
enum DeviceStatusBits : unsigned {
  kDevOk = 0u,
  kDevTmaTimeout = 1u << 0,   // an mbarrier wait for a TMA tile ran out of time
  kDevBadGeometry = 1u << 1,  // a launch saw an impossible tile geometry
};

// Bounded-wait budget for every device spin (ns of %globaltimer).
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------------------
// mbarrier + TMA (cp.async.bulk.tensor) wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// Wait for phase `parity` of `bar`; gives up after `limit_ns` and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity,
                                                  unsigned long long limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// As mbar_wait_bounded, but also gives up as soon as *abort is set (another
// thread of the CTA gave up first), so that no thread waits for an arrival
// that will never come.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, unsigned parity,
                                                   const volatile int* abort,
                                                   unsigned long long limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// 3-D tiled TMA load (x fastest).  The x coordinate must be a multiple of 4
// floats (16 B); callers guarantee it by construction.
__device__ __forceinline__ void tma_load_3d(void* dst, const void* tmap, uint64_t* bar, int x, int y,
                                            int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cta.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// Catmull-Rom (Keys, a = 0.5) weight of one tap, float arithmetic.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ float cr_cubic(float v) {
  v = fabsf(v);
  if (v < 1.f) return v * v * (1.5f * v - 2.5f) + 1.f;
  if (v < 2.f) return ((-0.5f * v + 2.5f) * v - 4.f) * v + 2.f;
  return 0.f;
}

__host__ __device__ __forceinline__ int floordiv(int a, int b) {
  int q = a / b;
  return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

// ---------------------------------------------------------------------------
// Streaming temporal moments of one pixel's time series x_0 .. x_{n-1} (float32).
//
//   mean   running mean (Welford: mean += (x - mean) / n)
//   m2     sum_t (x_t - mean)^2
//   c      sum_{t<n-1} (x_t - mean)(x_{t+1} - mean), the lag-1 co-moment about
//          the CURRENT mean -- what TAC2 needs at the end
//   a, b   x_{n-1} - mean and x_0 - mean (last and first value as deviations)
//
// Every update adds deviation-sized terms, so nothing cancels the way raw or
// shifted power sums do.  Adding x as frame k (k >= 1 frames in, d = x - mean,
// e = d / (k+1), mean' = mean + e): expanding the old pairs about mean' moves c
// by e (a + b) + (k-1) e^2 (the centred values sum to zero) and the new pair
// adds (a - e)(d - e); with k e^2 - e d = -e^2 this collapses to
//   c' = c + a d + e (b - e),   m2' = m2 + d (d - e),   a' = d - e,   b' = b - e.
// Two records of consecutive frames merge exactly with the pairwise formulas
// of Chan, Golub and LeVeque plus the one pair that straddles the boundary.
// AVG = mean, VAR = m2 / n, TAC2 = c / (n - 1)
// (sr_temporal_correlations.py:46-75, 205-221).
// ---------------------------------------------------------------------------
struct Moments {
  float mean, m2, c, a, b;
};

__host__ __device__ __forceinline__ Moments moments_start(float x) {
  return Moments{x, 0.f, 0.f, 0.f, 0.f};
}

// x is frame k of the series (k >= 1 frames already folded in); inv = 1 / (k + 1)
__device__ __forceinline__ void moments_push(Moments& s, float x, float inv) {
  const float d = x - s.mean;
  const float e = d * inv;
  s.mean = s.mean + e;
  const float bn = s.b - e;
  s.c = fmaf(e, bn, fmaf(s.a, d, s.c));
  const float u = d - e;
  s.m2 = fmaf(d, u, s.m2);
  s.a = u;
  s.b = bn;
}

// a <- a (+) b where b's nb frames follow a's na frames (full: all fields,
// else the mean only)
__device__ __forceinline__ void moments_merge(Moments& a, const Moments& b, int na, int nb,
                                              bool full) {
  if (nb == 0) return;
  if (na == 0) {
    a = b;
    return;
  }
  const float n = (float)na + (float)nb;
  const float dl = b.mean - a.mean;
  const float mn = fmaf(dl, __fdiv_rn((float)nb, n), a.mean);
  if (full) {
    const float da = mn - a.mean, db = mn - b.mean;
    const float ca = a.c + da * (a.a + a.b) + (float)(na - 1) * (da * da);
    const float cb = b.c + db * (b.a + b.b) + (float)(nb - 1) * (db * db);
    a.c = ca + cb + (a.a - da) * (b.b - db);
    a.m2 = a.m2 + b.m2 + (dl * dl) * __fdiv_rn((float)na * (float)nb, n);
    a.a = b.a - db;
    a.b = a.b - da;
  }
  a.mean = mn;
}

}  // namespace nx

// host-side error plumbing shared by the C-ABI translation units
namespace nx {
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);
}  // namespace nx

#define NX_CUDA_TRY(call)                                            \
  do {                                                               \
    cudaError_t _e = (call);                                         \
    if (_e != cudaSuccess) return ::nx::cuda_status(_e, #call);      \
  } while (0)
