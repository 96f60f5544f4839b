// FP32 FMA throughput probe: the denominator of the RGC kernel's roofline.
#include "common.cuh"

namespace {

__global__ void __launch_bounds__(256) ffma_probe_kernel(float* sink, int iters) {
  float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float b = 0.999f, c = 1e-4f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
    }
  }
  sink[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__global__ void __launch_bounds__(256) ffma2_probe_kernel(float* sink, int iters) {
  float2 a0 = make_float2(threadIdx.x * 1e-3f, 1.f), a1 = make_float2(2.f, 3.f);
  float2 a2 = make_float2(4.f, 5.f), a3 = make_float2(6.f, 7.f);
  const float2 b = make_float2(0.999f, 0.999f), c = make_float2(1e-4f, 1e-4f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = __ffma2_rn(a0, b, c); a1 = __ffma2_rn(a1, b, c);
      a2 = __ffma2_rn(a2, b, c); a3 = __ffma2_rn(a3, b, c);
    }
  }
  sink[blockIdx.x * blockDim.x + threadIdx.x] =
      a0.x + a0.y + a1.x + a1.y + a2.x + a2.y + a3.x + a3.y;
}

// One CTA waits on an mbarrier that nothing arrives on, with the same bounded
// wait the fused kernels use; on time-out it records the same status bit.
__global__ void wait_timeout_selftest_kernel(unsigned* status, unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    nx::mbar_init(&bar, 1);
    nx::fence_mbar_init();
  }
  __syncthreads();
  const bool ok = nx::mbar_wait_bounded(&bar, 0u, limit_ns);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(status, nx::kDevTmaTimeout);
  __syncthreads();
  if (threadIdx.x == 0) nx::mbar_inval(&bar);
}

}  // namespace

extern "C" int nx_selftest_wait_timeout(void* d_ws, size_t ws_bytes, unsigned long long limit_ns,
                                        void* stream) {
  if (!d_ws || ws_bytes < 256) return NX_ERR_WORKSPACE;
  if (limit_ns > 1000000000ull) return NX_ERR_INVALID_ARG;  // keep the self-test short
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(d_ws, 0, sizeof(unsigned), s);
  if (e == cudaSuccess) {
    wait_timeout_selftest_kernel<<<1, 64, 0, s>>>((unsigned*)d_ws, limit_ns);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? NX_OK : nx::cuda_status(e, "wait self-test");
}

extern "C" int nx_probe_ffma2(float* d_sink, int blocks, int iters, void* stream) {
  if (!d_sink || blocks < 1 || iters < 1) return NX_ERR_INVALID_ARG;
  ffma2_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_sink, iters);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NX_OK : nx::cuda_status(e, "ffma2 probe");
}

extern "C" int nx_probe_ffma(float* d_sink, int blocks, int iters, void* stream) {
  if (!d_sink || blocks < 1 || iters < 1) return NX_ERR_INVALID_ARG;
  ffma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_sink, iters);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NX_OK : nx::cuda_status(e, "ffma probe");
}
