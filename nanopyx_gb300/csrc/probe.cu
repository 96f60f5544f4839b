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

}  // namespace

extern "C" int nx_probe_ffma(float* d_sink, int blocks, int iters, void* stream) {
  if (!d_sink || blocks < 1 || iters < 1) return NX_ERR_INVALID_ARG;
  ffma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_sink, iters);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NX_OK : nx::cuda_status(e, "ffma probe");
}
