// Scoring of the eSRRF parameter sweep on the GPU: the numeric kernels behind
// ErrorMap (RSP / RSE) and FIRECalculator (FRC) that the reference's
// ParameterSweep calls per grid point
// (src/nanopyx/core/analysis/parameter_sweep.py:99-139).
//
// * Gaussian blur with scipy.ndimage.gaussian_filter's definition (the
//   reference's error_map.pyx:72-77,127-146): separable, axis 0 then axis 1,
//   kernel radius int(4 sigma + 0.5), weights exp(-x^2 / (2 sigma^2))
//   normalised to sum 1, mode 'reflect' (d c b a | a b c d | d c b a); an axis
//   with sigma <= 1e-15 is left as it is.  Where the kernel is longer than the
//   reflection period 2n the taps are folded onto it (the extension is
//   periodic), so any sigma costs at most 2n taps per output.
// * Moment sums of image pairs in float64 (regression, Pearson correlation and
//   RMSE of the error map), deterministic: fixed per-block partials, then one
//   block in fixed order.
// * FRC ring sums (frc.pyx:108-143,150-179): crop to the even square, Tukey
//   taper, 2-D FFT of both images (Stockham autosort, mixed radix, one CTA per
//   line, twiddles from a float64 table rounded once), and per ring radius the
//   bilinearly interpolated products a1 a2 + b1 b2, a1^2 + b1^2, a2^2 + b2^2
//   of the centred spectra summed in float64 over the reference's own sample
//   positions (float32 angles i * fl(1/r), cos/sin as the reference forms
//   them).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace nx {
namespace {

constexpr int kSumFields = 6;    // sx, sy, Sxx, Sxy, Syy, s(x-y)^2
constexpr int kFftThreads = 256;
constexpr int kMaxFftN = 8192;   // two complex line buffers in shared memory
constexpr int kFrcChunk = 8;     // image pairs per FFT launch

__host__ __device__ inline long long reflect_index(long long i, long long n) {
  // 'reflect' extension of [0, n): period 2n, the second half mirrored
  const long long p = 2 * n;
  long long m = i % p;
  if (m < 0) m += p;
  return m < n ? m : p - 1 - m;
}

// ---------------------------------------------------------------------------
// Gaussian blur, a batch of images per launch, each with its own sigma (and
// affine map): the Brent searches of several error maps advance in lockstep
// ---------------------------------------------------------------------------
struct BlurAxis {
  int taps;    // number of weights
  int offset;  // sample index of weight 0 relative to the output index
  int fold;    // weights folded onto the reflection period
};

constexpr int kBlurBatch = 32;  // images per launch
struct BlurBatch {
  int n, affine;
  int src[kBlurBatch];  // image index in the input stack
  int radius[kBlurBatch];
  double sigma[kBlurBatch];
  float alpha[kBlurBatch], beta[kBlurBatch];
  BlurAxis ax[2][kBlurBatch];  // taps == 1, offset 0: axis left as it is
};

// scipy's weights of one image and axis (blockIdx.x, blockIdx.y), in float64,
// normalised, folded onto the reflection period when the kernel is longer;
// stored as A (float, or double for float64 accumulation)
template <typename A>
__global__ void gauss_weights_kernel(const __grid_constant__ BlurBatch b, int H, int W,
                                     A* __restrict__ w0, A* __restrict__ w1) {
  __shared__ double red[256];
  const int z = blockIdx.x, axis = blockIdx.y;
  const int n = axis ? W : H;
  A* w = axis ? w1 + (size_t)z * 2 * W : w0 + (size_t)z * 2 * H;
  const BlurAxis ax = b.ax[axis][z];
  const double sigma = b.sigma[z];
  const int radius = b.radius[z];
  if (!(sigma > 1e-15)) {
    if (threadIdx.x == 0) w[0] = (A)1;
    return;
  }
  const double c = -0.5 / (sigma * sigma);
  double part = 0.0;
  for (int k = threadIdx.x; k <= 2 * radius; k += blockDim.x) {
    const double x = (double)(k - radius);
    part += exp(c * x * x);
  }
  red[threadIdx.x] = part;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const double total = red[0];
  if (!ax.fold) {
    for (int k = threadIdx.x; k <= 2 * radius; k += blockDim.x) {
      const double x = (double)(k - radius);
      w[k] = (A)(exp(c * x * x) / total);
    }
    return;
  }
  // folded: weight j collects every tap offset d with d = j (mod 2n)
  const int p = 2 * n;
  for (int j = threadIdx.x; j < p; j += blockDim.x) {
    double acc = 0.0;
    const long long d0 = j - (long long)((j + radius) / p) * p;  // smallest d >= -radius
    for (long long d = d0; d <= radius; d += p) acc += exp(c * (double)d * (double)d) / total;
    w[j] = (A)acc;
  }
}

template <typename A>
__device__ __forceinline__ A mac(A w, float v, A acc) {
  return fma(w, (A)v, acc);
}

// axis 0: out[z][y][x] = sum_j w[j] * src[reflect(y + offset + j)][x], the
// source mapped to alpha * v + beta first when the batch is affine.  A CTA
// computes 32 columns x 64 rows (8 rows per thread); with up to kStageTaps
// taps the weights and the column strip with its reflected halo rows are
// staged in shared memory, else the taps are read through the cache.  The
// accumulator is A; each pass rounds to float32 (as scipy writes a float32
// output array axis by axis).
constexpr int kTileCols = 32, kTileRows = 64, kRowsPerThread = 8;
constexpr int kStageTaps = 256;
template <typename A>
__global__ void __launch_bounds__(256) blur_axis0_kernel(const __grid_constant__ BlurBatch b,
                                                         const float* __restrict__ in, int H,
                                                         int W, const A* __restrict__ w0,
                                                         int staged, float* __restrict__ mid) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int z = blockIdx.z;
  const int x0 = blockIdx.x * kTileCols, y0 = blockIdx.y * kTileRows;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTileCols + tx;
  const float* src = in + (size_t)b.src[z] * H * W;
  const A* w = w0 + (size_t)z * 2 * H;
  const BlurAxis ax = b.ax[0][z];
  const float alpha = b.alpha[z], beta = b.beta[z];
  const int x = x0 + tx;
  A acc[kRowsPerThread];
#pragma unroll
  for (int q = 0; q < kRowsPerThread; ++q) acc[q] = (A)0;
  if (staged) {
    A* ws = reinterpret_cast<A*>(smraw);
    float* tile = reinterpret_cast<float*>(ws + kStageTaps);
    for (int k = tid; k < ax.taps; k += 256) ws[k] = w[k];
    // rows of the strip, 8 in flight per thread (the row index, reflected,
    // is the same for a whole warp: kTileCols = 32 lanes = one row)
    const int rows = kTileRows + ax.taps - 1;
    const bool colok = x < W;
    for (int k0 = ty; k0 < rows; k0 += 8 * 8) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + u * 8;
        v[u] = 0.f;
        if (k < rows && colok) {
          int r = y0 + ax.offset + k;
          if (r < 0 || r >= H) r = (int)reflect_index(r, H);
          v[u] = __ldg(src + (size_t)r * W + x);
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + u * 8;
        if (k < rows)
          tile[k * kTileCols + tx] = b.affine ? __fadd_rn(__fmul_rn(alpha, v[u]), beta) : v[u];
      }
    }
    __syncthreads();
    const float* col = tile + ty * kRowsPerThread * kTileCols + tx;
    // 8 taps at a time from a 16-value window of the column: each staged
    // value is read once per 8 taps instead of once per tap and output row
    // (the tap order of every output is unchanged)
    int j = 0;
    for (; j + 8 <= ax.taps; j += 8) {
      float win[16];
#pragma unroll
      for (int u = 0; u < 15; ++u) win[u] = col[(j + u) * kTileCols];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const A wj = ws[j + u];
#pragma unroll
        for (int q = 0; q < kRowsPerThread; ++q) acc[q] = mac(wj, win[q + u], acc[q]);
      }
    }
    for (; j < ax.taps; ++j) {
      const A wj = ws[j];
#pragma unroll
      for (int q = 0; q < kRowsPerThread; ++q) acc[q] = mac(wj, col[(q + j) * kTileCols], acc[q]);
    }
  } else if (x < W) {
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      const int y = y0 + ty * kRowsPerThread + q;
      if (y >= H) break;
      for (int j = 0; j < ax.taps; ++j) {
        long long r = (long long)y + ax.offset + j;
        if (r < 0 || r >= H) r = reflect_index(r, H);
        float v = __ldg(src + (size_t)r * W + x);
        if (b.affine) v = __fadd_rn(__fmul_rn(alpha, v), beta);
        acc[q] = mac(w[j], v, acc[q]);
      }
    }
  }
  if (x < W) {
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      const int y = y0 + ty * kRowsPerThread + q;
      if (y < H) mid[((size_t)z * H + y) * W + x] = (float)acc[q];
    }
  }
}

// axis 1: the row segment with its reflected halo (and the weights) staged in
// shared memory when they fit, else read through the cache
constexpr int kRowTile = 256;
template <typename A>
__global__ void __launch_bounds__(256) blur_axis1_kernel(const __grid_constant__ BlurBatch b,
                                                         const float* __restrict__ mid, int H,
                                                         int W, const A* __restrict__ w1,
                                                         int staged, float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int y = blockIdx.y, z = blockIdx.z;
  const int x0 = blockIdx.x * kRowTile;
  const float* row = mid + ((size_t)z * H + y) * W;
  const A* w = w1 + (size_t)z * 2 * W;
  const BlurAxis ax = b.ax[1][z];
  A* ws = reinterpret_cast<A*>(smraw);
  float* seg = reinterpret_cast<float*>(ws + ((ax.taps + 3) & ~3));
  if (staged) {
    for (int k = threadIdx.x; k < ax.taps; k += blockDim.x) ws[k] = w[k];
    const int span = kRowTile + ax.taps - 1;
    for (int k = threadIdx.x; k < span; k += blockDim.x) {
      long long c = (long long)x0 + ax.offset + k;
      if (c < 0 || c >= W) c = reflect_index(c, W);
      seg[k] = __ldg(row + c);
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < kRowTile; t += blockDim.x) {
    const int x = x0 + t;
    if (x >= W) break;
    A acc = (A)0;
    if (staged) {
      for (int j = 0; j < ax.taps; ++j) acc = mac(ws[j], seg[t + j], acc);
    } else {
      for (int j = 0; j < ax.taps; ++j) {
        long long c = (long long)x + ax.offset + j;
        if (c < 0 || c >= W) c = reflect_index(c, W);
        acc = mac(w[j], __ldg(row + c), acc);
      }
    }
    out[((size_t)z * H + y) * W + x] = (float)acc;
  }
}

template <typename A>
int run_blur_batch(const float* d_in, int H, int W, int n, const int* src_index,
                   const double* sigma, const float* alpha, const float* beta, float* d_out,
                   char* base, cudaStream_t s);

// ---------------------------------------------------------------------------
// Moment sums of (x, y) pairs: sums and centred second moments in float64.
// FP64 is slow on this GPU, so each thread sums a short run (at most
// kSumRun elements) in float32 and only the cross-thread reduction is in
// float64; the second moments are taken about the float32-rounded means
// (two passes) and corrected to the exact means, so nothing cancels.
// ---------------------------------------------------------------------------
constexpr int kSumRun = 32;         // elements per thread and pass (short float32 runs)
constexpr int kSumMaxBlocks = 2048;

__device__ inline void block_sum(double* v, int nf, double* red /* [nf][blockDim] */) {
  for (int f = 0; f < nf; ++f) red[f * blockDim.x + threadIdx.x] = v[f];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int f = 0; f < nf; ++f)
        red[f * blockDim.x + threadIdx.x] += red[f * blockDim.x + threadIdx.x + s];
    __syncthreads();
  }
  for (int f = 0; f < nf; ++f) v[f] = red[f * blockDim.x];
  __syncthreads();
}

// pass 1: sum x, sum y
__global__ void __launch_bounds__(256) moment_mean_kernel(const float* __restrict__ x,
                                                          const float* __restrict__ y,
                                                          long long n,
                                                          double* __restrict__ part) {
  __shared__ double red[2 * 256];
  const float* xs = x + (size_t)blockIdx.y * n;
  double v[2] = {0, 0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n;
       i0 += stride * kSumRun) {
    float sx = 0.f, sy = 0.f;
#pragma unroll 8
    for (int k = 0; k < kSumRun; ++k) {  // unrolled: the loads of a run in flight together
      const long long i = i0 + k * stride;
      const float a = i < n ? __ldg(xs + i) : 0.f, b = i < n ? __ldg(y + i) : 0.f;
      sx += a;
      sy += b;
    }
    v[0] += sx;
    v[1] += sy;
  }
  block_sum(v, 2, red);
  if (threadIdx.x == 0) {
    part[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 2 + 0] = v[0];
    part[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 2 + 1] = v[1];
  }
}

// per image: the two sums in fixed order, and the means rounded to float
// (sums: batch x 2 doubles; fmeans: batch x 2 floats)
__global__ void __launch_bounds__(256) moment_mean_final_kernel(const double* __restrict__ part,
                                                                int nparts, long long n,
                                                                double* __restrict__ sums,
                                                                float* __restrict__ fmeans) {
  __shared__ double red[2 * 256];
  double v[2] = {0, 0};
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
    v[0] += part[((size_t)blockIdx.x * nparts + b) * 2 + 0];
    v[1] += part[((size_t)blockIdx.x * nparts + b) * 2 + 1];
  }
  block_sum(v, 2, red);
  if (threadIdx.x == 0) {
    sums[blockIdx.x * 2 + 0] = v[0];
    sums[blockIdx.x * 2 + 1] = v[1];
    fmeans[blockIdx.x * 2 + 0] = (float)(v[0] / (double)n);
    fmeans[blockIdx.x * 2 + 1] = (float)(v[1] / (double)n);
  }
}

// pass 2: products about the float32-rounded means, and (x - y)^2
__global__ void __launch_bounds__(256) moment_centred_kernel(const float* __restrict__ x,
                                                             const float* __restrict__ y,
                                                             long long n,
                                                             const float* __restrict__ fmeans,
                                                             double* __restrict__ part) {
  __shared__ double red[4 * 256];
  const int z = blockIdx.y;
  const float* xs = x + (size_t)z * n;
  const float mx = fmeans[2 * z], my = fmeans[2 * z + 1];
  double v[4] = {0, 0, 0, 0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n;
       i0 += stride * kSumRun) {
    float cxx = 0.f, cxy = 0.f, cyy = 0.f, dd = 0.f;
#pragma unroll 8
    for (int k = 0; k < kSumRun; ++k) {  // out-of-range terms are (mean, mean): they add 0
      const long long i = i0 + k * stride;
      const float a = i < n ? __ldg(xs + i) : mx, b = i < n ? __ldg(y + i) : my;
      const float dx = a - mx, dy = b - my, d = i < n ? __fsub_rn(a, b) : 0.f;
      cxx = fmaf(dx, dx, cxx);
      cxy = fmaf(dx, dy, cxy);
      cyy = fmaf(dy, dy, cyy);
      dd = fmaf(d, d, dd);
    }
    v[0] += cxx;
    v[1] += cxy;
    v[2] += cyy;
    v[3] += dd;
  }
  block_sum(v, 4, red);
  if (threadIdx.x == 0)
    for (int f = 0; f < 4; ++f) part[((size_t)z * gridDim.x + blockIdx.x) * 4 + f] = v[f];
}

// per image: (sum x, sum y, Sxx, Sxy, Syy, sum (x-y)^2), S centred about the
// exact means: S(x - m~) = S(x - m) + n (m - m~)(...)
__global__ void __launch_bounds__(256) moment_final_kernel(const double* __restrict__ part,
                                                           int nparts, long long n,
                                                           const double* __restrict__ sums,
                                                           double* __restrict__ out) {
  __shared__ double red[4 * 256];
  const int z = blockIdx.x;
  double v[4] = {0, 0, 0, 0};
  for (int b = threadIdx.x; b < nparts; b += blockDim.x)
    for (int f = 0; f < 4; ++f) v[f] += part[((size_t)z * nparts + b) * 4 + f];
  block_sum(v, 4, red);
  if (threadIdx.x == 0) {
    const double sx = sums[2 * z], sy = sums[2 * z + 1];
    const double ex = sx / (double)n, ey = sy / (double)n;
    const double ox = ex - (double)(float)ex, oy = ey - (double)(float)ey;
    double* o = out + (size_t)z * kSumFields;
    o[0] = sx;
    o[1] = sy;
    o[2] = v[0] - (double)n * ox * ox;
    o[3] = v[1] - (double)n * ox * oy;
    o[4] = v[2] - (double)n * oy * oy;
    o[5] = v[3];
  }
}

int sum_blocks(long long n) {
  return (int)std::max<long long>(
      1, std::min<long long>(kSumMaxBlocks, (n + 256LL * kSumRun - 1) / (256LL * kSumRun)));
}

// ---------------------------------------------------------------------------
// FFT: one line of N complex values per CTA, Stockham autosort in shared
// memory.  Stage s with radix R after Ns = product of the earlier radices:
// group j < N/R, k = j mod Ns, inputs x[j + r N/R], outputs
// y[(j / Ns) Ns R + k + q Ns] = sum_r x[j + r N/R] w^(r (k + q Ns) N / (Ns R)),
// w = e^{-2 pi i / N} (one table lookup per term, exponent reduced mod N).
// ---------------------------------------------------------------------------
struct FftPlanDev {
  int N, nstages;
  int radix[24];
};

__device__ inline float2 cmul(float2 a, float2 b) {
  return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                     __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ inline float2 cadd(float2 a, float2 b) {
  return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
__device__ inline float2 csub(float2 a, float2 b) {
  return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}

// Lines of image z = 2 pair + which (blockIdx.y).
// mode 0: real input lines: row y of image `which` of the pair, at
//         (r0 + y, c0 ..) of a plane with row pitch `pitch` (planes
//         `stride` floats apart), multiplied by taper_x then taper_y as the
//         reference does
// mode 1: complex input lines (contiguous N x N per image)
// output: the transformed line written as column `line` of dst (transpose)
__global__ void __launch_bounds__(kFftThreads) fft_lines_kernel(
    const __grid_constant__ FftPlanDev plan, const float2* __restrict__ tw, int mode,
    const float* __restrict__ rsrc0, const float* __restrict__ rsrc1, long long stride, int pitch,
    int r0, int c0, const float* __restrict__ taper, const float* __restrict__ sub,
    const float2* __restrict__ csrc, float2* __restrict__ dst) {
  extern __shared__ float2 buf[];
  const int N = plan.N;
  const int line = blockIdx.x, z = blockIdx.y;
  float2* a = buf;
  float2* b = buf + N;
  if (mode == 0) {
    const float* row = ((z & 1) ? rsrc1 : rsrc0) + (size_t)(z >> 1) * stride +
                       (size_t)(r0 + line) * pitch + c0;
    if (taper) {
      const float ty = taper[line];
      for (int i = threadIdx.x; i < N; i += blockDim.x)
        a[i] = make_float2(__fmul_rn(__fmul_rn(row[i], taper[i]), ty), 0.f);
    } else if (sub) {  // high-pass line: base - sub_z (one N x N image each)
      const float* srow = sub + ((size_t)z * N + line) * N;
      for (int i = threadIdx.x; i < N; i += blockDim.x)
        a[i] = make_float2(__fsub_rn(row[i], srow[i]), 0.f);
    } else {
      for (int i = threadIdx.x; i < N; i += blockDim.x) a[i] = make_float2(row[i], 0.f);
    }
  } else {
    const float2* row = csrc + ((size_t)z * N + line) * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) a[i] = row[i];
  }
  __syncthreads();
  int Ns = 1;
  for (int s = 0; s < plan.nstages; ++s) {
    const int R = plan.radix[s];
    const int G = N / R;          // groups
    const int step = N / (Ns * R);
    for (int j = threadIdx.x; j < G; j += blockDim.x) {
      const int k = j % Ns;
      const int base = (j / Ns) * Ns * R + k;
      if (R == 2) {
        const float2 t = tw[k * step];
        const float2 u = a[j], v = cmul(a[j + G], t);
        b[base] = cadd(u, v);
        b[base + Ns] = csub(u, v);
      } else if (R == 4) {
        const float2 x0 = a[j];
        const float2 x1 = cmul(a[j + G], tw[k * step]);
        const float2 x2 = cmul(a[j + 2 * G], tw[2 * k * step]);
        const float2 x3 = cmul(a[j + 3 * G], tw[3 * k * step]);
        const float2 s02 = cadd(x0, x2), d02 = csub(x0, x2);
        const float2 s13 = cadd(x1, x3), d13 = csub(x1, x3);
        // forward transform: multiply d13 by -i
        const float2 md = make_float2(d13.y, -d13.x);
        b[base] = cadd(s02, s13);
        b[base + Ns] = cadd(d02, md);
        b[base + 2 * Ns] = csub(s02, s13);
        b[base + 3 * Ns] = csub(d02, md);
      } else {
        for (int q = 0; q < R; ++q) {
          const long long e0 = (long long)(k + q * Ns) * step;  // < N
          float2 acc = a[j];
          for (int r = 1; r < R; ++r) {
            const float2 t = tw[(int)((e0 * r) % N)];
            const float2 x = a[j + r * G];
            acc.x = fmaf(x.x, t.x, fmaf(-x.y, t.y, acc.x));
            acc.y = fmaf(x.x, t.y, fmaf(x.y, t.x, acc.y));
          }
          b[base + q * Ns] = acc;
        }
      }
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  float2* out = dst + (size_t)z * N * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) out[(size_t)i * N + line] = a[i];
}

// ring sums of the centred product images of pair blockIdx.y; one CTA per
// ring radius
__global__ void __launch_bounds__(256) frc_ring_kernel(const float2* __restrict__ F,
                                                       int N, const float2* __restrict__ pos,
                                                       const int* __restrict__ ring_start,
                                                       double* __restrict__ sums_all) {
  __shared__ double red[kSumFields * 256];
  const int r = blockIdx.x + 1;
  const float2* F1 = F + (size_t)blockIdx.y * 2 * N * N;
  const float2* F2 = F1 + (size_t)N * N;
  double* sums = sums_all + (size_t)blockIdx.y * (gridDim.x + 1) * 4;
  const int h = N / 2;
  double v[kSumFields] = {0, 0, 0, 0, 0, 0};
  const int s0 = ring_start[r - 1], s1 = ring_start[r];
  for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
    const float2 p = pos[s];
    const int xb = (int)p.x, yb = (int)p.y;
    float fx = __fsub_rn(p.x, (float)xb), fy = __fsub_rn(p.y, (float)yb);
    if (fx < 0.f) fx = 0.f;
    if (fy < 0.f) fy = 0.f;
    float c[4][3];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int yy = yb + (q >> 1), xx = xb + (q & 1);
      // fftshift: centred index i <-> spectrum index (i + N/2) mod N
      const size_t idx = (size_t)((yy + h) % N) * N + (xx + h) % N;
      const float2 u = F1[idx], w = F2[idx];
      c[q][0] = __fadd_rn(__fmul_rn(u.x, w.x), __fmul_rn(u.y, w.y));
      c[q][1] = __fadd_rn(__fmul_rn(u.x, u.x), __fmul_rn(u.y, u.y));
      c[q][2] = __fadd_rn(__fmul_rn(w.x, w.x), __fmul_rn(w.y, w.y));
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      // corners: 0 lower-left, 1 lower-right, 2 upper-left, 3 upper-right
      const float up = __fadd_rn(c[2][f], __fmul_rn(fx, __fsub_rn(c[3][f], c[2][f])));
      const float lo = __fadd_rn(c[0][f], __fmul_rn(fx, __fsub_rn(c[1][f], c[0][f])));
      v[f] += (double)__fadd_rn(lo, __fmul_rn(fy, __fsub_rn(up, lo)));
    }
  }
  block_sum(v, 3, red);
  if (threadIdx.x == 0) {
    sums[(size_t)r * 4 + 0] = v[0];
    sums[(size_t)r * 4 + 1] = v[1];
    sums[(size_t)r * 4 + 2] = v[2];
    sums[(size_t)r * 4 + 3] = (double)(s1 - s0);
  }
}


// ---------------------------------------------------------------------------
// Decorrelation analysis (src/nanopyx/core/analysis/decorr.pyx:64-118,
// 120-214 with transform/edges.pyx:9-49): edge apodisation, the padded
// square, the inscribed-disc spectral norm and the ring coefficients.
// ---------------------------------------------------------------------------
constexpr int kApodOffset = 20;  // pixels of the cosine roll-off

// sum and count of the pixels outside the circle of radius w/2 - 20
__global__ void __launch_bounds__(256) decorr_edge_kernel(const float* __restrict__ img, int h,
                                                          int w, double* __restrict__ part) {
  __shared__ double red[2 * 256];
  const float radius = (float)(w / 2 - kApodOffset);
  double v[2] = {0, 0};
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)h * w;
       e += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(e / w), x = (int)(e % w);
    const int dy = y - h / 2, dx = x - w / 2;
    const float dist = (float)(dy * dy + dx * dx);
    if (dist > radius * radius) {
      v[0] += img[e];
      v[1] += 1.0;
    }
  }
  block_sum(v, 2, red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = v[0];
    part[2 * blockIdx.x + 1] = v[1];
  }
}

__device__ __forceinline__ float decorr_apodized(const float* img, int h, int w, int y, int x,
                                                 float em) {
  const float pin = img[(size_t)y * w + x];
  const float x0 = fabsf((float)(x - w / 2)), y0 = fabsf((float)(y - h / 2));
  const double ex = fabs((double)x0 - (double)(w / 2)), ey = fabs((double)y0 - (double)(h / 2));
  if (ex <= kApodOffset || ey <= kApodOffset) {
    const float d = (float)fmin(ex, ey);
    const double pi = 3.14159265358979323846;
    const float c = (float)((cos((double)d * pi / kApodOffset - pi) + 1) / 2);
    return __fadd_rn(__fmul_rn(c, __fsub_rn(pin, em)), em);
  }
  if (abs(x - w / 2) > w / 2 && abs(y - h / 2) > h / 2) return em;
  return pin;
}

// the N x N square: the apodised image at rows 0 .. h-1, columns ox .. ox+w-1
// (ox = (N - w) / 2; the reference's copy loop leaves the row offset at 0),
// every other pixel the apodised image's first pixel
// the edge mean (float, as the reference keeps it) from the per-block sums
__global__ void __launch_bounds__(256) decorr_edge_final_kernel(const double* __restrict__ part,
                                                                int nparts,
                                                                float* __restrict__ em) {
  __shared__ double red[2 * 256];
  double v[2] = {0, 0};
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
    v[0] += part[2 * b];
    v[1] += part[2 * b + 1];
  }
  block_sum(v, 2, red);
  if (threadIdx.x == 0) *em = (float)(v[0] / v[1]);
}

__global__ void decorr_pad_kernel(const float* __restrict__ img, int h, int w, int N,
                                  const float* __restrict__ emp, float* __restrict__ out) {
  const float em = *emp;
  const float fill = decorr_apodized(img, h, w, 0, 0, em);
  const int ox = (N - w) / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)N * N;
       e += (long long)gridDim.x * blockDim.x) {
    const int yo = (int)(e / N), xo = (int)(e % N);
    float v = fill;
    if (yo < h && xo >= ox && xo < ox + w) v = decorr_apodized(img, h, w, yo, xo - ox, em);
    out[e] = v;
  }
}

// spectrum value at centred coordinates (ys, xs): natural index (+N/2 mod N);
// the DC term reads 0 when zero_dc
__device__ __forceinline__ float2 centred(const float2* F, int N, int ys, int xs, int zero_dc) {
  const int yn = (ys + N / 2) % N, xn = (xs + N / 2) % N;
  if (zero_dc && yn == 0 && xn == 0) return make_float2(0.f, 0.f);
  return F[(size_t)yn * N + xn];
}

// sum of |F|^2 over the inscribed disc: blocks (split, image) -> partials
constexpr int kDecSplits = 32;  // pixel-range splits per image (parallelism)
__global__ void __launch_bounds__(256) decorr_cr_kernel(const float2* __restrict__ Fall, int N,
                                                        int zero_dc, double* __restrict__ part) {
  __shared__ double red[2 * 256];
  const int z = blockIdx.y;
  const float2* F = Fall + (size_t)z * N * N;
  const double r2 = (double)N * N / 4;
  const long long nn = (long long)N * N;
  const long long e0 = nn * blockIdx.x / gridDim.x, e1 = nn * (blockIdx.x + 1) / gridDim.x;
  double v[2] = {0, 0};
  for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int ys = (int)(e / N), xs = (int)(e % N);
    const int dy = ys - N / 2, dx = xs - N / 2;
    if ((double)(dy * dy + dx * dx) < r2) {
      const float2 f = centred(F, N, ys, xs, zero_dc);
      v[0] += (double)__fadd_rn(__fmul_rn(f.x, f.x), __fmul_rn(f.y, f.y));
    }
  }
  block_sum(v, 1, red);
  if (threadIdx.x == 0) part[(size_t)z * gridDim.x + blockIdx.x] = v[0];
}

// the radial bin of every centred pixel for the band [crmin, crmax] (-1:
// not visited): the reference's x-major walk over the centred square
// (ox, ox + wb), stopping past x N + y = N^2/2 + N/2, bin
// round(linmap(dist)) of the float32 distance; stored at y N + x
__global__ void decorr_binmap_kernel(int N, float crmin, float crmax, int n_r,
                                     int* __restrict__ bins) {
  const int ox = (int)((float)N * (1.f - crmax) / 2.f);
  const int wb = (int)((float)N * crmax);
  const float kmax = (float)(N * N / 2 + N / 2);
  const float span = __fsub_rn(crmax, crmin), top = (float)(n_r - 1);
  const long long nn = (long long)N * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(e / N), x = (int)(e % N);
    int bin = -1;
    if (x >= ox && x < ox + wb && y >= ox && y < ox + wb && (float)(x * N + y) <= kmax) {
      const int dx = x - N / 2, dy = y - N / 2;
      float dist = (float)(dx * dx + dy * dy);
      // the reference's double sqrt of a float, rounded to float, is the
      // correctly rounded float sqrt
      dist = __fsqrt_rn(__fdiv_rn(__fmul_rn(4.f, dist), (float)N * (float)N));
      if (dist >= 0.f && dist <= crmax) {
        float m = __fmul_rn(__fdiv_rn(__fsub_rn(dist, crmin), span), top);
        if (m < 0.f) m = 0.f;
        const int d = (int)round((double)m);
        if (d < n_r) bin = d;
      }
    }
    bins[e] = bin;
  }
}

// ring coefficients: blocks (bin, image, split) sum, over the pixels of their
// bin, the float32 terms re * re/|F| + im * im/|F| and (re/|F|)^2 +
// (im/|F|)^2 (|F| in float64 from the float32 power, as the reference)
__global__ void __launch_bounds__(256) decorr_ring_kernel(const float2* __restrict__ Fall, int N,
                                                          int zero_dc,
                                                          const int* __restrict__ bins,
                                                          double* __restrict__ part) {
  __shared__ double red[2 * 256];
  const int bin = blockIdx.x, z = blockIdx.y, sp = blockIdx.z;
  const float2* F = Fall + (size_t)z * N * N;
  const long long nn = (long long)N * N;
  const long long e0 = nn * sp / gridDim.z, e1 = nn * (sp + 1) / gridDim.z;
  double v[2] = {0, 0};
  for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    if (__ldg(bins + e) != bin) continue;
    const float2 f = centred(F, N, (int)(e / N), (int)(e % N), zero_dc);
    const double mag = sqrt((double)__fadd_rn(__fmul_rn(f.x, f.x), __fmul_rn(f.y, f.y)));
    float nr = 0.f, ni = 0.f;
    if (mag != 0.0) {
      nr = (float)((double)f.x / mag);
      ni = (float)((double)f.y / mag);
    }
    v[0] += (double)__fadd_rn(__fmul_rn(f.x, nr), __fmul_rn(f.y, ni));
    v[1] += (double)__fadd_rn(__fmul_rn(nr, nr), __fmul_rn(ni, ni));
  }
  block_sum(v, 2, red);
  if (threadIdx.x == 0) {
    const size_t o = (((size_t)z * gridDim.x + bin) * gridDim.z + sp) * 2;
    part[o] = v[0];
    part[o + 1] = v[1];
  }
}

// per image: cr and the 2 n_r coefficients from the split partials, in order
__global__ void decorr_finish_kernel(const double* __restrict__ crp, int cr_splits,
                                     const double* __restrict__ ringp, int n_r, int splits,
                                     double* __restrict__ cr, double* __restrict__ coef) {
  const int z = blockIdx.x;
  for (int t = threadIdx.x; t <= n_r; t += blockDim.x) {
    if (t == n_r) {
      double c = 0;
      for (int k = 0; k < cr_splits; ++k) c += crp[(size_t)z * cr_splits + k];
      cr[z] = c;
    } else {
      double a = 0, b = 0;
      for (int k = 0; k < splits; ++k) {
        const size_t o = (((size_t)z * n_r + t) * splits + k) * 2;
        a += ringp[o];
        b += ringp[o + 1];
      }
      coef[(size_t)z * 2 * n_r + t] = a;
      coef[(size_t)z * 2 * n_r + n_r + t] = b;
    }
  }
}

BlurAxis blur_axis(double sigma, int radius, int n) {
  if (!(sigma > 1e-15)) return BlurAxis{1, 0, 0};  // scipy leaves the axis alone
  if (2LL * radius + 1 > 2LL * n) return BlurAxis{2 * n, 0, 1};
  return BlurAxis{2 * radius + 1, -radius, 0};
}

template <typename A>
int run_blur_batch(const float* d_in, int H, int W, int n, const int* src_index,
                   const double* sigma, const float* alpha, const float* beta, float* d_out,
                   char* base, cudaStream_t s) {
  const size_t plane = (size_t)H * W;
  const size_t k = (size_t)std::min(n, kBlurBatch);  // images per launch
  A* w0 = (A*)base;                                    // k x 2H weights, axis 0
  A* w1 = w0 + k * 2 * H;                              // k x 2W weights, axis 1
  float* mid = (float*)(base + ((k * (2 * (size_t)H + 2 * (size_t)W) * sizeof(double) + 255) /
                                256) * 256);
  for (int c0 = 0; c0 < n; c0 += kBlurBatch) {
    BlurBatch b{};
    b.n = std::min(kBlurBatch, n - c0);
    b.affine = alpha != nullptr;
    int max_taps0 = 1, max_taps1 = 1;
    for (int i = 0; i < b.n; ++i) {
      const int g = c0 + i;
      b.src[i] = src_index ? src_index[g] : g;
      b.sigma[i] = sigma[g];
      b.radius[i] = sigma[g] > 1e-15 ? (int)(4.0 * sigma[g] + 0.5) : 0;
      b.alpha[i] = alpha ? alpha[g] : 1.f;
      b.beta[i] = beta ? beta[g] : 0.f;
      b.ax[0][i] = blur_axis(sigma[g], b.radius[i], H);
      b.ax[1][i] = blur_axis(sigma[g], b.radius[i], W);
      max_taps0 = std::max(max_taps0, b.ax[0][i].taps);
      max_taps1 = std::max(max_taps1, b.ax[1][i].taps);
    }
    gauss_weights_kernel<A><<<dim3(b.n, 2), 256, 0, s>>>(b, H, W, w0, w1);
    NX_CUDA_TRY(cudaGetLastError());
    const int staged0 = max_taps0 <= kStageTaps;
    const size_t smem0 = staged0 ? kStageTaps * sizeof(A) +
                                       (size_t)(kTileRows + max_taps0 - 1) * kTileCols * sizeof(float)
                                 : 0;
    blur_axis0_kernel<A><<<dim3((W + kTileCols - 1) / kTileCols, (H + kTileRows - 1) / kTileRows,
                                b.n),
                           dim3(kTileCols, 256 / kTileCols), smem0, s>>>(b, d_in, H, W, w0,
                                                                         staged0, mid);
    NX_CUDA_TRY(cudaGetLastError());
    const size_t smem1 = ((size_t)max_taps1 + 3) / 4 * 4 * sizeof(A) +
                         ((size_t)kRowTile + max_taps1 - 1) * sizeof(float);
    const int staged1 = smem1 <= 48 * 1024;
    blur_axis1_kernel<A><<<dim3((W + kRowTile - 1) / kRowTile, H, b.n), 256,
                           staged1 ? smem1 : 0, s>>>(b, mid, H, W, w1, staged1,
                                                     d_out + (size_t)c0 * plane);
    NX_CUDA_TRY(cudaGetLastError());
  }
  return NX_OK;
}

}  // namespace
}  // namespace nx

// ---------------------------------------------------------------------------
// FRC plan: FFT factorisation and twiddles, Tukey taper, ring sample positions
// ---------------------------------------------------------------------------
struct nx_frc_plan {
  int N, device;
  nx::FftPlanDev fft;
  float2* tw = nullptr;
  float* taper = nullptr;
  float2* pos = nullptr;
  int* ring_start = nullptr;
  int n_rings = 0;  // rings 1 .. n_rings (the reference's r = 1 .. N/2 - 2)
};

namespace nx {
namespace {

void frc_plan_free(nx_frc_plan* p) {
  cudaFree(p->tw);
  cudaFree(p->taper);
  cudaFree(p->pos);
  cudaFree(p->ring_start);
  delete p;
}

// scipy.signal.windows.tukey(M, 0.25), symmetric, float64 then float32
std::vector<float> tukey_window(int M, double alpha) {
  std::vector<float> w(M, 1.f);
  if (M <= 1) return w;
  const double pi = 3.14159265358979323846;
  const int width = (int)std::floor(alpha * (M - 1) / 2.0);
  for (int n = 0; n < M; ++n) {
    double v = 1.0;
    if (n <= width)
      v = 0.5 * (1 + std::cos(pi * (-1 + 2.0 * n / alpha / (M - 1))));
    else if (n >= M - width - 1)
      v = 0.5 * (1 + std::cos(pi * (-2.0 / alpha + 1 + 2.0 * n / alpha / (M - 1))));
    w[n] = (float)v;
  }
  return w;
}

// radices: 4s first, then 2, 3, 5, 7, then remaining prime factors
bool fft_factor(int N, FftPlanDev& f) {
  f.N = N;
  f.nstages = 0;
  int n = N;
  auto push = [&](int r) {
    if (f.nstages >= 24) return false;
    f.radix[f.nstages++] = r;
    n /= r;
    return true;
  };
  while (n % 4 == 0)
    if (!push(4)) return false;
  for (int p : {2, 3, 5, 7})
    while (n % p == 0)
      if (!push(p)) return false;
  for (int p = 11; (long long)p * p <= n; p += 2)
    while (n % p == 0)
      if (!push(p)) return false;
  if (n > 1 && !push(n)) return false;
  return true;
}

template <class T>
int upload(const std::vector<T>& h, T** d) {
  cudaError_t e = cudaMalloc(d, std::max<size_t>(1, h.size()) * sizeof(T));
  if (e == cudaSuccess && !h.empty())
    e = cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? NX_OK : cuda_status(e, "FRC plan upload");
}

}  // namespace
}  // namespace nx

using namespace nx;

extern "C" {

size_t nx_gaussian_blur_batch_workspace_bytes(int H, int W, int n) {
  if (H < 1 || W < 1 || n < 1) return 256;
  const size_t k = (size_t)std::min(n, kBlurBatch);
  return 256 + ((k * (2 * (size_t)H + 2 * (size_t)W) * sizeof(double) + 255) / 256) * 256 +
         k * H * W * sizeof(float);
}

int nx_gaussian_blur_batch_ex(const float* d_in, int H, int W, int n, const int* src_index,
                              const double* sigma, const float* alpha, const float* beta,
                              int flags, float* d_out, void* d_ws, size_t ws_bytes,
                              void* stream) {
  if (H < 1 || W < 1 || n < 0) return nx::set_error("need H, W >= 1, n >= 0"), NX_ERR_INVALID_ARG;
  if (n == 0) return NX_OK;
  if (!d_in || !d_out || !sigma) return nx::set_error("NULL pointer"), NX_ERR_INVALID_ARG;
  if ((alpha == nullptr) != (beta == nullptr))
    return nx::set_error("alpha and beta go together"), NX_ERR_INVALID_ARG;
  if (flags & ~NX_BLUR_FLOAT64_SUMS) return nx::set_error("unknown blur flags"), NX_ERR_INVALID_ARG;
  if (!d_ws || ws_bytes < nx_gaussian_blur_batch_workspace_bytes(H, W, n)) {
    nx::set_error("workspace too small: need %zu bytes",
                  nx_gaussian_blur_batch_workspace_bytes(H, W, n));
    return NX_ERR_WORKSPACE;
  }
  for (int i = 0; i < n; ++i) {
    if (!(sigma[i] <= 1e7)) return nx::set_error("sigma must be <= 1e7"), NX_ERR_INVALID_ARG;
    if (src_index && src_index[i] < 0) return nx::set_error("negative image index"), NX_ERR_INVALID_ARG;
  }
  char* base = (char*)d_ws + 256;
  cudaStream_t s = (cudaStream_t)stream;
  return (flags & NX_BLUR_FLOAT64_SUMS)
             ? run_blur_batch<double>(d_in, H, W, n, src_index, sigma, alpha, beta, d_out, base, s)
             : run_blur_batch<float>(d_in, H, W, n, src_index, sigma, alpha, beta, d_out, base, s);
}

int nx_gaussian_blur_batch(const float* d_in, int H, int W, int n, const int* src_index,
                           const double* sigma, const float* alpha, const float* beta,
                           float* d_out, void* d_ws, size_t ws_bytes, void* stream) {
  return nx_gaussian_blur_batch_ex(d_in, H, W, n, src_index, sigma, alpha, beta, 0, d_out, d_ws,
                                   ws_bytes, stream);
}

size_t nx_gaussian_blur_workspace_bytes(int H, int W) {
  return nx_gaussian_blur_batch_workspace_bytes(H, W, 1);
}

int nx_gaussian_blur(const float* d_in, int H, int W, double sigma, int affine, float alpha,
                     float beta, float* d_out, void* d_ws, size_t ws_bytes, void* stream) {
  if (d_in && d_in == d_out) return nx::set_error("blur cannot run in place"), NX_ERR_INVALID_ARG;
  return nx_gaussian_blur_batch(d_in, H, W, 1, nullptr, &sigma, affine ? &alpha : nullptr,
                                affine ? &beta : nullptr, d_out, d_ws, ws_bytes, stream);
}

size_t nx_moment_sums_workspace_bytes(int batch) {
  const size_t b = (size_t)std::max(batch, 1);
  return 256 + b * kSumMaxBlocks * 4 * sizeof(double) + b * 2 * sizeof(double) +
         b * 2 * sizeof(float);
}

int nx_moment_sums(const float* d_x, const float* d_y, long long n, int batch, double* d_sums,
                   void* d_ws, size_t ws_bytes, void* stream) {
  if (n < 1 || batch < 1) return nx::set_error("need n >= 1, batch >= 1"), NX_ERR_INVALID_ARG;
  if (!d_x || !d_y || !d_sums) return nx::set_error("NULL pointer"), NX_ERR_INVALID_ARG;
  if (batch > 65535) return nx::set_error("batch must be <= 65535"), NX_ERR_INVALID_ARG;
  if (!d_ws || ws_bytes < nx_moment_sums_workspace_bytes(batch)) {
    nx::set_error("workspace too small: need %zu bytes", nx_moment_sums_workspace_bytes(batch));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)((char*)d_ws + 256);                    // batch x blocks x 4
  double* means = part + (size_t)batch * kSumMaxBlocks * 4;       // batch x 2 (the sums)
  float* fmeans = (float*)(means + (size_t)batch * 2);            // batch x 2
  const int nb = sum_blocks(n);
  moment_mean_kernel<<<dim3(nb, batch), 256, 0, s>>>(d_x, d_y, n, part);
  NX_CUDA_TRY(cudaGetLastError());
  moment_mean_final_kernel<<<batch, 256, 0, s>>>(part, nb, n, means, fmeans);
  NX_CUDA_TRY(cudaGetLastError());
  moment_centred_kernel<<<dim3(nb, batch), 256, 0, s>>>(d_x, d_y, n, fmeans, part);
  NX_CUDA_TRY(cudaGetLastError());
  moment_final_kernel<<<batch, 256, 0, s>>>(part, nb, n, means, d_sums);
  NX_CUDA_TRY(cudaGetLastError());
  return NX_OK;
}

int nx_frc_plan_create(nx_frc_plan** out, int N) {
  if (!out) return nx::set_error("plan out-pointer is NULL"), NX_ERR_INVALID_ARG;
  *out = nullptr;
  if (N < 6 || N % 2 || N > kMaxFftN)
    return nx::set_error("FRC size must be even and in [6, %d]", kMaxFftN), NX_ERR_INVALID_ARG;
  auto* p = new nx_frc_plan();
  p->N = N;
  cudaGetDevice(&p->device);
  if (!fft_factor(N, p->fft)) {
    delete p;
    return nx::set_error("FFT size %d has too many factors", N), NX_ERR_INVALID_ARG;
  }
  const double pi = 3.14159265358979323846;
  std::vector<float2> tw(N);
  for (int k = 0; k < N; ++k) {
    const double a = -2.0 * pi * (double)k / N;
    tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  // ring sample positions, r = 1 .. max_r - 1 with max_r = N/2 - 1
  // (frc.pyx:150-179): angles fl32(i * fl32(1/r)) below fl32(2 pi), then
  // x = max_r + 1 + r cos, y = max_r + 1 + r sin, sin = +-sqrt(1 - cos^2)
  const int max_r = N / 2 - 1;
  p->n_rings = max_r - 1;
  std::vector<float2> pos;
  std::vector<int> start{0};
  const float limit = (float)(pi * 2);
  for (int r = 1; r < max_r; ++r) {
    const float step = (float)(1.0 / r);
    const long long cnt = (long long)std::ceil((double)limit / (double)step);
    for (long long i = 0; i < cnt; ++i) {
      const float ang = (float)i * step;
      const float ca = (float)std::cos((double)ang);
      const float c2 = ca * ca;
      const float om = 1.0f - c2;
      double sn = std::sqrt((double)om);
      if ((double)ang > pi) sn = -sn;  // the reference compares with the double pi
      const float sa = (float)sn;
      const float rf = (float)r;
      const float x = (float)(max_r + 1) + rf * ca;
      const float y = (float)(max_r + 1) + rf * sa;
      pos.push_back(make_float2(x, y));
    }
    start.push_back((int)pos.size());
  }
  int rc = upload(tw, &p->tw);
  if (!rc) rc = upload(tukey_window(N, 0.25), &p->taper);
  if (!rc) rc = upload(pos, &p->pos);
  if (!rc) rc = upload(start, &p->ring_start);
  if (rc) {
    frc_plan_free(p);
    return rc;
  }
  const int smem = 2 * N * (int)sizeof(float2);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fft_lines_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) {
      frc_plan_free(p);
      return cuda_status(e, "FFT shared memory");
    }
  }
  *out = p;
  return NX_OK;
}

int nx_frc_plan_destroy(nx_frc_plan* p) {
  if (p) frc_plan_free(p);
  return NX_OK;
}

int nx_frc_rings(const nx_frc_plan* p) { return p ? p->n_rings : 0; }

size_t nx_frc_workspace_bytes(const nx_frc_plan* p, int pairs) {
  if (!p || pairs < 1) return 256;
  return 256 + (size_t)4 * std::min(pairs, kFrcChunk) * p->N * p->N * sizeof(float2);
}

int nx_frc_ring_sums(const nx_frc_plan* p, const float* d_img1, const float* d_img2, int pairs,
                     long long stride, int pitch, int r0, int c0, double* d_sums, void* d_ws,
                     size_t ws_bytes, void* stream) {
  if (!p) return nx::set_error("plan is NULL"), NX_ERR_INVALID_ARG;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->device) return nx::set_error("plan made on another device"), NX_ERR_INVALID_ARG;
  if (pairs < 0) return nx::set_error("pairs must be >= 0"), NX_ERR_INVALID_ARG;
  if (pairs == 0) return NX_OK;
  if (!d_img1 || !d_img2 || !d_sums) return nx::set_error("NULL pointer"), NX_ERR_INVALID_ARG;
  if (pitch < p->N || r0 < 0 || c0 < 0 || c0 + p->N > pitch)
    return nx::set_error("crop window outside the image rows"), NX_ERR_INVALID_ARG;
  if (pairs > 1 && stride < (long long)(r0 + p->N) * pitch)
    return nx::set_error("image stride smaller than the crop window"), NX_ERR_INVALID_ARG;
  if (!d_ws || ws_bytes < nx_frc_workspace_bytes(p, pairs)) {
    nx::set_error("workspace too small: need %zu bytes", nx_frc_workspace_bytes(p, pairs));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int N = p->N;
  const int chunk = std::min(pairs, kFrcChunk);
  float2* T = (float2*)((char*)d_ws + 256);  // (2 chunk, N, N): transposed after pass 1
  float2* F = T + (size_t)2 * chunk * N * N;  // (2 chunk, N, N): spectra, natural layout
  const int smem = 2 * N * (int)sizeof(float2);
  const size_t rows = (size_t)p->n_rings + 1;
  for (int q0 = 0; q0 < pairs; q0 += chunk) {
    const int q = std::min(chunk, pairs - q0);
    fft_lines_kernel<<<dim3(N, 2 * q), kFftThreads, smem, s>>>(
        p->fft, p->tw, 0, d_img1 + (size_t)q0 * stride, d_img2 + (size_t)q0 * stride, stride,
        pitch, r0, c0, p->taper, nullptr, nullptr, T);
    NX_CUDA_TRY(cudaGetLastError());
    fft_lines_kernel<<<dim3(N, 2 * q), kFftThreads, smem, s>>>(
        p->fft, p->tw, 1, nullptr, nullptr, 0, 0, 0, 0, p->taper, nullptr, T, F);
    NX_CUDA_TRY(cudaGetLastError());
    double* out = d_sums + (size_t)q0 * rows * 4;
    NX_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)q * rows * 4 * sizeof(double), s));
    frc_ring_kernel<<<dim3(p->n_rings, q), 256, 0, s>>>(F, N, p->pos, p->ring_start, out);
    NX_CUDA_TRY(cudaGetLastError());
  }
  return NX_OK;
}

size_t nx_decorr_prepare_workspace_bytes(int h, int w) {
  (void)h;
  (void)w;
  return 256 + 2 * 1024 * sizeof(double) + 256;
}

int nx_decorr_prepare(const float* d_img, int h, int w, float* d_out, int N, void* d_ws,
                      size_t ws_bytes, void* stream) {
  if (h < 1 || w < 1 || N < h || N < w) return nx::set_error("bad decorrelation image shape"), NX_ERR_INVALID_ARG;
  if (!d_img || !d_out) return nx::set_error("NULL pointer"), NX_ERR_INVALID_ARG;
  if (!d_ws || ws_bytes < nx_decorr_prepare_workspace_bytes(h, w))
    return nx::set_error("workspace too small"), NX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)((char*)d_ws + 256);
  float* em = (float*)(part + 2 * 1024);
  const int nb = (int)std::min<long long>(1024, ((long long)h * w + 255) / 256);
  decorr_edge_kernel<<<nb, 256, 0, s>>>(d_img, h, w, part);
  NX_CUDA_TRY(cudaGetLastError());
  decorr_edge_final_kernel<<<1, 256, 0, s>>>(part, nb, em);
  NX_CUDA_TRY(cudaGetLastError());
  const long long n = (long long)N * N;
  decorr_pad_kernel<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, s>>>(
      d_img, h, w, N, em, d_out);
  NX_CUDA_TRY(cudaGetLastError());
  return NX_OK;
}

size_t nx_decorr_coefs_workspace_bytes(const nx_frc_plan* p, int B, int n_r) {
  if (!p || B < 1 || n_r < 1) return 256;
  // spectra and transposes, the bin map, the split partials of cr and the rings
  return 256 + (size_t)2 * B * p->N * p->N * sizeof(float2) +
         ((size_t)p->N * p->N + 64) * sizeof(int) + 256 +
         (size_t)B * kDecSplits * sizeof(double) +
         (size_t)B * n_r * kDecSplits * 2 * sizeof(double);
}

int nx_decorr_coefs(const nx_frc_plan* p, const float* d_base, const float* d_sub, int B,
                    int zero_dc, float crmin, float crmax, int n_r, double* d_cr,
                    double* d_coef, void* d_ws, size_t ws_bytes, void* stream) {
  if (!p) return nx::set_error("plan is NULL"), NX_ERR_INVALID_ARG;
  if (B < 1 || B > 65535 || n_r < 2 || n_r > 65535)
    return nx::set_error("need 1 <= B <= 65535, 2 <= n_r <= 65535"), NX_ERR_INVALID_ARG;
  if (!d_base || !d_cr || !d_coef) return nx::set_error("NULL pointer"), NX_ERR_INVALID_ARG;
  if (!(crmax > crmin) || !(crmax <= 1.f))
    return nx::set_error("need crmin < crmax <= 1"), NX_ERR_INVALID_ARG;
  if (!d_ws || ws_bytes < nx_decorr_coefs_workspace_bytes(p, B, n_r)) {
    nx::set_error("workspace too small: need %zu bytes",
                  nx_decorr_coefs_workspace_bytes(p, B, n_r));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int N = p->N;
  float2* T = (float2*)((char*)d_ws + 256);
  float2* F = T + (size_t)B * N * N;
  const int smem = 2 * N * (int)sizeof(float2);
  // image z: d_base - d_sub[z] with a subtrahend, else d_base[z]
  const long long nn = (long long)N * N;
  const float* r0 = d_base;
  const float* r1 = d_sub ? d_base : d_base + nn;
  const long long stride = d_sub ? 0 : 2 * nn;
  fft_lines_kernel<<<dim3(N, B), kFftThreads, smem, s>>>(p->fft, p->tw, 0, r0, r1, stride, N, 0,
                                                         0, nullptr, d_sub, nullptr, T);
  NX_CUDA_TRY(cudaGetLastError());
  fft_lines_kernel<<<dim3(N, B), kFftThreads, smem, s>>>(p->fft, p->tw, 1, nullptr, nullptr, 0, 0,
                                                         0, 0, nullptr, nullptr, T, F);
  NX_CUDA_TRY(cudaGetLastError());
  int* bins = (int*)(F + (size_t)B * N * N);
  double* crp = (double*)(bins + (size_t)N * N + 64);
  crp = (double*)(((uintptr_t)crp + 255) & ~(uintptr_t)255);
  double* ringp = crp + (size_t)B * kDecSplits;
  const unsigned nb = (unsigned)std::min<long long>((nn + 255) / 256, 4096);
  decorr_binmap_kernel<<<nb, 256, 0, s>>>(N, crmin, crmax, n_r, bins);
  NX_CUDA_TRY(cudaGetLastError());
  decorr_cr_kernel<<<dim3(kDecSplits, B), 256, 0, s>>>(F, N, zero_dc, crp);
  NX_CUDA_TRY(cudaGetLastError());
  const int splits = (int)std::max<long long>(1, std::min<long long>(kDecSplits, nn / 4096));
  decorr_ring_kernel<<<dim3(n_r, B, splits), 256, 0, s>>>(F, N, zero_dc, bins, ringp);
  NX_CUDA_TRY(cudaGetLastError());
  decorr_finish_kernel<<<B, 64, 0, s>>>(crp, kDecSplits, ringp, n_r, splits, d_cr, d_coef);
  NX_CUDA_TRY(cudaGetLastError());
  return NX_OK;
}

}  // extern "C"
