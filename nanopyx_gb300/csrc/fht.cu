// Fourier ("FHT") interpolation of the use_fht=True eSRRF path
// (src/nanopyx/core/transform/interpolation.py:22-290; used by
// _le_esrrf.pyx:183-188), on the GPU as dense linear algebra.
//
// The reference interpolates a frame (or a 256-pixel tile of it) by
//   1. tiling it with alternating mirror images and cropping the central
//      N x N square, N the power of two covering both sides;
//   2. moving its spectrum (real FFT along x, complex along y) into an
//      L x L zero spectrum, L = N mag (the upper half of the y frequencies to
//      the top end), inverting, and
//   3. rescaling the result onto the frame's [min, max] and cropping the
//      central (mag h) x (mag w) window;
// frames over 256 px a side are done in overlapping 256-pixel tiles blended
// with Hann windows.  Steps 1-2 are linear and separable:
//   Z = A_re X C_re^T - A_im X C_im^T,
//   A[i][n] = (1/L) sum_{f=-(N-N2)}^{N2-1} e^{2 pi i f (i/L - n/N)}, N2 = ceil(N/2)
//   C[j][m] = (1/L) sum_{k=0}^{N/2} c_k e^{2 pi i k (j/L - m/N)}, c_0 = 1, else 2
// (the one unpaired y frequency makes A complex; the half spectrum along x
// gives C), so the interpolation is two batched FP32 GEMMs with operators
// formed once in float64 on the host.  FP32 on the CUDA cores, not TF32 on the
// tensor cores: the reference transforms in float64, and a 10-bit mantissa
// would not hold the 1e-4 parity bar.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace nx {
namespace {

constexpr int kFhtTile = 256;     // tile side of the reference's tiled path
constexpr int kFhtOverlap = 16;
constexpr int kFhtChunk = 8;      // frames per GEMM batch

int pow2_ceil(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

// ---------------------------------------------------------------------------
// batched FP32 GEMM, row major: C = A B, 64 x 64 tiles, 4 x 4 per thread
// ---------------------------------------------------------------------------
struct GemmBatch {
  int inner;                    // batch index z = outer * inner + inner_index
  long long sa_o, sa_i, sb_o, sb_i, sc_o, sc_i;
};

constexpr int kGB = 64, kGK = 16;

__global__ void __launch_bounds__(256) sgemm_kernel(const float* __restrict__ A,
                                                    const float* __restrict__ B,
                                                    float* __restrict__ C, int M, int N, int K,
                                                    int lda, int ldb, int ldc, GemmBatch bt) {
  __shared__ __align__(16) float As[kGK][kGB + 4];
  __shared__ __align__(16) float Bs[kGK][kGB + 4];
  const int zo = blockIdx.z / bt.inner, zi = blockIdx.z % bt.inner;
  A += zo * bt.sa_o + zi * bt.sa_i;
  B += zo * bt.sb_o + zi * bt.sb_i;
  C += zo * bt.sc_o + zi * bt.sc_i;
  const int m0 = blockIdx.y * kGB, n0 = blockIdx.x * kGB;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kGK) {
    for (int e = threadIdx.x; e < kGB * kGK; e += 256) {
      const int r = e / kGK, c = e % kGK;  // A tile: row r, column c
      const int gm = m0 + r, gk = k0 + c;
      As[c][r] = (gm < M && gk < K) ? __ldg(A + (size_t)gm * lda + gk) : 0.f;
      const int br = e / kGB, bc = e % kGB;  // B tile: row br, column bc
      const int bk = k0 + br, bn = n0 + bc;
      Bs[br][bc] = (bk < K && bn < N) ? __ldg(B + (size_t)bk * ldb + bn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kGK; ++k) {
      const float4 a = *reinterpret_cast<const float4*>(&As[k][ty * 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[k][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn < N) C[(size_t)gm * ldc + gn] = acc[i][j];
    }
  }
}

cudaError_t gemm(const float* A, const float* B, float* C, int M, int N, int K, int lda, int ldb,
                 int ldc, int batches, const GemmBatch& bt, cudaStream_t s) {
  const dim3 grid((unsigned)((N + kGB - 1) / kGB), (unsigned)((M + kGB - 1) / kGB),
                  (unsigned)batches);
  sgemm_kernel<<<grid, 256, 0, s>>>(A, B, C, M, N, K, lda, ldb, ldc, bt);
  return cudaGetLastError();
}

// order-preserving int image of a float, for atomicMin / atomicMax
__device__ __forceinline__ int ordered(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unordered(int i) {
  return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

__device__ __forceinline__ void block_minmax(float lo, float hi, int* slot) {
  __shared__ float slo[32], shi[32];
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    slo[w] = lo;
    shi[w] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < nw; ++k) {
      lo = fminf(lo, slo[k]);
      hi = fmaxf(hi, shi[k]);
    }
    atomicMin(slot, ordered(lo));
    atomicMax(slot + 1, ordered(hi));
  }
}

// mirror-padded N x N square of tile (r0, c0, th, tw) of every frame of the
// chunk; slot[z] = (min, max) of the tile (every tile pixel is in the square:
// the upright centre copy lies inside the central crop)
__global__ void fht_gather_kernel(const float* __restrict__ in, int H, int W, int r0, int c0,
                                  int th, int tw, int N, int kh, int kw, int y_roi, int x_roi,
                                  float* __restrict__ X, int* __restrict__ mm) {
  const int z = blockIdx.y;
  const float* f = in + (size_t)z * H * W;
  float lo = INFINITY, hi = -INFINITY;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * N; e += gridDim.x * blockDim.x) {
    const int y = e / N, x = e % N;
    const int yp = y + y_roi, xp = x + x_roi;
    const int cy = yp / th, yy = yp % th, cx = xp / tw, xx = xp % tw;
    const int row = ((cy - (kh - 1) / 2) & 1) ? th - 1 - yy : yy;
    const int col = ((cx - (kw - 1) / 2) & 1) ? tw - 1 - xx : xx;
    const float v = __ldg(f + (size_t)(r0 + row) * W + (c0 + col));
    X[(size_t)z * N * N + e] = v;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  block_minmax(lo, hi, mm + 4 * z);
}

__global__ void fht_mm_init_kernel(int* __restrict__ mm, int n) {
  for (int k = threadIdx.x; k < 4 * n; k += blockDim.x) mm[k] = (k & 1) ? INT_MIN : INT_MAX;
}

__global__ void fht_zminmax_kernel(const float* __restrict__ Z, long long n,
                                   int* __restrict__ mm) {
  const int z = blockIdx.y;
  const float* p = Z + (size_t)z * n;
  float lo = INFINITY, hi = -INFINITY;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const float v = p[e];
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  block_minmax(lo, hi, mm + 4 * z + 2);
}

// rescale onto the tile's [min, max] (the reference's float32 steps
// -= out_min, *= scale, += orig_min), crop, and either store (one piece) or
// add the Hann-weighted piece (tiled: output += piece * outer(wr, wc)).
// The scale is a float64 quotient of the float32 extremes rounded once
// (interpolation.py takes the extremes as Python floats), or float32
// arithmetic throughout (f32_scale: _interpolation.pyx keeps them in C floats).
__global__ void fht_finish_kernel(const float* __restrict__ Z, int L, const int* __restrict__ mm,
                                  int oh, int ow, int y_roi, int x_roi,
                                  const float* __restrict__ wr, const float* __restrict__ wc,
                                  float* __restrict__ out, int outH, int outW, int R0, int C0,
                                  int f32_scale) {
  const int z = blockIdx.y;
  const float lo = unordered(mm[4 * z]), hi = unordered(mm[4 * z + 1]);
  const float zlo = unordered(mm[4 * z + 2]), zhi = unordered(mm[4 * z + 3]);
  const bool resc = zhi != zlo;
  float scale = 1.f;
  if (resc)
    scale = f32_scale ? __fdiv_rn(__fsub_rn(hi, lo), __fsub_rn(zhi, zlo))
                      : __double2float_rn(__ddiv_rn((double)hi - (double)lo,
                                                    (double)zhi - (double)zlo));
  const float* zp = Z + (size_t)z * L * L;
  float* o = out + (size_t)z * outH * outW;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)oh * ow;
       e += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(e / ow), x = (int)(e % ow);
    float v = zp[(size_t)(y_roi + y) * L + (x_roi + x)];
    if (resc) v = __fadd_rn(__fmul_rn(__fsub_rn(v, zlo), scale), lo);
    const size_t oi = (size_t)(R0 + y) * outW + (C0 + x);
    if (wr) {
      const float win = __fmul_rn(wr[y], wc[x]);
      o[oi] = __fadd_rn(o[oi], __fmul_rn(v, win));
    } else {
      o[oi] = v;
    }
  }
}

__global__ void fht_weight_kernel(const float* __restrict__ wr, const float* __restrict__ wc,
                                  int oh, int ow, float* __restrict__ wgt, int outW, int R0,
                                  int C0) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)oh * ow;
       e += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(e / ow), x = (int)(e % ow);
    const size_t oi = (size_t)(R0 + y) * outW + (C0 + x);
    wgt[oi] = __fadd_rn(wgt[oi], __fmul_rn(wr[y], wc[x]));
  }
}

__global__ void fht_normalize_kernel(float* __restrict__ out, const float* __restrict__ wgt,
                                     long long plane, int frames) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < plane * frames;
       e += (long long)gridDim.x * blockDim.x) {
    const float w = wgt[e % plane];
    if (w > 0.f) out[e] = __fdiv_rn(out[e], w);
  }
}

unsigned blocks_for(long long n, int per = 256, long long cap = 4096) {
  return (unsigned)std::max<long long>(1, std::min<long long>((n + per - 1) / per, cap));
}

}  // namespace
}  // namespace nx

// ---------------------------------------------------------------------------
// plan: tile layout, operators per padded size, windows, blending weights
// ---------------------------------------------------------------------------
struct nx_fht_plan {
  struct Ops {
    int N, L;
    float* ct;    // [2][N][L]: C_re^T then C_im^T
    float* acat;  // [L][2N]: A_re | -A_im
  };
  struct Tile {
    int r0, c0, th, tw, ops, kh, kw, y_roi, x_roi;
    float *wr, *wc;  // Hann windows (tiled path), device
  };
  int H, W, mag, device, variant;
  bool tiled;
  std::vector<Ops> ops;
  std::vector<Tile> tiles;
  std::vector<float*> bufs;  // every device allocation of the plan
  float* wgt = nullptr;      // (H mag, W mag) blending weights (tiled path)
  size_t frame_floats = 0;   // workspace floats per frame of a chunk
};

namespace nx {
namespace {

std::vector<int> tile_starts(int dim) {
  const int step = std::max(1, kFhtTile - 2 * kFhtOverlap);
  std::vector<int> s;
  for (int v = 0; v < dim; v += step) s.push_back(v);
  if (!s.empty() && s.back() + kFhtTile < dim) s.push_back(std::max(0, dim - kFhtTile));
  return s;
}

// The float64 operators of one padded size, rounded once to float.  Both sums
// are geometric series: sum_{f=a}^{b} e^{2 pi i f t} = e^{i pi (a+b) t}
// sin(pi (b-a+1) t) / sin(pi t), and (b - a + 1) at t = 0 -- the only integer
// phase, since t = (i - n mag) / L lies in (-1, 1).  With |t| >= 1 / L the
// quotient is well conditioned.
// full: both axes keep the whole complex spectrum f = -N/2 .. N/2-1 (the
// fft2 / centred-block / ifft2 form of _interpolation.pyx:153-200), i.e. C = A.
void build_ops(int N, int mag, bool full, std::vector<float>& ct, std::vector<float>& acat) {
  const int L = N * mag;
  const int N2 = (N + 1) / 2;
  const int fa = -(N - N2), fb = N2 - 1;  // y frequencies kept
  const int K = N / 2;                    // x frequencies kept: 0 .. K
  const double pi = 3.14159265358979323846;
  ct.assign((size_t)2 * N * L, 0.f);
  acat.assign((size_t)L * 2 * N, 0.f);
  for (int i = 0; i < L; ++i)
    for (int n = 0; n < N; ++n) {
      const double t = (double)(i - n * mag) / L;  // i / L - n / N
      const bool zero = i == n * mag;
      // A: sum over f = fa .. fb
      const double da = zero ? (double)(fb - fa + 1)
                             : std::sin(pi * (fb - fa + 1) * t) / std::sin(pi * t);
      const double pa = pi * (fa + fb) * t;
      acat[(size_t)i * 2 * N + n] = (float)(std::cos(pa) * da / L);
      acat[(size_t)i * 2 * N + N + n] = (float)(-std::sin(pa) * da / L);
      if (full) {
        ct[(size_t)n * L + i] = acat[(size_t)i * 2 * N + n];
        ct[(size_t)N * L + (size_t)n * L + i] = (float)(std::sin(pa) * da / L);
        continue;
      }
      // C: 2 sum_{k=0}^{K} e^{2 pi i k t} - 1
      const double dc = zero ? (double)(K + 1) : std::sin(pi * (K + 1) * t) / std::sin(pi * t);
      const double pc = pi * K * t;
      ct[(size_t)n * L + i] = (float)((2.0 * std::cos(pc) * dc - 1.0) / L);
      ct[(size_t)N * L + (size_t)n * L + i] = (float)(2.0 * std::sin(pc) * dc / L);
    }
}

std::vector<float> hann_inner(int n) {
  // numpy.hanning(n + 2)[1:-1] cast to float32
  std::vector<float> w(n);
  const double pi = 3.14159265358979323846;
  for (int k = 1; k <= n; ++k) w[k - 1] = (float)(0.5 - 0.5 * std::cos(2.0 * pi * k / (n + 1)));
  return w;
}

int fht_upload(nx_fht_plan* p, const std::vector<float>& h, float** out) {
  float* d = nullptr;
  cudaError_t e = cudaMalloc(&d, h.size() * sizeof(float));
  if (e != cudaSuccess) return cuda_status(e, "FHT plan allocation");
  p->bufs.push_back(d);
  e = cudaMemcpy(d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e, "FHT plan upload");
  *out = d;
  return NX_OK;
}

void fht_plan_free(nx_fht_plan* p) {
  for (float* b : p->bufs) cudaFree(b);
  delete p;
}

}  // namespace
}  // namespace nx

using namespace nx;

extern "C" {

int nx_fht_plan_create(nx_fht_plan** out, int H, int W, int magnification) {
  return nx_fht_plan_create_ex(out, H, W, magnification, NX_FHT_TILED);
}

int nx_fht_plan_create_ex(nx_fht_plan** out, int H, int W, int magnification, int variant) {
  if (!out) return nx::set_error("plan out-pointer is NULL"), NX_ERR_INVALID_ARG;
  if (variant != NX_FHT_TILED && variant != NX_FHT_FULL_SPECTRUM)
    return nx::set_error("unknown Fourier interpolation variant %d", variant), NX_ERR_INVALID_ARG;
  *out = nullptr;
  if (H < 1 || W < 1) return nx::set_error("image must have H, W >= 1"), NX_ERR_INVALID_ARG;
  if (magnification < 1 || magnification > 64)
    return nx::set_error("magnification must be in [1, 64]"), NX_ERR_INVALID_ARG;
  if ((long long)H * magnification >= (1LL << 30) || (long long)W * magnification >= (1LL << 30))
    return nx::set_error("magnified image too large"), NX_ERR_INVALID_ARG;
  auto* p = new nx_fht_plan();
  p->H = H;
  p->W = W;
  p->mag = magnification;
  p->variant = variant;
  cudaGetDevice(&p->device);
  p->tiled = variant == NX_FHT_TILED && (H > kFhtTile || W > kFhtTile);
  std::vector<int> rs{0}, cs{0};
  if (p->tiled) {
    rs = tile_starts(H);
    cs = tile_starts(W);
  }
  for (int r0 : rs)
    for (int c0 : cs) {
      nx_fht_plan::Tile t{};
      t.r0 = r0;
      t.c0 = c0;
      t.th = p->tiled ? std::min(r0 + kFhtTile, H) - r0 : H;
      t.tw = p->tiled ? std::min(c0 + kFhtTile, W) - c0 : W;
      const int N = std::max(pow2_ceil(t.th), pow2_ceil(t.tw));
      t.kh = (N + t.th - 1) / t.th;
      t.kh += 1 - t.kh % 2;  // odd number of copies
      t.kw = (N + t.tw - 1) / t.tw;
      t.kw += 1 - t.kw % 2;
      t.y_roi = (t.kh * t.th - N) / 2;
      t.x_roi = (t.kw * t.tw - N) / 2;
      t.ops = -1;
      for (size_t k = 0; k < p->ops.size(); ++k)
        if (p->ops[k].N == N) t.ops = (int)k;
      if (t.ops < 0) {
        nx_fht_plan::Ops o{N, N * magnification, nullptr, nullptr};
        std::vector<float> ct, acat;
        build_ops(N, magnification, variant == NX_FHT_FULL_SPECTRUM, ct, acat);
        int rc = fht_upload(p, ct, &o.ct);
        if (!rc) rc = fht_upload(p, acat, &o.acat);
        if (rc) {
          fht_plan_free(p);
          return rc;
        }
        p->ops.push_back(o);
        t.ops = (int)p->ops.size() - 1;
      }
      if (p->tiled) {
        int rc = fht_upload(p, hann_inner(t.th * magnification), &t.wr);
        if (!rc) rc = fht_upload(p, hann_inner(t.tw * magnification), &t.wc);
        if (rc) {
          fht_plan_free(p);
          return rc;
        }
      }
      p->tiles.push_back(t);
    }
  for (const auto& o : p->ops)
    p->frame_floats = std::max(p->frame_floats,
                               (size_t)o.N * o.N + (size_t)2 * o.N * o.L + (size_t)o.L * o.L);
  if (p->tiled) {
    // blending weights: the windows summed in the reference's tile order
    const size_t plane = (size_t)H * magnification * W * magnification;
    cudaError_t e = cudaMalloc(&p->wgt, plane * sizeof(float));
    if (e == cudaSuccess) p->bufs.push_back(p->wgt);
    if (e == cudaSuccess) e = cudaMemset(p->wgt, 0, plane * sizeof(float));
    for (const auto& t : p->tiles) {
      if (e != cudaSuccess) break;
      const long long n = (long long)t.th * magnification * t.tw * magnification;
      fht_weight_kernel<<<blocks_for(n), 256>>>(t.wr, t.wc, t.th * magnification,
                                                t.tw * magnification, p->wgt,
                                                W * magnification, t.r0 * magnification,
                                                t.c0 * magnification);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      const int rc = cuda_status(e, "FHT plan weights");
      fht_plan_free(p);
      return rc;
    }
  }
  *out = p;
  return NX_OK;
}

int nx_fht_plan_destroy(nx_fht_plan* p) {
  if (p) fht_plan_free(p);
  return NX_OK;
}

size_t nx_fht_workspace_bytes(const nx_fht_plan* p, int T) {
  if (!p || T < 1) return 256;
  const size_t tc = (size_t)std::min(T, kFhtChunk);
  return 256 + ((tc * p->frame_floats * sizeof(float) + 255) / 256) * 256 +
         tc * 4 * sizeof(int);
}

int nx_fht_interpolate(const nx_fht_plan* p, const float* d_in, int T, float* d_out, void* d_ws,
                       size_t ws_bytes, void* stream) {
  if (!p) return nx::set_error("plan is NULL"), NX_ERR_INVALID_ARG;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->device) return nx::set_error("plan made on another device"), NX_ERR_INVALID_ARG;
  if (T < 0) return nx::set_error("T must be >= 0"), NX_ERR_INVALID_ARG;
  if (T == 0) return NX_OK;
  if (!d_in || !d_out) return nx::set_error("NULL input/output"), NX_ERR_INVALID_ARG;
  if (!d_ws || ws_bytes < nx_fht_workspace_bytes(p, T)) {
    nx::set_error("workspace too small: need %zu bytes", nx_fht_workspace_bytes(p, T));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int mag = p->mag;
  const int outH = p->H * mag, outW = p->W * mag;
  const long long plane = (long long)outH * outW;
  char* base = (char*)d_ws + 256;
  float* work = (float*)base;
  int* mm = (int*)(base + ((std::min(T, kFhtChunk) * p->frame_floats * sizeof(float) + 255) /
                           256) * 256);
  for (int t0 = 0; t0 < T; t0 += kFhtChunk) {
    const int tc = std::min(kFhtChunk, T - t0);
    const float* in = d_in + (size_t)t0 * p->H * p->W;
    float* out = d_out + (size_t)t0 * plane;
    if (p->tiled) NX_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)tc * plane * sizeof(float), s));
    for (const auto& t : p->tiles) {
      const auto& o = p->ops[t.ops];
      const int N = o.N, L = o.L;
      float* X = work;
      float* U = X + (size_t)tc * N * N;
      float* Z = U + (size_t)tc * 2 * N * L;
      // (min, max) slots of the tile input and of the interpolated square
      fht_mm_init_kernel<<<1, 32, 0, s>>>(mm, tc);
      NX_CUDA_TRY(cudaGetLastError());
      fht_gather_kernel<<<dim3(blocks_for((long long)N * N, 256, 256), (unsigned)tc), 256, 0,
                          s>>>(in, p->H, p->W, t.r0, t.c0, t.th, t.tw, N, t.kh, t.kw, t.y_roi,
                               t.x_roi, X, mm);
      NX_CUDA_TRY(cudaGetLastError());
      // U = X [C_re^T | C_im^T] stacked: batch (frame, part)
      GemmBatch b1{2, (long long)N * N, 0, 0, (long long)N * L, (long long)2 * N * L,
                   (long long)N * L};
      NX_CUDA_TRY(gemm(X, o.ct, U, N, L, N, N, L, L, 2 * tc, b1, s));
      // Z = [A_re | -A_im] [U_re ; U_im]
      GemmBatch b2{1, 0, 0, (long long)2 * N * L, 0, (long long)L * L, 0};
      NX_CUDA_TRY(gemm(o.acat, U, Z, L, L, 2 * N, 2 * N, L, L, tc, b2, s));
      fht_zminmax_kernel<<<dim3(blocks_for((long long)L * L, 256, 512), (unsigned)tc), 256, 0,
                           s>>>(Z, (long long)L * L, mm);
      NX_CUDA_TRY(cudaGetLastError());
      const int oh = t.th * mag, ow = t.tw * mag;
      fht_finish_kernel<<<dim3(blocks_for((long long)oh * ow, 256, 1024), (unsigned)tc), 256, 0,
                          s>>>(Z, L, mm, oh, ow, (L - oh) / 2, (L - ow) / 2,
                               p->tiled ? t.wr : nullptr, p->tiled ? t.wc : nullptr, out, outH,
                               outW, t.r0 * mag, t.c0 * mag, p->variant == NX_FHT_FULL_SPECTRUM);
      NX_CUDA_TRY(cudaGetLastError());
    }
    if (p->tiled) {
      fht_normalize_kernel<<<blocks_for(plane * tc), 256, 0, s>>>(out, p->wgt, plane, tc);
      NX_CUDA_TRY(cudaGetLastError());
    }
  }
  return NX_OK;
}

}  // extern "C"
