// eSRRF-3D: radial gradient convergence of volumes
// (src/nanopyx/core/transform/_le_esrrf3d.pyx:65-140).
//
// Per frame of a (T, S, H, W) stack, as the reference:
//   1. gradients at the input resolution: central differences along x and y,
//      the backward difference along z, halved, indices clamped
//      (src/include/_c_gradients.c:75-116);
//   2. the frame and its three gradients magnified by Catmull-Rom x mxy in
//      every slice; the reference's "linear" z step then repeats each slice
//      mz times (its slice coordinate sM / mz is an integer division, so the
//      second weight is 0, _interpolation.pyx:54-88) -- here the repeat is an
//      index mapping, never materialised;
//   3. at every output voxel inside the margins the RGC over the window of
//      input-pixel offsets (src/include/_c_sr_radial_gradient_convergence.c:
//      92-204) in the reference's float32 operation order (its few double
//      steps -- exp, pow, the quotient of square roots -- in float32, within
//      a few ulp: FP64 runs at a small fraction of FP32 here), to the power
//      `sensitivity`, times the interpolated intensity;
//   4. the running mean (mode "average") or Welford variance (mode "std",
//      sqrt(M2 / T) at the end) over the frames, in the reference's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace nx {
namespace {

struct Rgc3d {
  int S, H, W, mxy, mz, Hm, Wm, Sm;
  int margin, margin_z;
  int s0, s1, z0, z1;  // window offsets, inclusive
  float tSS, tSO, tSS_z, tSO_z, sensitivity;
  int iw, mode;
  // floor(x / mz) = (x * mz_magic) >> 32 in 64-bit arithmetic for 0 <= x,
  // x * mz < 2^32
  // (mz_magic = floor(2^32 / mz) + 1: the excess x (mz_magic - 2^32 / mz) / 2^32
  // stays below 1 / mz, so it never crosses the next integer)
  unsigned long long mz_magic;
};

__global__ void gradient3d_kernel(const float* __restrict__ v, int S, int H, int W,
                                  float* __restrict__ gc, float* __restrict__ gr,
                                  float* __restrict__ gs) {
  const long long n = (long long)S * H * W;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % W), y = (int)((e / W) % H), z = (int)(e / ((long long)H * W));
    const int xp = x >= W - 1 ? W - 1 : x + 1, xm = x <= 0 ? 0 : x - 1;
    const int yp = y >= H - 1 ? H - 1 : y + 1, ym = y <= 0 ? 0 : y - 1;
    const int zm = z <= 0 ? 0 : z - 1;
    const float* sl = v + (size_t)z * H * W;
    gc[e] = __fsub_rn(sl[(size_t)y * W + xp], sl[(size_t)y * W + xm]) / 2;
    gr[e] = __fsub_rn(sl[(size_t)yp * W + x], sl[(size_t)ym * W + x]) / 2;
    gs[e] = __fsub_rn(sl[(size_t)y * W + x], v[((size_t)zm * H + y) * W + x]) / 2;
  }
}

// one thread per output voxel inside the margins; gx/gy/gz/img: (S, Hm, Wm),
// the xy-magnified volumes (slice zM of the z-magnified volume is slice
// zM / mz of these).  The window samples sit at whole input-pixel offsets
// (i, j, k) from the voxel's centre, so their distance weights, validity
// (distance != 0, xy distance <= tSO, signed z offset <= tSO_z) and inverse
// distances depend on the offset alone: `tab` holds (weight, 1 / distance)
// per offset, weight 0 where a sample does not count.  Per voxel only the
// in-volume tests and the gradient indices use the voxel's float coordinates,
// exactly as the reference forms them.
__global__ void __launch_bounds__(256) rgc3d_kernel(const __grid_constant__ Rgc3d p,
                                                    const float* __restrict__ gx,
                                                    const float* __restrict__ gy,
                                                    const float* __restrict__ gz,
                                                    const float* __restrict__ img,
                                                    const float2* __restrict__ tab, int frame,
                                                    float* __restrict__ out,
                                                    float* __restrict__ mean) {
  const int nx = p.Wm - 2 * p.margin, ny = p.Hm - 2 * p.margin, nz = p.Sm - 2 * p.margin_z;
  const long long n = (long long)nx * ny * nz;
  const size_t plane = (size_t)p.Hm * p.Wm;
  const int nI = p.s1 - p.s0 + 1, nK = p.z1 - p.z0 + 1;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    int cM, rM, sM;
    if (n < (1LL << 31)) {  // 32-bit index arithmetic
      const unsigned u = (unsigned)e;
      cM = p.margin + (int)(u % (unsigned)nx);
      rM = p.margin + (int)((u / (unsigned)nx) % (unsigned)ny);
      sM = p.margin_z + (int)(u / ((unsigned)nx * (unsigned)ny));
    } else {
      cM = p.margin + (int)(e % nx);
      rM = p.margin + (int)((e / nx) % ny);
      sM = p.margin_z + (int)(e / ((long long)nx * ny));
    }
    const float xc = __fdiv_rn((float)cM, (float)p.mxy);
    const float yc = __fdiv_rn((float)rM, (float)p.mxy);
    const float zc = __fdiv_rn((float)sM, (float)p.mz);
    float rgc = 0.f, wsum = 0.f;
    for (int j = p.s0; j <= p.s1; ++j) {
      const float vy = __fadd_rn(yc, (float)j);
      if (!(0.f < vy && vy <= (float)(p.H - 1))) continue;
      const size_t ry = (size_t)(int)__fmul_rn((float)p.mxy, vy) * p.Wm;
      for (int i = p.s0; i <= p.s1; ++i) {
        const float vx = __fadd_rn(xc, (float)i);
        if (!(0.f < vx && vx <= (float)(p.W - 1))) continue;
        const size_t rxy = ry + (int)__fmul_rn((float)p.mxy, vx);
        const float2* trow = tab + ((size_t)(j - p.s0) * nI + (i - p.s0)) * nK;
        for (int k = p.z0; k <= p.z1; ++k) {
          const float2 t = __ldg(trow + (k - p.z0));
          if (t.x == 0.f) continue;
          const float vz = __fadd_rn(zc, (float)k);
          if (!(0.f < vz && vz <= (float)(p.S - 1))) continue;
          // slice of the xy-magnified volumes: (int)(vz mz) / mz, vz > 0
          const unsigned zm = (unsigned)(int)__fmul_rn(vz, (float)p.mz);
          const size_t li = (size_t)((zm * p.mz_magic) >> 32) * plane + rxy;
          const float Gx = __ldg(gx + li), Gy = __ldg(gy + li), Gz = __ldg(gz + li);
          wsum = __fadd_rn(wsum, t.x);
          const float fi = (float)i, fj = (float)j, fk = (float)k;
          const float gdr = fmaf(Gz, fk, fmaf(Gy, fj, Gx * fi));
          if (gdr < 0.f) {
            const float c1 = fmaf(Gy, fk, -Gz * fj);
            const float c2 = fmaf(Gz, fi, -Gx * fk);
            const float c3 = fmaf(Gx, fj, -Gy * fi);
            const float num = fmaf(c3, c3, fmaf(c2, c2, c1 * c1));
            const float den = fmaf(Gz, Gz, fmaf(Gy, Gy, Gx * Gx));
            // |c| / |G| / distance; 0 / 0 (no gradient) counts as the distance
            // itself in the reference, i.e. a zero contribution
            const float dk = den > 0.f ? sqrtf(num) * rsqrtf(den) * t.y : 1.f;
            rgc = fmaf(1.f - dk, t.x, rgc);
          }
        }
      }
    }
    rgc = __fdiv_rn(rgc, wsum);
    if (rgc >= 0.f && p.sensitivity > 1.f)
      rgc = powf(rgc, p.sensitivity);
    else if (rgc < 0.f)
      rgc = 0.f;
    if (p.iw) rgc = __fmul_rn(rgc, __ldg(img + (size_t)(sM / p.mz) * plane + (size_t)rM * p.Wm + cM));
    const size_t o = ((size_t)sM * p.Hm + rM) * p.Wm + cM;
    const float fr = (float)(frame + 1);
    if (p.mode == 0) {
      out[o] = __fadd_rn(out[o], __fdiv_rn(__fsub_rn(rgc, out[o]), fr));
    } else {
      const float delta = __fsub_rn(rgc, mean[o]);
      mean[o] = __fadd_rn(mean[o], __fdiv_rn(delta, fr));
      const float delta2 = __fsub_rn(rgc, mean[o]);
      out[o] = __fadd_rn(out[o], __fmul_rn(delta, delta2));
    }
  }
}

__global__ void std_finish_kernel(float* __restrict__ out, long long n, float frames) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    out[e] = __fsqrt_rn(__fdiv_rn(out[e], frames));
}

unsigned grid_of(long long n) {
  return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 32));
}

size_t rup(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace nx

using namespace nx;

extern "C" {

// window offsets per axis are at most 2 int(radius) + 2 <= kMaxWin
constexpr int kMaxWin = 64;

size_t nx_esrrf3d_workspace_bytes(int S, int H, int W, int magnification_xy,
                                  int magnification_z, int mode) {
  if (S < 1 || H < 1 || W < 1 || magnification_xy < 1 || magnification_z < 1) return 256;
  const size_t vol = (size_t)S * H * W;
  const size_t volm = (size_t)S * H * magnification_xy * W * magnification_xy;
  const size_t out = volm * magnification_z;
  return 256 + rup(3 * (size_t)S * sizeof(float)) + rup(3 * vol * sizeof(float)) +
         rup(4 * volm * sizeof(float)) + (mode ? rup(out * sizeof(float)) : 0) +
         rup((size_t)kMaxWin * kMaxWin * kMaxWin * sizeof(float2));
}

int nx_esrrf3d_st(const float* d_in, int T, int S, int H, int W, int magnification_xy,
                  int magnification_z, double radius, double radius_z, float sensitivity,
                  int mode, int do_intensity_weighting, float* d_out, void* d_ws,
                  size_t ws_bytes, void* stream) {
  if (T < 1 || S < 1 || H < 1 || W < 1) return nx::set_error("bad stack shape"), NX_ERR_INVALID_ARG;
  if (magnification_xy < 1 || magnification_z < 1)
    return nx::set_error("magnifications must be >= 1"), NX_ERR_INVALID_ARG;
  if (!(radius > 0) || !(radius_z > 0))
    return nx::set_error("radius and radius_z must be > 0"), NX_ERR_INVALID_ARG;
  if (mode != 0 && mode != 1) return nx::set_error("mode must be 0 (average) or 1 (std)"), NX_ERR_INVALID_ARG;
  if (!d_in || !d_out) return nx::set_error("NULL input/output"), NX_ERR_INVALID_ARG;
  const size_t need = nx_esrrf3d_workspace_bytes(S, H, W, magnification_xy, magnification_z, mode);
  if (!d_ws || ws_bytes < need) {
    nx::set_error("workspace too small: need %zu bytes", need);
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int mxy = magnification_xy, mz = magnification_z;
  Rgc3d p{};
  p.S = S;
  p.H = H;
  p.W = W;
  p.mxy = mxy;
  p.mz = mz;
  p.Hm = H * mxy;
  p.Wm = W * mxy;
  p.Sm = S * mz;
  if ((unsigned long long)p.Sm * (unsigned long long)mz >= (1ULL << 32))
    return nx::set_error("S * magnification_z^2 must be below 2^32"), NX_ERR_INVALID_ARG;
  p.mz_magic = (1ULL << 32) / (unsigned long long)mz + 1;
  // the reference's scalars (_le_esrrf3d.pyx:73-86): radius and radius_z are
  // Python floats, sigma and the thresholds C floats
  const float sigma = (float)(radius / 2.355);
  const float sigma_z = (float)(radius_z / 2.355);
  p.margin = (int)(radius * mxy);
  p.margin_z = (int)(radius_z * mz);
  p.tSS = 2 * sigma * sigma;
  p.tSO = 2 * sigma + 1;
  p.tSS_z = 2 * sigma_z * sigma_z;
  p.tSO_z = 2 * sigma_z + 1;
  const float fwhm = (float)radius, fwhm_z = (float)radius_z;
  p.s0 = -(int)fwhm;
  p.s1 = (int)(fwhm + 1);
  p.z0 = -(int)fwhm_z;
  p.z1 = (int)(fwhm_z + 1);
  p.sensitivity = sensitivity;
  p.iw = do_intensity_weighting ? 1 : 0;
  p.mode = mode;
  const int nI = p.s1 - p.s0 + 1, nK = p.z1 - p.z0 + 1;
  if (nI > kMaxWin || nK > kMaxWin)
    return nx::set_error("radius too large for the 3-D window"), NX_ERR_INVALID_ARG;
  // per-offset (weight, 1 / distance), the reference's _c_calculate_dw3D
  // (src/include/_c_sr_radial_gradient_convergence.c:96-102) at whole-pixel
  // offsets; weight 0 where the sample does not count
  std::vector<float2> tab((size_t)nI * nI * nK);
  for (int j = p.s0; j <= p.s1; ++j)
    for (int i = p.s0; i <= p.s1; ++i)
      for (int k = p.z0; k <= p.z1; ++k) {
        const double dxy2 = (double)i * i + (double)j * j;
        const double d = std::sqrt(dxy2 + (double)k * k), dxy = std::sqrt(dxy2);
        float w = 0.f, inv = 0.f;
        if (d != 0 && dxy <= (double)p.tSO && (double)k <= (double)p.tSO_z) {
          const float wxy = (float)std::exp(-dxy2 / (double)p.tSS);
          const float wz = (float)std::exp(-(double)k * k / (double)p.tSS_z);
          const float D = (float)(d * (double)(wxy * wz));
          w = (float)std::pow((double)D, 4.0);
          inv = (float)(1.0 / d);
        }
        tab[((size_t)(j - p.s0) * nI + (i - p.s0)) * nK + (k - p.z0)] = make_float2(w, inv);
      }
  const size_t vol = (size_t)S * H * W;
  const size_t volm = (size_t)S * p.Hm * p.Wm;
  const long long nout = (long long)p.Sm * p.Hm * p.Wm;
  char* b = (char*)d_ws + 256;
  float* zeros = (float*)b;
  b += rup(3 * (size_t)S * sizeof(float));
  float* G = (float*)b;  // (3, S, H, W)
  b += rup(3 * vol * sizeof(float));
  float* M = (float*)b;  // (4, S, Hm, Wm): image, gx, gy, gz magnified in xy
  b += rup(4 * volm * sizeof(float));
  float* mean = mode ? (float*)b : nullptr;
  if (mode) b += rup((size_t)nout * sizeof(float));
  float2* dtab = (float2*)b;
  NX_CUDA_TRY(cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(float2),
                              cudaMemcpyHostToDevice, s));
  NX_CUDA_TRY(cudaMemsetAsync(zeros, 0, 3 * (size_t)S * sizeof(float), s));
  NX_CUDA_TRY(cudaMemsetAsync(d_out, 0, (size_t)nout * sizeof(float), s));
  if (mean) NX_CUDA_TRY(cudaMemsetAsync(mean, 0, (size_t)nout * sizeof(float), s));
  const bool inside = p.Wm - 2 * p.margin > 0 && p.Hm - 2 * p.margin > 0 &&
                      p.Sm - 2 * p.margin_z > 0;
  const long long ninner = inside ? (long long)(p.Wm - 2 * p.margin) *
                                        (p.Hm - 2 * p.margin) * (p.Sm - 2 * p.margin_z)
                                  : 0;
  for (int f = 0; f < T; ++f) {
    const float* frame = d_in + (size_t)f * vol;
    gradient3d_kernel<<<grid_of((long long)vol), 256, 0, s>>>(frame, S, H, W, G, G + vol,
                                                               G + 2 * vol);
    NX_CUDA_TRY(cudaGetLastError());
    const float *img, *gx, *gy, *gz;
    if (mxy > 1) {
      NX_CUDA_TRY(launch_cr_shift_magnify(frame, S, H, W, zeros, zeros, (float)mxy, (float)mxy,
                                          p.Hm, p.Wm, M, s));
      NX_CUDA_TRY(launch_cr_shift_magnify(G, 3 * S, H, W, zeros, zeros, (float)mxy, (float)mxy,
                                          p.Hm, p.Wm, M + volm, s));
      img = M;
      gx = M + volm;
      gy = M + 2 * volm;
      gz = M + 3 * volm;
    } else {
      img = frame;
      gx = G;
      gy = G + vol;
      gz = G + 2 * vol;
    }
    if (ninner > 0) {
      rgc3d_kernel<<<grid_of(ninner), 256, 0, s>>>(p, gx, gy, gz, img, dtab, f, d_out, mean);
      NX_CUDA_TRY(cudaGetLastError());
    }
  }
  if (mode == 1) {
    std_finish_kernel<<<grid_of(nout), 256, 0, s>>>(d_out, nout, (float)T);
    NX_CUDA_TRY(cudaGetLastError());
  }
  return NX_OK;
}

}  // extern "C"
