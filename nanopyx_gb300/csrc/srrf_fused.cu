// Fused SRRF radiality kernel (sm_103a): one CTA owns a 32 x TY tile of input
// pixels, loops over frames, and per frame
//   1. stages the input tile + halo in shared memory,
//   2. forms the central-difference gradients   (_c_gradients.c:3-25),
//   3. Catmull-Rom-magnifies the intensity      (_c_interpolation_catmull_rom.c:21-52),
//   4. evaluates radiality over the 12-point ring for the thread's M outputs
//      (_c_sr_radiality.c:15-51): two Catmull-Rom interpolations of the gradient
//      per ring point from shared memory.
// The reference's ring positions depend on the output row only through
// y0 = (j + 0.5) + yRing and on the column only through x0 = (i + 0.5) + xRing, so
// the tap rows / columns and Catmull-Rom weights of every (output row, ring
// point) and (output column, ring point) are tabulated once per tile in shared
// memory, in the reference's own float32 arithmetic (x0 rounded, x0 / m IEEE).
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "internal.h"

namespace nx {

namespace {

constexpr int kRing = 12;
constexpr int kHalo = 5;  // input rows/cols around the tile: ring radius <= 2 px

template <int M>
struct SrrfTile {
  // tile rows: the eSRRF kernel's, except m = 5, where 6 rows (960 threads,
  // 64 registers, no spills) measured 2.5 % faster than 4 (640 threads, 95
  // registers) on the 500 x 512 x 512 stack: more warps hide the shared loads
  static constexpr int TY = (M == 5) ? 6 : TileRows<M>::TY;
  static constexpr int TX = 32;
  static constexpr int NT = 32 * TY * M;
  static constexpr int IH = TY + 2 * kHalo;  // input tile rows
  static constexpr int IW = TX + 2 * kHalo;
  static constexpr int OY = TY * M, OX = TX * M;
  static constexpr int RIW = TX + 4;
  static constexpr int al(int n) { return (n + 31) / 32 * 32; }
  static constexpr int O_IN = 0;                        // input tile
  static constexpr int O_G = O_IN + al(IH * IW);        // gradient float2 (gx, gy)
  static constexpr int O_RI = O_G + al(IH * IW * 2);    // intensity row pass
  static constexpr int O_RW = O_RI + al(OY * RIW);      // intensity row weights [OY][5]
  static constexpr int O_CW = O_RW + al(OY * 5);        // intensity col weights [OX][5]
  static constexpr int O_RT = O_CW + al(OX * 5);        // ring row taps [OY][12][8]
  // ring column taps of output column (lane, px) as 5 weights on the columns
  // cb .. cb + 4 of the row-pass buffer, cb = the first tap of px = 0 (the taps
  // of px = 1 .. M-1 start at cb or cb + 1): [ring][px][lane] float4 (weights
  // 0..3) and float (weight 4), lane-contiguous
  static constexpr int O_CW4 = O_RT + al(OY * kRing * 8);
  static constexpr int O_CW1 = O_CW4 + al(kRing * M * TX * 4);
  static constexpr int O_CB = O_CW1 + al(kRing * M * TX);  // [ring][lane] int: cb - x_start
  // per-warp row pass of the gradient interpolation: [warp][ring][IW] float2,
  // plus one zeroed float2 after the last ring (read with weight 0)
  static constexpr int RBW = kRing * IW * 2 + 2;
  static constexpr int O_RB = O_CB + al(kRing * TX);
  static constexpr int FLOATS = O_RB + (NT / 32) * RBW;
  static constexpr size_t SMEM = size_t(FLOATS) * 4;
};

struct SrrfParams {
  const float* in;      // (T, h, w)
  const float* interp;  // (T, h*M, w*M) magnified intensity, or nullptr: computed here
  float* out;           // (T, h*M, w*M)
  int T, h, w;
  int tiles_x, tiles_y;
  int chunks;           // frame chunks (grid y)
  int border, positivity, iw;
  float rr;         // ring radius * M (float, as the reference)
  float inv_rr;     // 1 / rr
  float xr[kRing], yr[kRing];
};

// ring tap entry: [0] first tap index (int bits), [1..4] weights, [5] centre
// minus ring point (yc - y0 or xc - x0), [6] inside flag (1 / 0)
__device__ __forceinline__ void ring_entry(float* e, float c, float ring, int M, int n) {
  const float p0 = __fadd_rn(c, ring);
  const float r = __fdiv_rn(p0, (float)M);
  const int ri = (int)floorf(r - 0.5f);
  e[0] = __int_as_float(ri - 1);
#pragma unroll
  for (int t = 0; t < 4; ++t) e[1 + t] = cr_cubic(r - ((float)(ri - 1 + t) + 0.5f));
  e[5] = __fsub_rn(c, p0);
  e[6] = (r >= 0.f && r < (float)n) ? 1.f : 0.f;
  e[7] = 0.f;
}

template <int M>
__global__ void __launch_bounds__(SrrfTile<M>::NT, 1) srrf_fused_kernel(const SrrfParams p) {
  using G = SrrfTile<M>;
  constexpr int TY = G::TY;
  extern __shared__ __align__(128) float sm[];
  float* tin = sm + G::O_IN;
  float2* grad = reinterpret_cast<float2*>(sm + G::O_G);
  float* ri = sm + G::O_RI;
  float* rw = sm + G::O_RW;
  float* cw = sm + G::O_CW;
  float* rt = sm + G::O_RT;
  float4* cw4 = reinterpret_cast<float4*>(sm + G::O_CW4);
  float* cw1 = sm + G::O_CW1;
  int* cbt = reinterpret_cast<int*>(sm + G::O_CB);
  float2* rb = reinterpret_cast<float2*>(sm + G::O_RB + (threadIdx.x >> 5) * G::RBW);

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int ty = warp % TY;
  const int py = warp / TY;
  const int tile = blockIdx.x;
  const int f_begin = (int)((long long)blockIdx.y * p.T / p.chunks);
  const int f_end = (int)((long long)(blockIdx.y + 1) * p.T / p.chunks);
  const int nx0 = (tile % p.tiles_x) * G::TX;
  const int ny0 = (tile / p.tiles_x) * TY;
  const int h = p.h, w = p.w;
  const int rowsM = h * M, colsM = w * M;
  const int y_start = ny0 - kHalo, x_start = nx0 - kHalo;

  // ---- per-tile tables ------------------------------------------------------
  for (int i = tid; i < G::OY; i += G::NT) {
    const int yM = ny0 * M + i;
    const int nyo = ny0 + i / M;
    const float ry = __fdiv_rn((float)yM, (float)M);
    const int rb = (int)floorf(ry - 0.5f);
    float w5[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int k = rb - 1 + t - (nyo - 2);
      const float wt = cr_cubic(ry - ((float)(rb - 1 + t) + 0.5f));
#pragma unroll
      for (int kk = 0; kk < 5; ++kk) w5[kk] = (k == kk) ? wt : w5[kk];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) rw[i * 5 + k] = w5[k];
    const float yc = (float)yM + 0.5f;
    for (int s = 0; s < kRing; ++s) ring_entry(rt + (i * kRing + s) * 8, yc, p.yr[s], M, h);
  }
  for (int i = tid; i < G::OX; i += G::NT) {
    const int xM = nx0 * M + i;
    const int nxo = nx0 + i / M;
    const float rx = __fdiv_rn((float)xM, (float)M);
    const int cb = (int)floorf(rx - 0.5f);
    float w5[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int k = cb - 1 + t - (nxo - 2);
      const float wt = cr_cubic(rx - ((float)(cb - 1 + t) + 0.5f));
#pragma unroll
      for (int kk = 0; kk < 5; ++kk) w5[kk] = (k == kk) ? wt : w5[kk];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) cw[i * 5 + k] = w5[k];
  }
  for (int i = tid; i < kRing * G::TX; i += G::NT) {
    const int s = i / G::TX, ln = i % G::TX;
    int cb = 0;
    for (int px = 0; px < M; ++px) {
      float e[8];
      ring_entry(e, (float)((nx0 + ln) * M + px) + 0.5f, p.xr[s], M, w);
      const int c0 = __float_as_int(e[0]);
      if (px == 0) cb = c0;
      // 0 or 1: the M phases of one lane span less than one input pixel
      const int off = min(max(c0 - cb, 0), 1);
      // a column outside the image contributes nothing (the reference skips
      // it): all its weights are zero
      float w5[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      if (e[6] != 0.f) {
#pragma unroll
        for (int u = 0; u < 4; ++u) w5[u + off] = e[1 + u];
      }
      cw4[(s * M + px) * G::TX + ln] = make_float4(w5[0], w5[1], w5[2], w5[3]);
      cw1[(s * M + px) * G::TX + ln] = w5[4];
    }
    cbt[s * G::TX + ln] = cb - x_start;
  }
  if ((tid & 31) == 0) rb[kRing * G::IW] = make_float2(0.f, 0.f);

  const int ny = ny0 + ty, nx = nx0 + lane;
  const int j = ny * M + py;  // output row
  const int lo_j = (1 + p.border) * M, hi_j = (h - 1 - p.border) * M;
  const int lo_i = (1 + p.border) * M, hi_i = (w - 1 - p.border) * M;
  const bool row_ok = j >= lo_j && j < hi_j && ny < h;
  const float* rrow = rt + ((ty * M + py) * kRing) * 8;
  const size_t plane = (size_t)rowsM * colsM;

  const bool own_intensity = p.interp == nullptr;
  for (int f = f_begin; f < f_end; ++f) {
    __syncthreads();  // tables ready / previous frame's shared data consumed
    const float* src = p.in + (size_t)f * h * w;
    for (int i = tid; i < G::IH * G::IW; i += G::NT) {
      const int r = y_start + i / G::IW, c = x_start + i % G::IW;
      tin[i] = (r >= 0 && r < h && c >= 0 && c < w) ? __ldg(src + (size_t)r * w + c) : 0.f;
    }
    __syncthreads();
    // gradients (zero outside rows/cols 1..n-2) and the intensity row pass
    for (int i = tid; i < G::IH * G::IW; i += G::NT) {
      const int rl = i / G::IW, cl = i % G::IW;
      const int r = y_start + rl, c = x_start + cl;
      float2 g = make_float2(0.f, 0.f);
      if (r >= 1 && r < h - 1 && c >= 1 && c < w - 1 && rl >= 1 && rl < G::IH - 1 && cl >= 1 &&
          cl < G::IW - 1) {
        g.x = __fadd_rn(-tin[i - 1], tin[i + 1]);
        g.y = __fadd_rn(-tin[i - G::IW], tin[i + G::IW]);
      }
      grad[i] = g;
    }
    for (int i = tid; own_intensity && i < G::OY * G::RIW; i += G::NT) {
      const int oy = i / G::RIW, cc = i % G::RIW;
      const int nyo = ny0 + oy / M;
      const float* w5 = rw + oy * 5;
      const float* col = tin + (nyo - 2 - y_start) * G::IW + (nx0 - 2 + cc - x_start);
      float sum = 0.f;
#pragma unroll
      for (int k = 0; k < 5; ++k) sum = fmaf(w5[k], col[k * G::IW], sum);
      ri[i] = sum;
    }
    __syncthreads();
    // row pass of the ring interpolation: the ring points of this warp's output
    // row share their tap rows and weights, so each (ring point, tile column)
    // sum over the 4 tap rows is formed once per warp (same fma order as the
    // 16-tap form: rows first, then columns)
    for (int idx = lane; idx < kRing * G::IW; idx += 32) {
      const int s = idx / G::IW, c = idx - s * G::IW;
      const float4 rA = *reinterpret_cast<const float4*>(rrow + s * 8);
      const float4 rB = *reinterpret_cast<const float4*>(rrow + s * 8 + 4);
      float2 v = make_float2(0.f, 0.f);
      if (rB.z != 0.f) {
        const int r0 = __float_as_int(rA.x) - y_start;
        const float wr[4] = {rA.y, rA.z, rA.w, rB.x};
        const float2* gp = grad + r0 * G::IW + c;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const float2 g = gp[t * G::IW];
          v.x = fmaf(g.x, wr[t], v.x);
          v.y = fmaf(g.y, wr[t], v.y);
        }
      }
      rb[idx] = v;
    }
    __syncwarp();
    // radiality of this thread's M outputs, ring point by ring point: the M
    // columns share one window of 5 row-pass columns (cb .. cb + 4), each
    // output weights it with its own 5-vector (its 4 taps and a zero), which
    // is the 4-tap fma sequence of the reference with a + 0 at one end
    float div[M];
#pragma unroll
    for (int px = 0; px < M; ++px) div[px] = 0.f;
    const float yc = (float)j + 0.5f;
#pragma unroll 2
    for (int s = 0; s < kRing; ++s) {
      const float dy = __fsub_rn(yc, __fadd_rn(yc, p.yr[s]));  // yc - y0
      const float2* rp = rb + s * G::IW + cbt[s * G::TX + lane];
      float2 col[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) col[k] = rp[k];
#pragma unroll
      for (int px = 0; px < M; ++px) {
        const float4 wa = cw4[(s * M + px) * G::TX + lane];
        const float we = cw1[(s * M + px) * G::TX + lane];
        const float wv[5] = {wa.x, wa.y, wa.z, wa.w, we};
        const float xc = (float)(nx * M + px) + 0.5f;
        const float dx = __fsub_rn(xc, __fadd_rn(xc, p.xr[s]));  // xc - x0
        float vgx = 0.f, vgy = 0.f;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          vgx = fmaf(col[k].x, wv[k], vgx);
          vgy = fmaf(col[k].y, wv[k], vgy);
        }
        float dk = 0.f;
        const float g2 = vgx * vgx + vgy * vgy;
        if (g2 != 0.f) {
          // |vGy (xc - x0) - vGx (yc - y0)| / GMag / ringRadius
          dk = 1.f - fabsf(vgy * dx - vgx * dy) * rsqrtf(g2) * p.inv_rr;
          dk = dk * dk;
        }
        if (vgx * p.xr[s] + vgy * p.yr[s] > 0.f) div[px] -= dk;
        else div[px] += dk;
      }
    }
#pragma unroll
    for (int px = 0; px < M; ++px) {
      const int i = nx * M + px;  // output column
      float val = 0.f;
      if (row_ok && nx < w && i >= lo_i && i < hi_i) {
        const float dv = div[px] / 12.f;
        val = p.positivity ? fmaxf(dv, 0.f) : dv;
        if (p.iw) {
          if (own_intensity) {
            // column pass of the intensity magnification (5 taps of the row pass)
            const float* w5 = cw + (lane * M + px) * 5;
            const float* rr = ri + (ty * M + py) * G::RIW + lane;
            float sum = 0.f;
#pragma unroll
            for (int k = 0; k < 5; ++k) sum = fmaf(w5[k], rr[k], sum);
            val *= sum;
          } else {
            val *= __ldg(p.interp + (size_t)f * plane + (size_t)j * colsM + i);
          }
        }
      }
      if (ny < h && nx < w) p.out[(size_t)f * plane + (size_t)j * colsM + i] = val;
    }
  }
}

template <int M>
cudaError_t launch_srrf_m(const SrrfParams& prm, cudaStream_t s) {
  using G = SrrfTile<M>;
  static int attr_done = -1;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (attr_done != dev) {
    e = cudaFuncSetAttribute(srrf_fused_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)G::SMEM);
    if (e != cudaSuccess) return e;
    attr_done = dev;
  }
  SrrfParams q = prm;
  q.tiles_x = (prm.w + G::TX - 1) / G::TX;
  q.tiles_y = (prm.h + G::TY - 1) / G::TY;
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (long long)q.tiles_x * q.tiles_y;
  q.chunks = (int)std::max<long long>(1, std::min<long long>(prm.T, (2LL * sms + tiles - 1) / tiles));
  srrf_fused_kernel<M><<<dim3((unsigned)tiles, (unsigned)q.chunks), G::NT, G::SMEM, s>>>(q);
  return cudaGetLastError();
}

}  // namespace

// fused radiality for m in {2, 3, 4, 5, 6, 8} and ring radius <= 2 px; returns
// cudaErrorNotSupported otherwise (the caller then uses the per-pixel kernel)
cudaError_t launch_srrf_fused(const float* in, const float* img_interp, int T, int h, int w,
                              int M, const RingCoords& rc, float ring_radius, int border,
                              int positivity, int iw, float* out, cudaStream_t s) {
  if (!(ring_radius >= 0.f && ring_radius <= 2.0f)) return cudaErrorNotSupported;
  SrrfParams p;
  memset(&p, 0, sizeof(p));
  p.in = in;
  p.interp = img_interp;
  p.out = out;
  p.T = T;
  p.h = h;
  p.w = w;
  p.border = border;
  p.positivity = positivity;
  p.iw = iw;
  p.rr = rc.radius;
  p.inv_rr = rc.radius != 0.f ? 1.f / rc.radius : 0.f;
  for (int k = 0; k < kRing; ++k) {
    p.xr[k] = rc.x[k];
    p.yr[k] = rc.y[k];
  }
  if ((long long)T * h * w == 0) return cudaSuccess;
  switch (M) {
    case 2: return launch_srrf_m<2>(p, s);
    case 3: return launch_srrf_m<3>(p, s);
    case 4: return launch_srrf_m<4>(p, s);
    case 5: return launch_srrf_m<5>(p, s);
    case 6: return launch_srrf_m<6>(p, s);
    case 8: return launch_srrf_m<8>(p, s);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace nx
