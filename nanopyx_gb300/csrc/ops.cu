// Standalone Liquid-Engine ops of the eSRRF / SRRF path, temporal
// correlations and macro-pixel correction (sm_103a).
//
// These follow the reference's float32 arithmetic per output pixel (they are
// the drop-ins for the individual ops and the general fallback of the fused
// kernel); the fused frame-loop kernel in esrrf_fused.cuh is the hot path.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "internal.h"

namespace nx {

namespace {

constexpr int kBlock = 256;

inline unsigned grid_for(long long n, int block = kBlock) {
  long long g = (n + block - 1) / block;
  if (g > 1048576) g = 1048576;  // grid-stride beyond this
  if (g < 1) g = 1;
  return (unsigned)g;
}

// _c_interpolate (src/include/_c_interpolation_catmull_rom.c:21-52) in float:
// pixel-centre taps, out-of-image taps skipped, 0 outside the image.
__device__ __forceinline__ float cr_interp(const float* __restrict__ img, float r, float c,
                                           int rows, int cols) {
  if (r < 0.f || r >= (float)rows || c < 0.f || c >= (float)cols) return 0.f;
  const int r_int = (int)floorf(r - 0.5f);
  const int c_int = (int)floorf(c - 0.5f);
  float q = 0.f;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int cn = c_int - 1 + j;
    if (cn < 0 || cn >= cols) continue;
    float p = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int rn = r_int - 1 + i;
      if (rn < 0 || rn >= rows) continue;
      p = fmaf(__ldg(img + (size_t)rn * cols + cn), cr_cubic(r - ((float)rn + 0.5f)), p);
    }
    q = fmaf(p, cr_cubic(c - ((float)cn + 0.5f)), q);
  }
  return q;
}

__global__ void cr_shift_magnify_kernel(const float* __restrict__ in, int T, int H, int W,
                                        const float* __restrict__ shift_r,
                                        const float* __restrict__ shift_c, float mag_r,
                                        float mag_c, int rowsM, int colsM,
                                        float* __restrict__ out) {
  const long long plane = (long long)rowsM * colsM;
  const long long n = plane * T;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(idx / plane);
    const long long rem = idx - (long long)t * plane;
    const int i = (int)(rem / colsM);
    const int j = (int)(rem - (long long)i * colsM);
    const float row = __fsub_rn(__fdiv_rn((float)i, mag_r), shift_r[t]);
    const float col = __fsub_rn(__fdiv_rn((float)j, mag_c), shift_c[t]);
    out[idx] = cr_interp(in + (size_t)t * H * W, row, col, H, W);
  }
}

// Tiled form of the same resampling for magnifications >= 1: one CTA per
// (frame, up-to-64-row x 256-column output tile).  The sample coordinates and the
// four Catmull-Rom weights of every output row and column of the tile are
// computed once; the input patch the tile reads (zero outside the image, the
// value the reference's skipped taps contribute) is staged in shared memory;
// a vertical pass forms, for every output row and patch column, the 4-tap
// column sum p the per-pixel kernel forms, and the horizontal pass adds the 4
// column taps in the same order -- the same float operations as
// cr_shift_magnify_kernel, so the same results, with 4 shared loads and one
// coalesced store per output instead of 16 global loads and 20 weight
// evaluations.
constexpr int kCrTileCols = 256;
constexpr int kCrMaxTileRows = 64;

// Patch rows / columns a tile can touch at magnification mag >= 1: the taps of
// n consecutive outputs start within floor((n - 1) / mag) + 1 input pixels of
// each other (the extra 1 covers the float rounding of i / mag - shift), plus
// the 4 taps, plus one spare.
inline int cr_patch_extent(int n_out, float mag) {
  return (int)std::floor((double)(n_out - 1) / (double)mag) + 6;
}

// shared memory of a tile of `rows` output rows
inline size_t cr_tile_smem(int rows, float mag_r, float mag_c) {
  const int PR = cr_patch_extent(rows, mag_r), PC = cr_patch_extent(kCrTileCols, mag_c);
  return (size_t)(PR + rows) * PC * sizeof(float) + rows * (sizeof(float4) + sizeof(int));
}

// Output rows per tile: the most (up to 64) whose staging fits in 72 KB, so
// that the stores of a tile outweigh its weight set-up and patch load (64 rows
// beat 32 and 128 at m = 5: 0.53 ms against 0.60 and 0.55 for 100 frames)
inline int cr_tile_rows(float mag_r, float mag_c) {
  for (int rows = kCrMaxTileRows; rows > 32; rows /= 2)
    if (cr_tile_smem(rows, mag_r, mag_c) <= 72 * 1024) return rows;
  return 32;
}

__global__ void __launch_bounds__(kCrTileCols)
    cr_magnify_tiled_kernel(const float* __restrict__ in, int H, int W,
                            const float* __restrict__ shift_r, const float* __restrict__ shift_c,
                            float mag_r, float mag_c, int rowsM, int colsM, int TR, int PR,
                            int PC, float* __restrict__ out) {
  // the float4 row weights first, at the 16-byte aligned base
  extern __shared__ __align__(16) float crs[];
  float4* wr = reinterpret_cast<float4*>(crs);                  // [TR]
  int* rbase = reinterpret_cast<int*>(wr + TR);                 // [TR]
  float* patch = reinterpret_cast<float*>(rbase + TR);          // [PR][PC]
  float* P = patch + PR * PC;                                   // [TR][PC]
  const int t = blockIdx.z;
  const int i0 = blockIdx.y * TR;
  const int j0 = blockIdx.x * kCrTileCols;
  const float sr = shift_r[t], sc = shift_c[t];
  const int tid = threadIdx.x;
  // first patch row / column: the first tap of the tile's first output row / column
  const float row0 = __fsub_rn(__fdiv_rn((float)i0, mag_r), sr);
  const float col0 = __fsub_rn(__fdiv_rn((float)j0, mag_c), sc);
  const int pr0 = (int)floorf(row0 - 0.5f) - 1;
  const int pc0 = (int)floorf(col0 - 0.5f) - 1;
  // this thread's output column: coordinate, validity, patch offset, weights
  const int j = j0 + tid;
  const float col = __fsub_rn(__fdiv_rn((float)j, mag_c), sc);
  const int c_int = (int)floorf(col - 0.5f);
  const int ci = c_int - 1 - pc0;
  const bool cval = j < colsM && !(col < 0.f || col >= (float)W) && ci >= 0 && ci + 3 < PC;
  float wc[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) wc[k] = cr_cubic(col - ((float)(c_int - 1 + k) + 0.5f));
  for (int il = tid; il < TR; il += kCrTileCols) {
    const int i = i0 + il;
    const float row = __fsub_rn(__fdiv_rn((float)i, mag_r), sr);
    const int r_int = (int)floorf(row - 0.5f);
    const int rb = r_int - 1 - pr0;
    const bool rval = i < rowsM && !(row < 0.f || row >= (float)H) && rb >= 0 && rb + 3 < PR;
    float w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) w[k] = cr_cubic(row - ((float)(r_int - 1 + k) + 0.5f));
    wr[il] = make_float4(w[0], w[1], w[2], w[3]);
    rbase[il] = rval ? rb : -1;
  }
  // patch and vertical pass in warp rows: lanes across the columns, no
  // division by the runtime patch width
  const int lane = tid & 31, warp = tid >> 5;
  const float* f = in + (size_t)t * H * W;
  for (int pr = warp; pr < PR; pr += kCrTileCols / 32) {
    const int r = pr0 + pr;
    const bool rin = r >= 0 && r < H;
    for (int pc = lane; pc < PC; pc += 32) {
      const int c = pc0 + pc;
      patch[pr * PC + pc] = (rin && c >= 0 && c < W) ? __ldg(f + (size_t)r * W + c) : 0.f;
    }
  }
  __syncthreads();
  // vertical pass: P[i][c] = sum_l w_l(i) patch[rbase(i) + l][c] (fma order of
  // the per-pixel kernel: l = 0..3); a row outside the image is all zero
  for (int il = warp; il < TR; il += kCrTileCols / 32) {
    const int rb = rbase[il];
    const float4 w = wr[il];
    for (int c = lane; c < PC; c += 32) {
      float p = 0.f;
      if (rb >= 0) {
        const float* pc = patch + rb * PC + c;
        p = fmaf(pc[0], w.x, p);
        p = fmaf(pc[PC], w.y, p);
        p = fmaf(pc[2 * PC], w.z, p);
        p = fmaf(pc[3 * PC], w.w, p);
      }
      P[il * PC + c] = p;
    }
  }
  __syncthreads();
  if (j >= colsM) return;
  float* o = out + ((size_t)t * rowsM + i0) * colsM + j;
  const int iend = min(TR, rowsM - i0);
  if (cval) {
    // an all-zero P row gives q = +0, the reference's value for a row
    // outside the image, so the loop needs no per-row test
    const float* pp = P + ci;
#pragma unroll 4
    for (int il = 0; il < iend; ++il, pp += PC, o += colsM) {
      float q = 0.f;
#pragma unroll
      for (int k = 0; k < 4; ++k) q = fmaf(pp[k], wc[k], q);
      *o = q;
    }
  } else {
    for (int il = 0; il < iend; ++il, o += colsM) *o = 0.f;
  }
}

// _c_gradient_roberts_cross (src/include/_c_gradients.c:53-73), same
// evaluation order, so bit-identical to the reference.
__global__ void roberts_cross_kernel(const float* __restrict__ in, int T, int H, int W,
                                     float* __restrict__ gc, float* __restrict__ gr) {
  const long long plane = (long long)H * W;
  const long long n = plane * T;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(idx / plane);
    const long long rem = idx - (long long)t * plane;
    const int r1 = (int)(rem / W);
    const int c1 = (int)(rem - (long long)r1 * W);
    const int r0 = r1 > 0 ? r1 - 1 : 0;
    const int c0 = c1 > 0 ? c1 - 1 : 0;
    const float* f = in + (size_t)t * plane;
    const float a = f[(size_t)r0 * W + c1];
    const float b = f[(size_t)r1 * W + c0];
    const float d = f[(size_t)r0 * W + c0];
    const float e = f[(size_t)r1 * W + c1];
    gc[idx] = __fsub_rn(__fadd_rn(__fsub_rn(a, b), e), d);
    gr[idx] = __fsub_rn(__fadd_rn(__fadd_rn(-a, b), e), d);
  }
}

__device__ __forceinline__ float apply_sensitivity(float r, int mode, int n, float s) {
  if (mode == 1) {
    const float base = r;
    for (int k = 1; k < n; ++k) r *= base;
  } else if (mode == 2) {
    r = powf(r, s);
  }
  return r;
}

// _c_calculate_rgc (src/include/_c_sr_radial_gradient_convergence.c:17-90) per
// output pixel, float32 as the reference (the FP64 distance weight is
// evaluated in float), reading the given 2m-magnified gradient images.
__global__ void rgc_kernel(const float* __restrict__ gc, const float* __restrict__ gr,
                           const float* __restrict__ img, int T, int rowsM, int colsM, int M,
                           RgcScalars sc, int iw, float* __restrict__ out) {
  const long long plane = (long long)rowsM * colsM;
  const long long n = plane * T;
  const int grad_w = (int)((float)colsM * 2.0f);
  const long long gplane = (long long)(2 * rowsM) * grad_w;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(idx / plane);
    const long long rem = idx - (long long)t * plane;
    const int yM = (int)(rem / colsM);
    const int xM = (int)(rem - (long long)yM * colsM);
    if (yM < sc.margin || yM >= rowsM - sc.margin || xM < sc.margin ||
        xM >= colsM - sc.margin) {
      out[idx] = 0.f;
      continue;
    }
    const float* Gx = gc + (size_t)t * gplane;
    const float* Gy = gr + (size_t)t * gplane;
    const float xc = __fdiv_rn((float)xM + 0.5f, (float)M);
    const float yc = __fdiv_rn((float)yM + 0.5f, (float)M);
    float rgc = 0.f, wsum = 0.f;
    const int by = (int)(2.0f * yc), bx = (int)(2.0f * xc);
    for (int j = sc.start; j < sc.end; ++j) {
      const float vy = (float)(by + j) / 2.0f;
      if (!(0.f < vy && vy <= (float)(rowsM - 1))) continue;
      for (int i = sc.start; i < sc.end; ++i) {
        const float vx = (float)(bx + i) / 2.0f;
        if (!(0.f < vx && vx <= (float)(colsM - 1))) continue;
        const float dx = vx - xc;
        const float dy = vy - yc;
        const float d = sqrtf(dx * dx + dy * dy);
        if (d != 0.f && d <= sc.tSO) {
          float pos_y = vy * (float)M * 2.0f;
          float pos_x = vx * (float)M * 2.0f;
          if (pos_y >= (float)rowsM * 2.0f) pos_y = (float)rowsM * 2.0f - 1.f;
          if (pos_x >= (float)colsM * 2.0f) pos_x = (float)colsM * 2.0f - 1.f;
          if (pos_y < 0.f) pos_y = 0.f;
          if (pos_x < 0.f) pos_x = 0.f;
          const size_t g = (size_t)(int)pos_y * grad_w + (int)pos_x;
          const float gx = __ldg(Gx + g), gy = __ldg(Gy + g);
          const float tt = d * expf(-(d * d) / sc.tSS);
          const float w = (tt * tt) * (tt * tt);
          wsum += w;
          if (gx * dx + gy * dy < 0.f) {
            float dk = fabsf(gy * dx - gx * dy) / sqrtf(gx * gx + gy * gy);
            if (isnan(dk)) dk = d;
            dk = 1.f - dk / d;
            rgc += dk * w;
          }
        }
      }
    }
    rgc = wsum > 0.f ? rgc / wsum : 0.f;
    rgc = rgc < 0.f ? 0.f : apply_sensitivity(rgc, sc.sens_mode, sc.sens_int, sc.sens);
    out[idx] = iw ? rgc * img[idx] : rgc;
  }
}

// _c_gradient_radiality (src/include/_c_gradients.c:3-25)
__global__ void gradient_radiality_kernel(const float* __restrict__ in, int T, int h, int w,
                                          float* __restrict__ gx, float* __restrict__ gy) {
  const long long plane = (long long)h * w;
  const long long n = plane * T;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(idx / plane);
    const long long rem = idx - (long long)t * plane;
    const int j = (int)(rem / w);
    const int i = (int)(rem - (long long)j * w);
    float vx = 0.f, vy = 0.f;
    if (j >= 1 && j < h - 1 && i >= 1 && i < w - 1) {
      const float* f = in + (size_t)t * plane;
      vx = __fadd_rn(-f[(size_t)j * w + i - 1], f[(size_t)j * w + i + 1]);
      vy = __fadd_rn(-f[(size_t)(j - 1) * w + i], f[(size_t)(j + 1) * w + i]);
    }
    gx[idx] = vx;
    gy[idx] = vy;
  }
}

// _c_calculate_radiality_per_subpixel (src/include/_c_sr_radiality.c:15-51)
__global__ void radiality_kernel(const float* __restrict__ gx, const float* __restrict__ gy,
                                 const float* __restrict__ img_interp, int T, int h, int w,
                                 int M, RingCoords rc, int border, int positivity, int iw,
                                 float* __restrict__ out) {
  const int rowsM = h * M, colsM = w * M;
  const long long plane = (long long)rowsM * colsM;
  const long long n = plane * T;
  const int lo_j = (1 + border) * M, hi_j = (h - 1 - border) * M;
  const int lo_i = (1 + border) * M, hi_i = (w - 1 - border) * M;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int t = (int)(idx / plane);
    const long long rem = idx - (long long)t * plane;
    const int j = (int)(rem / colsM);
    const int i = (int)(rem - (long long)j * colsM);
    if (j < lo_j || j >= hi_j || i < lo_i || i >= hi_i) {
      out[idx] = 0.f;
      continue;
    }
    const float* GX = gx + (size_t)t * h * w;
    const float* GY = gy + (size_t)t * h * w;
    const float xc = (float)i + 0.5f;
    const float yc = (float)j + 0.5f;
    float div = 0.f;
#pragma unroll 2
    for (int s = 0; s < 12; ++s) {
      const float xr = rc.x[s], yr = rc.y[s];
      const float x0 = __fadd_rn(xc, xr);
      const float y0 = __fadd_rn(yc, yr);
      const float ry = __fdiv_rn(y0, (float)M);
      const float rx = __fdiv_rn(x0, (float)M);
      const float vgx = cr_interp(GX, ry, rx, h, w);
      const float vgy = cr_interp(GY, ry, rx, h, w);
      const float gmag = sqrtf(vgx * vgx + vgy * vgy);
      float dk = 0.f;
      if (gmag != 0.f) {
        dk = 1.f - (fabsf(vgy * (xc - x0) - vgx * (yc - y0)) / gmag) / rc.radius;
        dk = dk * dk;
      }
      if (vgx * xr + vgy * yr > 0.f) div -= dk;
      else div += dk;
    }
    div /= 12.f;
    const float cgh = positivity ? fmaxf(div, 0.f) : div;
    out[idx] = iw ? cgh * img_interp[idx] : cgh;
  }
}

// ---------------------------------------------------------------------------
// temporal records: planes mean, M2, C, A, B of Moments (common.cuh)
// ---------------------------------------------------------------------------
__global__ void record_push_frame_kernel(const float* __restrict__ frame, long long n,
                                         float* __restrict__ rec, int it) {
  const float inv = __frcp_rn((float)(it + 1));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = frame[i];
    Moments m = moments_start(v);
    if (it > 0) {
      m = Moments{rec[i], rec[n + i], rec[2 * n + i], rec[3 * n + i], rec[4 * n + i]};
      moments_push(m, v, inv);
    }
    rec[i] = m.mean;
    rec[n + i] = m.m2;
    rec[2 * n + i] = m.c;
    rec[3 * n + i] = m.a;
    rec[4 * n + i] = m.b;
  }
}

__global__ void record_merge_kernel(float* __restrict__ acc, const float* __restrict__ blk,
                                    long long n, int na, int nb) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    Moments a{acc[i], acc[n + i], acc[2 * n + i], acc[3 * n + i], acc[4 * n + i]};
    const Moments b{blk[i], blk[n + i], blk[2 * n + i], blk[3 * n + i], blk[4 * n + i]};
    moments_merge(a, b, na, nb, true);
    acc[i] = a.mean;
    acc[n + i] = a.m2;
    acc[2 * n + i] = a.c;
    acc[3 * n + i] = a.a;
    acc[4 * n + i] = a.b;
  }
}

// Merges the `nchunks` consecutive records of one timepoint in frame order and
// writes the correlations of corr_mask.  full: 5-field records; else one field
// (the mean) per record.
__device__ __forceinline__ void finalize_pixel(const float* __restrict__ rec, int F,
                                               int nchunks, int nf, long long n, int corr_mask,
                                               float* __restrict__ out, long long out_stride,
                                               bool full, long long i) {
  {
    Moments a{0.f, 0.f, 0.f, 0.f, 0.f};
    int na = 0;
    for (int c = 0; c < nchunks; ++c) {
      const int nc = (int)((long long)(c + 1) * nf / nchunks - (long long)c * nf / nchunks);
      const float* r = rec + (size_t)c * F * n;
      Moments b{r[i], 0.f, 0.f, 0.f, 0.f};
      if (full) b = Moments{r[i], r[n + i], r[2 * n + i], r[3 * n + i], r[4 * n + i]};
      moments_merge(a, b, na, nc, full);
      na += nc;
    }
    const float fn = (float)na;
    int ci = 0;
    if (corr_mask & NX_CORR_AVG) out[(ci++) * out_stride + i] = a.mean;
    if (corr_mask & NX_CORR_VAR) {
      const float v = __fdiv_rn(a.m2, fn);
      out[(ci++) * out_stride + i] = v > 0.f ? v : 0.f;
    }
    if (corr_mask & NX_CORR_TAC2) out[(ci++) * out_stride + i] = __fdiv_rn(a.c, fn - 1.f);
  }
}

__global__ void finalize_kernel(const float* __restrict__ rec, int F, int nchunks, int nf,
                                long long n, int corr_mask, float* __restrict__ out,
                                long long out_stride, bool full) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    finalize_pixel(rec, F, nchunks, nf, n, corr_mask, out, out_stride, full, i);
}

// a batch's finalisations in one launch: block -> job by binary search on
// the jobs' first blocks, one pixel per thread
__global__ void finalize_jobs_kernel(const FinalizeJob* __restrict__ jobs, int njobs) {
  int lo = 0, hi = njobs - 1;
  const int bx = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].block0 <= bx) lo = mid;
    else hi = mid - 1;
  }
  const FinalizeJob j = jobs[lo];
  const long long i = (long long)(bx - j.block0) * blockDim.x + threadIdx.x;
  if (i < j.n)
    finalize_pixel(j.rec, j.F, j.nchunks, j.nf, j.n, j.corr_mask, j.out, j.out_stride,
                   j.full != 0, i);
}

// sr_temporal_correlations.py:46-75,205-221 on a resident stack, float32 and
// in numpy's order (sequential over frames, no contraction)
__global__ void temporal_stack_kernel(const float* __restrict__ x, int T, long long n, int corr,
                                      float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int t = 0; t < T; ++t) s = __fadd_rn(s, x[(size_t)t * n + i]);
    const float mean = __fdiv_rn(s, (float)T);
    if (corr == NX_CORR_AVG) {
      out[i] = mean;
    } else if (corr == NX_CORR_VAR) {
      float q = 0.f;
      for (int t = 0; t < T; ++t) {
        const float c = __fsub_rn(x[(size_t)t * n + i], mean);
        q = __fadd_rn(q, __fmul_rn(c, c));
      }
      out[i] = __fdiv_rn(q, (float)T);
    } else {
      float q = 0.f;
      float prev = T > 0 ? __fsub_rn(x[i], mean) : 0.f;
      for (int t = 1; t < T; ++t) {
        const float c = __fsub_rn(x[(size_t)t * n + i], mean);
        q = __fadd_rn(q, __fmul_rn(prev, c));
        prev = c;
      }
      out[i] = __fdiv_rn(q, (float)(T - 1));
    }
  }
}

// VAR and TAC2 with each CTA's 128 pixels x T frames staged in shared memory,
// so the stack is read from HBM once (the two-pass per-pixel kernel reads it
// twice); identical operations and order.
constexpr int kTcPix = 128;
constexpr int kTcMaxFrames = 400;  // 128 x 400 floats = 200 KB of shared memory

__global__ void __launch_bounds__(kTcPix)
    temporal_stack_smem_kernel(const float* __restrict__ x, int T, long long n, int corr,
                               bool vec, float* __restrict__ out) {
  extern __shared__ __align__(16) float ts[];  // [T][kTcPix]
  const long long p0 = (long long)blockIdx.x * kTcPix;
  const int tid = threadIdx.x;
  const long long i = p0 + tid;
  const bool in = i < n;
  if (vec) {
    // every 16-byte piece of the CTA's T x 128 block as one asynchronous copy,
    // all issued before the single wait (enough bytes in flight to fill HBM)
    for (int k = tid; k < T * (kTcPix / 4); k += kTcPix) {
      const int t = k / (kTcPix / 4), c = (k % (kTcPix / 4)) * 4;
      const unsigned dst = smem_addr(ts + t * kTcPix + c);
      const float* src = x + (size_t)t * n + p0 + c;
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    __syncthreads();
  } else {
    for (int t = 0; t < T; ++t) ts[t * kTcPix + tid] = in ? __ldg(x + (size_t)t * n + i) : 0.f;
  }
  if (!in) return;  // each thread reads back only its own column
  float s = 0.f;
  for (int t = 0; t < T; ++t) s = __fadd_rn(s, ts[t * kTcPix + tid]);
  const float mean = __fdiv_rn(s, (float)T);
  if (corr == NX_CORR_AVG) {
    out[i] = mean;
  } else if (corr == NX_CORR_VAR) {
    float q = 0.f;
    for (int t = 0; t < T; ++t) {
      const float c = __fsub_rn(ts[t * kTcPix + tid], mean);
      q = __fadd_rn(q, __fmul_rn(c, c));
    }
    out[i] = __fdiv_rn(q, (float)T);
  } else {
    float q = 0.f;
    float prev = __fsub_rn(ts[tid], mean);
    for (int t = 1; t < T; ++t) {
      const float c = __fsub_rn(ts[t * kTcPix + tid], mean);
      q = __fadd_rn(q, __fmul_rn(prev, c));
      prev = c;
    }
    out[i] = __fdiv_rn(q, (float)(T - 1));
  }
}

// sr_temporal_correlations.py:4-43 (orders 0, 1, -1) and :111-157 (ACRF
// orders 2, 3, 4 without lag-time integration), float32 per pixel
__global__ void srrf_temporal_kernel(const float* __restrict__ x, int T, long long n, int order,
                                     float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (order == 0) {
      float m = -INFINITY;
      for (int t = 0; t < T; ++t) m = fmaxf(m, x[(size_t)t * n + i]);
      out[i] = m;
      continue;
    }
    if (order == -1) {
      // sum_{t0 <= t1} r+_t0 r+_t1 / (T (T + 1) / 2), r+ = max(r, 0)
      float s1 = 0.f, s2 = 0.f;
      for (int t = 0; t < T; ++t) {
        const float r = fmaxf(x[(size_t)t * n + i], 0.f);
        s1 += r;
        s2 = fmaf(r, r, s2);
      }
      const float cnt = 0.5f * (float)T * (float)(T + 1);
      out[i] = 0.5f * (s1 * s1 + s2) / fmaxf(cnt, 1.f);
      continue;
    }
    float s = 0.f;
    for (int t = 0; t < T; ++t) s = __fadd_rn(s, x[(size_t)t * n + i]);
    const float mean = __fdiv_rn(s, (float)T);
    if (order == 1) {
      out[i] = mean;
      continue;
    }
    float ab = 0.f, abc = 0.f, abcd = 0.f, cd = 0.f, ac = 0.f, bd = 0.f, ad = 0.f, bc = 0.f;
    for (int t = 0; t < T - order; ++t) {
      const float a = __fsub_rn(x[(size_t)t * n + i], mean);
      const float b = __fsub_rn(x[(size_t)(t + 1) * n + i], mean);
      ab = __fadd_rn(ab, __fmul_rn(a, b));
      if (order == 3) {
        const float c = __fsub_rn(x[(size_t)(t + 2) * n + i], mean);
        abc = __fadd_rn(__fadd_rn(abc, __fmul_rn(a, b)), c);
      }
      if (order == 4) {
        const float c = __fsub_rn(x[(size_t)(t + 2) * n + i], mean);
        const float d = __fsub_rn(x[(size_t)(t + 3) * n + i], mean);
        abcd = __fadd_rn(abcd, __fmul_rn(__fmul_rn(__fmul_rn(a, b), c), d));
        cd = __fadd_rn(cd, __fmul_rn(c, d));
        ac = __fadd_rn(ac, __fmul_rn(a, c));
        bd = __fadd_rn(bd, __fmul_rn(b, d));
        ad = __fadd_rn(ad, __fmul_rn(a, d));
        bc = __fadd_rn(bc, __fmul_rn(b, c));
      }
    }
    float v;
    if (order == 3) v = fabsf(abc);
    else if (order == 4) v = fabsf(abcd - ab * cd - ac * bd - ad * bc);
    else v = fabsf(ab);
    out[i] = __fdiv_rn(v, (float)T);
  }
}

// ACRF of order 2, 3, 4 with lag-time integration
// (sr_temporal_correlations.py:111-121,159-200), one pixel per thread, the
// reference's float32 operations in its order (no contraction).  Per level:
// the lag products over t < n_iter (ab restarts, abc and the order-4 sums run
// on across levels), and frame t, once read, is replaced in place by
// sum_{k < order-1} frame[t*order + k] / order for t < n_bin (else 0) --
// zeroed first, so the k = 0 term of t = 0 reads the zero.  The last level's
// correlation over n_binned is the result; 0 when no level runs.
__global__ void srrf_acrf_integrated_kernel(float* __restrict__ im, int T, long long n, int order,
                                            AcrfSchedule sch, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float* x = im + i;
    float s = 0.f;
    for (int t = 0; t < T; ++t) s = __fadd_rn(s, x[(size_t)t * n]);
    const float mean = __fdiv_rn(s, (float)T);
    const float fo = (float)order;
    float res = 0.f;
    float abc = 0.f, abcd = 0.f, cd = 0.f, ac = 0.f, bd = 0.f, ad = 0.f, bc = 0.f;
    for (int L = 0; L < sch.n_levels; ++L) {
      float ab = 0.f;
      const int n_iter = sch.n_iter[L], n_bin = sch.n_bin[L];
      for (int t = 0; t < n_iter; ++t) {
        const float a = __fsub_rn(x[(size_t)t * n], mean);
        const float b = __fsub_rn(x[(size_t)(t + 1) * n], mean);
        const float pab = __fmul_rn(a, b);
        ab = __fadd_rn(ab, pab);
        if (order == 3) {
          const float c = __fsub_rn(x[(size_t)(t + 2) * n], mean);
          abc = __fadd_rn(__fadd_rn(abc, pab), c);
        } else if (order == 4) {
          const float c = __fsub_rn(x[(size_t)(t + 2) * n], mean);
          const float d = __fsub_rn(x[(size_t)(t + 3) * n], mean);
          abcd = __fadd_rn(abcd, __fmul_rn(__fmul_rn(pab, c), d));
          cd = __fadd_rn(cd, __fmul_rn(c, d));
          ac = __fadd_rn(ac, __fmul_rn(a, c));
          bd = __fadd_rn(bd, __fmul_rn(b, d));
          ad = __fadd_rn(ad, __fmul_rn(a, d));
          bc = __fadd_rn(bc, __fmul_rn(b, c));
        }
        float v = 0.f;
        if (t < n_bin) {
          const int tb = t * order;
          for (int k = 0; k < order - 1; ++k) {
            const float src = (tb + k == t) ? v : x[(size_t)(tb + k) * n];
            v = __fadd_rn(v, __fdiv_rn(src, fo));
          }
        }
        x[(size_t)t * n] = v;
      }
      float num;
      if (order == 3) {
        num = fabsf(abc);
      } else if (order == 4) {
        num = __fsub_rn(__fsub_rn(__fsub_rn(abcd, __fmul_rn(ab, cd)), __fmul_rn(ac, bd)),
                        __fmul_rn(ad, bc));
        num = fabsf(num);
      } else {
        num = fabsf(ab);
      }
      res = __fdiv_rn(num, sch.n_binned[L]);
    }
    out[i] = res;
  }
}

// macro-pixel map, stage 1: block (s, py, chunk) sums the macro-pixel rows
// [chunk*rpc, (chunk+1)*rpc) of phase row py; thread t owns phase px = t % M
// (blockDim is a multiple of M); Kahan sums, fixed-order block reduction.
__global__ void mpc_partial_kernel(const float* __restrict__ img, int rowsM, int colsM, int M,
                                   int nch, float* __restrict__ part) {
  extern __shared__ float red[];
  const int s = blockIdx.x;
  const int py = blockIdx.y;
  const int ch = blockIdx.z;
  const int rows = rowsM / M, cols = colsM / M;
  const int rpc = (rows + nch - 1) / nch;
  const int r0 = ch * rpc, r1 = min(rows, r0 + rpc);
  const float* f = img + (size_t)s * rowsM * colsM;
  float sum = 0.f, comp = 0.f;
  for (int ry = r0; ry < r1; ++ry) {
    const float* row = f + (size_t)(ry * M + py) * colsM;
    for (int x = threadIdx.x; x < cols * M; x += blockDim.x) {
      const float yk = row[x] - comp;
      const float tk = sum + yk;
      comp = (tk - sum) - yk;
      sum = tk;
    }
  }
  red[threadIdx.x] = sum;
  __syncthreads();
  if ((int)threadIdx.x < M) {
    float tot = 0.f, c2 = 0.f;
    for (int t = threadIdx.x; t < (int)blockDim.x; t += M) {
      const float yk = red[t] - c2;
      const float tk = tot + yk;
      c2 = (tk - tot) - yk;
      tot = tk;
    }
    part[(((size_t)s * M + py) * nch + ch) * M + threadIdx.x] = tot;
  }
}

// stage 2: every block rebuilds its slice's M x M map from the partials (fixed
// order) and divides its pixels by the map value of their phase when non-zero.
__global__ void mpc_apply_kernel(float* __restrict__ img, int rowsM, int colsM, int M, int nch,
                                 const float* __restrict__ part) {
  extern __shared__ float cmap[];
  const int s = blockIdx.y;
  const int rows = rowsM / M, cols = colsM / M;
  const float inv_n = 1.f / (float)((long long)rows * cols);
  for (int k = threadIdx.x; k < M * M; k += blockDim.x) {
    const int py = k / M, px = k % M;
    const float* pp = part + ((size_t)s * M + py) * nch * M + px;
    float tot = 0.f, c2 = 0.f;
    for (int ch = 0; ch < nch; ++ch) {
      const float yk = pp[(size_t)ch * M] - c2;
      const float tk = tot + yk;
      c2 = (tk - tot) - yk;
      tot = tk;
    }
    cmap[k] = (rows * cols > 0) ? tot * inv_n : 0.f;
  }
  __syncthreads();
  const long long plane = (long long)rowsM * colsM;
  float* f = img + (size_t)s * plane;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < plane;
       idx += (long long)gridDim.x * blockDim.x) {
    const int yM = (int)(idx / colsM);
    const int xM = (int)(idx - (long long)yM * colsM);
    const float c = cmap[(yM % M) * M + (xM % M)];
    if (c != 0.f) f[idx] = __fdiv_rn(f[idx], c);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
cudaError_t launch_cr_shift_magnify(const float* in, int T, int H, int W, const float* shift_r,
                                    const float* shift_c, float mag_r, float mag_c, int rowsM,
                                    int colsM, float* out, cudaStream_t s) {
  const long long n = (long long)T * rowsM * colsM;
  if (n == 0) return cudaSuccess;
  if (mag_r >= 1.f && mag_c >= 1.f && T <= 65535 && rowsM / 32 < 65535) {
    // shared memory for the largest tile staging (32 rows at magnification 1,
    // or any tile cr_tile_rows picks: <= 72 KB); each launch uses what its
    // magnifications need
    static const size_t smem_max = std::max<size_t>(cr_tile_smem(32, 1.f, 1.f), 72 * 1024);
    static int attr_dev = -1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (attr_dev != dev) {
      e = cudaFuncSetAttribute(cr_magnify_tiled_kernel,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
      if (e != cudaSuccess) return e;
      attr_dev = dev;
    }
    const int TR = cr_tile_rows(mag_r, mag_c);
    const int PR = cr_patch_extent(TR, mag_r), PC = cr_patch_extent(kCrTileCols, mag_c);
    const size_t smem = cr_tile_smem(TR, mag_r, mag_c);
    const dim3 grid((unsigned)((colsM + kCrTileCols - 1) / kCrTileCols),
                    (unsigned)((rowsM + TR - 1) / TR), (unsigned)T);
    cr_magnify_tiled_kernel<<<grid, kCrTileCols, smem, s>>>(in, H, W, shift_r, shift_c, mag_r,
                                                            mag_c, rowsM, colsM, TR, PR, PC, out);
    return cudaGetLastError();
  }
  cr_shift_magnify_kernel<<<grid_for(n), kBlock, 0, s>>>(in, T, H, W, shift_r, shift_c, mag_r,
                                                         mag_c, rowsM, colsM, out);
  return cudaGetLastError();
}

cudaError_t launch_roberts_cross(const float* in, int T, int H, int W, float* gc, float* gr,
                                 cudaStream_t s) {
  const long long n = (long long)T * H * W;
  if (n == 0) return cudaSuccess;
  roberts_cross_kernel<<<grid_for(n), kBlock, 0, s>>>(in, T, H, W, gc, gr);
  return cudaGetLastError();
}

RgcScalars rgc_scalars(int M, float radius, float sensitivity, int pad_edges) {
  RgcScalars sc{};
  const float sigma = (float)((double)radius / 2.355);
  const float fwhm = radius;
  sc.tSS = 2.0f * sigma * sigma;
  sc.tSO = 2.0f * sigma + 1.0f;
  sc.start = -(int)(2.0f * fwhm);
  sc.end = (int)(2.0f * fwhm + 1.0f);
  sc.margin = pad_edges ? 0 : (int)((double)fwhm * (double)M);
  sc.sens = sensitivity;
  if (!(sensitivity > 1.0f)) {
    sc.sens_mode = 0;
  } else if (sensitivity == std::floor(sensitivity) && sensitivity <= 16.0f) {
    sc.sens_mode = 1;
    sc.sens_int = (int)sensitivity;
  } else {
    sc.sens_mode = 2;
  }
  return sc;
}

cudaError_t launch_rgc(const float* gc, const float* gr, const float* img, int T, int rowsM,
                       int colsM, int M, const RgcScalars& sc, int iw, float* out,
                       cudaStream_t s) {
  const long long n = (long long)T * rowsM * colsM;
  if (n == 0) return cudaSuccess;
  rgc_kernel<<<grid_for(n), kBlock, 0, s>>>(gc, gr, img, T, rowsM, colsM, M, sc, iw, out);
  return cudaGetLastError();
}

cudaError_t launch_gradient_radiality(const float* in, int T, int h, int w, float* gx, float* gy,
                                      cudaStream_t s) {
  const long long n = (long long)T * h * w;
  if (n == 0) return cudaSuccess;
  gradient_radiality_kernel<<<grid_for(n), kBlock, 0, s>>>(in, T, h, w, gx, gy);
  return cudaGetLastError();
}

RingCoords ring_coords(int M, float ring_radius) {
  // _le_radiality.pyx:92-104: float32 ring of 12 points at ringRadius * m
  RingCoords rc{};
  rc.radius = (float)((double)ring_radius * (double)M);
  const float step = (float)((3.14159265358979323846 * 2.0) / 12.0);
  for (int k = 0; k < 12; ++k) {
    const float arg = step * (float)k;
    rc.x[k] = (float)(std::cos((double)arg) * (double)rc.radius);
    rc.y[k] = (float)(std::sin((double)arg) * (double)rc.radius);
  }
  return rc;
}

cudaError_t launch_radiality(const float* gx, const float* gy, const float* img_interp, int T,
                             int h, int w, int M, const RingCoords& rc, int border, int positivity,
                             int iw, float* out, cudaStream_t s) {
  const long long n = (long long)T * h * M * w * M;
  if (n == 0) return cudaSuccess;
  radiality_kernel<<<grid_for(n), kBlock, 0, s>>>(gx, gy, img_interp, T, h, w, M, rc, border,
                                                  positivity, iw, out);
  return cudaGetLastError();
}

cudaError_t launch_record_push_frame(const float* frame, long long n, float* rec, int it,
                                     cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  record_push_frame_kernel<<<grid_for(n), kBlock, 0, s>>>(frame, n, rec, it);
  return cudaGetLastError();
}

cudaError_t launch_record_merge(float* acc, const float* blk, long long n, int n_acc, int n_blk,
                                cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  record_merge_kernel<<<grid_for(n), kBlock, 0, s>>>(acc, blk, n, n_acc, n_blk);
  return cudaGetLastError();
}

cudaError_t launch_finalize_jobs(const FinalizeJob* jobs, int njobs, int total_blocks,
                                 cudaStream_t s) {
  if (njobs == 0 || total_blocks == 0) return cudaSuccess;
  finalize_jobs_kernel<<<total_blocks, kBlock, 0, s>>>(jobs, njobs);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const float* rec, int F, int nchunks, int nf, long long n,
                            int corr_mask, float* out, long long out_stride, bool full,
                            cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  finalize_kernel<<<grid_for(n), kBlock, 0, s>>>(rec, F, nchunks, nf, n, corr_mask, out,
                                                 out_stride, full);
  return cudaGetLastError();
}

cudaError_t launch_temporal_stack(const float* stack, int T, long long n, int corr, float* out,
                                  cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const long long blocks = (n + kTcPix - 1) / kTcPix;
  // AVG reads the stack once in the per-pixel kernel already; VAR and TAC2
  // re-read it there, so they stage each pixel block in shared memory
  if (corr != NX_CORR_AVG && T >= 1 && T <= kTcMaxFrames && blocks <= 0x7fffffffLL) {
    // 16-byte copies need a 16-byte aligned base, whole 4-pixel pieces in every
    // frame (n % 4 == 0) and a whole last block
    const bool vec = (reinterpret_cast<uintptr_t>(stack) & 15u) == 0 && n % kTcPix == 0;
    static int attr_dev = -1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (attr_dev != dev) {
      e = cudaFuncSetAttribute(temporal_stack_smem_kernel,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(kTcMaxFrames * kTcPix * sizeof(float)));
      if (e != cudaSuccess) return e;
      attr_dev = dev;
    }
    temporal_stack_smem_kernel<<<(unsigned)blocks, kTcPix, (size_t)T * kTcPix * sizeof(float),
                                 s>>>(stack, T, n, corr, vec, out);
    return cudaGetLastError();
  }
  temporal_stack_kernel<<<grid_for(n), kBlock, 0, s>>>(stack, T, n, corr, out);
  return cudaGetLastError();
}

cudaError_t launch_srrf_temporal(const float* stack, int T, long long n, int order, float* out,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  srrf_temporal_kernel<<<grid_for(n), kBlock, 0, s>>>(stack, T, n, order, out);
  return cudaGetLastError();
}

cudaError_t launch_srrf_acrf_integrated(float* im, int T, long long n, int order,
                                        const AcrfSchedule& sch, float* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  srrf_acrf_integrated_kernel<<<grid_for(n), kBlock, 0, s>>>(im, T, n, order, sch, out);
  return cudaGetLastError();
}

// partial-sum chunks of the macro-pixel map per (slice, phase row)
static int mpc_chunks(int rowsM, int M) { return std::max(1, std::min(kMpcChunks, rowsM / M)); }

size_t mpc_scratch_bytes(int S, int rowsM, int M) {
  return (size_t)std::max(S, 1) * M * M * mpc_chunks(rowsM, M) * sizeof(float);
}

cudaError_t launch_mpc(float* img, int S, int rowsM, int colsM, int M, float* map,
                       cudaStream_t s) {
  if ((long long)S * rowsM * colsM == 0) return cudaSuccess;
  const int rows = rowsM / M;
  const int nch = mpc_chunks(rowsM, M);
  const int block = M <= 32 ? 32 * M : ((1024 / M) * M);
  if (rows > 0) {
    mpc_partial_kernel<<<dim3((unsigned)S, (unsigned)M, (unsigned)nch), block,
                         block * sizeof(float), s>>>(img, rowsM, colsM, M, nch, map);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  } else {
    cudaError_t e = cudaMemsetAsync(map, 0, (size_t)S * M * M * nch * sizeof(float), s);
    if (e != cudaSuccess) return e;
  }
  const long long plane = (long long)rowsM * colsM;
  unsigned gx = (unsigned)std::min<long long>((plane + 1023) / 1024, 4096);
  mpc_apply_kernel<<<dim3(gx, (unsigned)S), 256, (size_t)M * M * sizeof(float), s>>>(
      img, rowsM, colsM, M, nch, map);
  return cudaGetLastError();
}

}  // namespace nx
