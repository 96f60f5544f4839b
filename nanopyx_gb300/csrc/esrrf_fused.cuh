// Fused eSRRF frame-loop kernel (sm_103a), warp-specialised.
//
// One CTA works through units -- (stack, 32 x TY tile of input pixels = a
// 32M x TY*M tile of output pixels, timepoint, frame chunk) -- two frames per
// pass.  Its producer warps, per pass,
//   1. receive the input tiles + halo by TMA (two sets of buffers, mbarrier),
//      or by plain loads when the row pitch is not 16-byte aligned;
//   2. compute Roberts-Cross gradients          (_c_gradients.c:53-73) and the
//      row pass of the intensity magnification  (_c_interpolation_catmull_rom.c:21-52);
//   3. Catmull-Rom-interpolate the gradients on the half-pixel grid -- the only
//      positions the reference RGC ever reads from its 2m-magnified gradient
//      images (rows/cols k*m, clamped to 2*m*H-1;
//      _c_sr_radial_gradient_convergence.c:45-61) -- on packed f32x2
//      arithmetic over the frame pair, and normalise them into a
//      double-buffered slot;
// while its consumer warps, one thread per input pixel and output row phase,
//   4. evaluate RGC for the thread's M output pixels with FP64-derived phase
//      tables of the distance weights      (_c_sr_radial_gradient_convergence.c:17-90),
//      on packed f32x2 arithmetic (both frames in one register pair);
//   5. apply ^sensitivity, the intensity (column pass) and the margin, and
//      either write the per-frame value (eSRRF_ST stack) or fold it into
//      per-pixel streaming temporal moments kept in shared memory (Welford
//      mean and M2, lag-1 co-moment, last and first value as deviations; see
//      Moments).
// Nothing of size (T, 2Hm, 2Wm) or (T, Hm, Wm) is ever materialised for the
// temporal modes.
#pragma once

#include <cuda.h>

#include <algorithm>

#include "common.cuh"

namespace nx {

enum FusedMode : int { kModeStack = 0, kModeSum = 1, kModeFull = 2 };

__host__ __device__ constexpr int mode_fields(int mode) {
  return mode == kModeFull ? 5 : (mode == kModeSum ? 1 : 0);
}

constexpr int kMaxSens = 4;    // sensitivities sharing one RGC pass (AVG mode)
constexpr int kMaxTmaps = 24;  // TMA descriptors carried in the kernel parameters

struct FusedParams {
  const float* in;     // (T, H, W)
  int T, H, W;
  int rowsM, colsM;
  int tiles_x;
  int fpt;             // frames per timepoint
  int n_tp;            // number of timepoints
  int chunks;          // chunks per timepoint (the last timepoint uses min(chunks, its frames))
  int margin;
  int iw;
  int cy_base, cx_base;  // first tap row/col of the clamped half-grid index 2H / 2W
  float cy[4], cx[4];
  const float* tbl;      // [M][2J+1][3][NS4*4]  (a = dx*w/d, b = dy*w/d, w) per sample
  const float* inv_wsum; // [M][M]
  const float* wfull;    // [M][M][2J+1][2J+1]
  float* out;            // stack (T, rowsM, colsM) or records [n_tp*chunks][F][rowsM][colsM]
  unsigned* status;
  int tmap;              // index into the kernel's TMA descriptor pack, or -1: plain loads
  int tiles_y;
  int F;                 // record fields: 5 (VAR/TAC2) or n_sens (AVG: the mean per sensitivity)
  int n_sens;            // AVG mode: sensitivities evaluated on the same RGC (others: 1)
  int sens_mode_k[kMaxSens];  // 0: none (s <= 1), 1: integer power sens_int_k, 2: powf(sens_k)
  int sens_int_k[kMaxSens];
  float sens_k[kMaxSens];
  unsigned long long wait_ns;  // bound of every producer/consumer wait (0: kWaitLimitNs)
  // failure-detection self-test only (0 in every computation): the producers
  // withhold the `full` arrival of the first pass of each CTA's first unit, so
  // the consumers' bounded wait runs out and the CTA takes its abort path
  int test_withhold_full;
};

struct TmapPack {
  CUtensorMap m[kMaxTmaps];
};

// Work list of one launch: units = (item, tile, timepoint, frame chunk), tiles
// fastest.  One item may be carried by value (`single`); several live in
// device memory with their first unit index in `unit_start`.  With `counter`
// CTAs take units dynamically (persistent launch), else unit = blockIdx.x.
struct UnitTable {
  const FusedParams* items;
  const int* unit_start;  // [n_items + 1]
  int n_items;
  int total_units;
  unsigned* counter;
  int ns_cap;  // largest n_sens among the items (sizes the AVG-mode temporal state)
  FusedParams single;
};

template <int M>
struct TileRows {
  // input-pixel rows per CTA tile (32*TY*M threads <= 640); measured: TY = 4 beats
  // TY = 2 at m = 5 by 4 % despite one CTA per SM (less halo work per pixel)
  static constexpr int TY = (M <= 2) ? 8 : (M <= 5 ? 4 : 2);
};

// Warp roles of the eSRRF kernel.  Each CTA runs 32 * TY * M consumer threads
// (one per input pixel and output row phase: RGC, normalisation, temporal
// update) and one producer warpgroup that prepares the gradient and intensity
// tiles of the next frames (TMA, Roberts-Cross, Catmull-Rom passes,
// normalisation) into a double-buffered slot while the consumers work on the
// current one.  The consumers' RGC is FMA-pipe bound and the preparation is
// load/ALU bound, so the two overlap on the SM.
template <int M, int V = 0>
struct EsrrfTile {
  // rows per tile: as many consumer warps as the registers allow without
  // spilling (m = 5: 20 consumer + 4 producer warps at 80 registers measured
  // 12 % faster than 15 + 4 at 96, 40 % faster than 10 + 4)
  static constexpr int TY = (M <= 2) ? 8 : (M <= 5 ? 4 : (M == 6 ? 2 : 1));
  // producer threads: the preparation per input pixel is the same for every m
  // while the RGC work grows with m^2, so small m needs more producers.
  // Measured (200 x 512 x 512, VAR): m = 5 best with one warpgroup (96 or 64
  // threads slower); m = 2: 6.31 / 4.74 / 4.15 / 4.23 ms with 128 / 256 / 384 /
  // 512; m = 3: 9.23 / 7.60 / 7.75 ms with 128 / 256 / 384; m = 4 (4 rows):
  // 12.12 / 11.82 ms with 128 / 256 (3 rows: 12.41 / 12.48); m = 5: 16.92 /
  // 18.11 ms with 128 / 256.
  // Tile variant V = 1 (instantiated for m = 2, 4, 5) has one producer warp
  // group fewer (m = 5: 3 warps), for the tiling autotuner to weigh against
  // the default on a given batch.
  static constexpr int NP_DEFAULT = (M <= 2) ? 384 : (M <= 4 ? 256 : 128);
  static constexpr int NP_ALT = (M <= 2) ? 256 : (M <= 4 ? 128 : 96);
  static constexpr int NP = V == 0 ? NP_DEFAULT : NP_ALT;
  static constexpr int NT = 32 * TY * M + NP;
  // one CTA per SM: registers for the consumers (m = 8 with 2 CTAs per SM at
  // 80 registers measured 11 % slower than 1 CTA)
  static constexpr int MIN_BLOCKS = 1;
};

// Frames per pass (FP).  With FP = 2 a consumer carries two consecutive frames
// through each pass: the RGC core runs on packed f32x2 arithmetic (frame pair
// in one register pair, one phase-table load for both frames) and the
// producers share their index and weight work between the two frames.
// Results are bit-identical to FP = 1 (the same IEEE operations per frame).
// Instantiations whose FP = 2 shared-memory layout does not fit a CTA use FP = 1.
template <int M, int J, int TY, int FP, int NP_ = EsrrfTile<M>::NP>
struct Geo {
  static constexpr int TX = 32;
  static constexpr int W2 = 2 * J + 1;
  static constexpr int NQ = 2 * J + 2;
  static constexpr int HG_R = 2 * TY + 2 * J;
  static constexpr int HG_C = 2 * TX + 2 * J;
  static constexpr int HGP = TX + J;
  static constexpr int RLO = (J + 1) / 2 + 2;
  static constexpr int RHI = TY + (J - 1) / 2 + 2;
  static constexpr int NRY = RLO + RHI;
  static constexpr int CLO = (J + 1) / 2 + 2;
  static constexpr int CHI = TX + (J - 1) / 2 + 2;
  static constexpr int NCX = CLO + CHI;
  static constexpr int IY = RLO + 1;
  static constexpr int BH = NRY + 1;
  static constexpr int IX = ((CLO + 1 + 3) / 4) * 4;
  static constexpr int BW = ((IX + CHI + 3) / 4) * 4;
  static constexpr int NS = M * W2;
  static constexpr int NS4 = (NS + 3) / 4;
  static constexpr int OY = TY * M;
  static constexpr int OX = TX * M;
  static constexpr int RIW = TX + 4;
  static constexpr int NTC = 32 * TY * M;        // consumer threads
  static constexpr int NP = NP_;                 // producer threads
  static constexpr int NT = NTC + NP;
  // prepared passes in flight between producers and consumers (3 or 4
  // measured no faster: the producers keep up)
  static constexpr int NSLOT = 2;
  // phase-table block per (py, jj), in float4:
  //   FP = 1: a[NS4] b[NS4] w[NS4]   (4 samples per float4)
  //   FP = 2: (a, b, -b, w) per sample, each value broadcast into a frame pair
  //           (measured 12 % faster than storing the pairs duplicated)
  static constexpr int TBLK = FP >= 2 ? 4 * NS4 : 3 * NS4;
  // unit gradients of one slot: FP = 1: float2 (nx, ny) per half-grid sample;
  // FP >= 2: one plane per frame pair of float4 (nx0, nx1, ny0, ny1)
  static constexpr int HG_PLANE = HG_R * 2 * HGP;  // samples per plane

  __host__ __device__ static constexpr int al(int n) { return (n + 31) / 32 * 32; }
  // shared-memory layout (in floats, 128-byte aligned blocks)
  static constexpr int O_INB = 0;
  static constexpr int S_INB = al(BH * BW);  // 2 * FP input tiles (two sets of FP frames)
  static constexpr int O_G = O_INB + 2 * FP * S_INB;
  static constexpr int S_G = al(NRY * NCX);  // Roberts-Cross gc, gr per frame
  static constexpr int O_T1 = O_G + 2 * FP * S_G;
  static constexpr int S_T1 = al(NRY * HG_C);  // column-pass gx, gy per frame
  static constexpr int O_HG = O_T1 + 2 * FP * S_T1;
  static constexpr int S_HG = al(HG_R * 2 * HGP * 2 * FP);  // one slot: float2 / float4 gradients
  static constexpr int O_RI = O_HG + NSLOT * S_HG;          // NSLOT slots
  static constexpr int S_RI = al(OY * RIW);  // intensity row pass per frame
  static constexpr int O_TB = O_RI + NSLOT * FP * S_RI;     // NSLOT slots of FP planes
  static constexpr int S_TB = al(M * W2 * TBLK * 4);
  static constexpr int O_RW = O_TB + S_TB;
  static constexpr int S_RW = al(OY * 5);
  static constexpr int O_CW = O_RW + S_RW;
  static constexpr int S_CW = al(OX * 5);
  // per-output temporal state kept out of registers, [px][consumer] planes:
  //   FULL: float4 (mean, M2, C, A) then float B;  SUM: the mean per sensitivity
  static constexpr int O_TW = O_CW + S_CW;     // 1 / sum w per output
  static constexpr int O_TK = O_TW + M * NTC;
  static constexpr int S_TK_FULL = 5 * M * NTC;
  static constexpr int O_BAR_FULL = O_TK + S_TK_FULL;
  // AVG mode keeps the running mean of ns_cap sensitivities per output
  __host__ __device__ static constexpr int o_bar(int mode, int ns_cap) {
    return mode == 1 ? O_TK + ns_cap * M * NTC : (mode == 2 ? O_BAR_FULL : O_TK);
  }
  // 2 NSLOT + 1 + 2 FP (<= 11) mbarriers after o_bar
  __host__ __device__ static constexpr size_t smem_bytes(int mode, int ns_cap) {
    return size_t(o_bar(mode, ns_cap) + 32) * 4;
  }
};

constexpr size_t kMaxSmemPerBlock = 227 * 1024;
constexpr size_t kSmemBudget = kMaxSmemPerBlock - sizeof(FusedParams) - 64;

// compile-time configuration of one instantiation
template <int M, int J, int MODE, int V = 0>
struct FusedCfg {
  static constexpr int TY = EsrrfTile<M, V>::TY;
  static constexpr int NP = EsrrfTile<M, V>::NP;
  static constexpr int NSC = MODE == kModeSum ? kMaxSens : 1;
  // FP = 4 (two frame pairs per pass sharing the table loads) is supported by
  // the code but not selected: it does not fit shared memory with the VAR/TAC2
  // or AVG state at m = 5, and in stack mode it measured 9 % slower.
  static constexpr int FP = Geo<M, J, TY, 2, NP>::smem_bytes(MODE, NSC) <= kSmemBudget ? 2 : 1;
  using G = Geo<M, J, TY, FP, NP>;
};

__device__ __forceinline__ float f4c(const float4& v, int e) {
  return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}

__device__ __forceinline__ float apply_sens(float r, int mode, int n, float s) {
  if (mode == 1) {
    const float base = r;
    for (int k = 1; k < n; ++k) r *= base;
  } else if (mode == 2) {
    r = powf(r, s);
  }
  return r;
}

// geometry of one unit (tile, timepoint, frame chunk), shared by both roles
struct UnitGeo {
  int nx0, ny0, H, W, f0, f1;
  int kb_y, kb_x, RY0, CX0, y_start, x_start, kmax_y, kmax_x;
};

// ---------------------------------------------------------------------------
// producer warpgroup: input tiles -> slot s (unit gradients hg, intensity rows ri)
// ---------------------------------------------------------------------------
template <int M, int J, int TY, int FP, int NP>
struct Producer {
  using G = Geo<M, J, TY, FP, NP>;
  float* inb;
  // Roberts-Cross gradients and the column pass's half-grid columns:
  //   FP = 1: plane 0 gc / gx, plane 1 gr / gy;
  //   FP >= 2: per frame pair pp one plane of float4 (gc, gc', gr, gr') /
  //            (gx, gx', gy, gy'), so the passes run on packed frame pairs
  float* gsm;
  float* t1;
  float* hg0;  // slot 0; slot s at hg0 + s * S_HG
  float* ri0;  // slot s, frame fr at ri0 + (s * FP + fr) * S_RI
  const float* rw;
  int ptid;

  __device__ void roberts_and_rows(const FusedParams& p, const UnitGeo& u, const float* const* tin,
                                   int s) const {
    for (int i = ptid; i < G::NRY * G::NCX; i += G::NP) {
      const int rl = i / G::NCX, cl = i % G::NCX;
      const int r = u.RY0 + rl, c = u.CX0 + cl;
      const bool in = r >= 0 && r < u.H && c >= 0 && c < u.W;
      const int r0 = r > 0 ? r - 1 : 0;
      const int c0 = c > 0 ? c - 1 : 0;
      const int ia = (r0 - u.y_start) * G::BW + (c - u.x_start);   // image[r0][c1]
      const int ib = (r - u.y_start) * G::BW + (c0 - u.x_start);   // image[r1][c0]
      const int id = (r0 - u.y_start) * G::BW + (c0 - u.x_start);  // image[r0][c0]
      const int ie = (r - u.y_start) * G::BW + (c - u.x_start);    // image[r1][c1]
      float gc[FP], gr[FP];
#pragma unroll
      for (int fr = 0; fr < FP; ++fr) {
        gc[fr] = gr[fr] = 0.f;
        if (in) {
          const float a = tin[fr][ia], bb = tin[fr][ib], d = tin[fr][id], e = tin[fr][ie];
          gc[fr] = __fsub_rn(__fadd_rn(__fsub_rn(a, bb), e), d);
          gr[fr] = __fsub_rn(__fadd_rn(__fadd_rn(-a, bb), e), d);
        }
      }
      if constexpr (FP >= 2) {
        // frame pair pp: float4 (gc, gc', gr, gr') per position
#pragma unroll
        for (int pp = 0; pp < FP / 2; ++pp)
          reinterpret_cast<float4*>(gsm)[pp * G::S_G + i] =
              make_float4(gc[2 * pp], gc[2 * pp + 1], gr[2 * pp], gr[2 * pp + 1]);
      } else {
        gsm[i] = gc[0];
        gsm[G::S_G + i] = gr[0];
      }
    }
    float* ri = ri0 + s * FP * G::S_RI;
    for (int i = ptid; i < G::OY * G::RIW; i += G::NP) {
      const int oy = i / G::RIW, cc = i % G::RIW;
      const int nyo = u.ny0 + oy / M;
      float w5[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) w5[k] = rw[oy * 5 + k];
      const int off = (nyo - 2 - u.y_start) * G::BW + (u.nx0 - 2 + cc - u.x_start);
#pragma unroll
      for (int fr = 0; fr < FP; ++fr) {
        const float* col = tin[fr] + off;
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < 5; ++k) sum = fmaf(w5[k], col[k * G::BW], sum);
        ri[fr * G::S_RI + i] = sum;
      }
    }
  }

  // gradient column pass onto the half-grid columns
  // (each row's even half-grid columns first, then its odd ones, so that the
  // lanes of a warp mostly take the same odd / even branch).  With frame
  // pairs the planes hold float4 (x, x', y, y') per position and the taps run
  // as packed f32x2 operations: the same IEEE operations per frame.
  __device__ void column_pass(const FusedParams& p, const UnitGeo& u) const {
    const int twoW = 2 * u.W;
    constexpr int HALF = (G::HG_C + 1) / 2;
    for (int i = ptid; i < G::NRY * G::HG_C; i += G::NP) {
      const int rl = i / G::HG_C, j = i - rl * G::HG_C;
      const int kxl = j < HALF ? 2 * j : 2 * (j - HALF) + 1;
      const int o = rl * G::HG_C + kxl;
      const int kx = u.kb_x + kxl;
      const bool valid = kx >= 1 && kx <= u.kmax_x;
      if constexpr (FP >= 2) {
#pragma unroll
        for (int pp = 0; pp < FP / 2; ++pp) {
          const float4* g4 = reinterpret_cast<const float4*>(gsm) + pp * G::S_G + rl * G::NCX;
          float2 vc = make_float2(0.f, 0.f), vr = make_float2(0.f, 0.f);
          if (valid) {
            if (kx >= twoW) {
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                const float4 q = g4[p.cx_base + t - u.CX0];
                const float2 w = make_float2(p.cx[t], p.cx[t]);
                vc = __ffma2_rn(w, make_float2(q.x, q.y), vc);
                vr = __ffma2_rn(w, make_float2(q.z, q.w), vr);
              }
            } else if (kx & 1) {
              const float4 q = g4[((kx - 1) >> 1) - u.CX0];
              vc = make_float2(q.x, q.y);
              vr = make_float2(q.z, q.w);
            } else {
              const float4* g = g4 + (kx >> 1) - 2 - u.CX0;
              const float2 c0 = make_float2(-0.0625f, -0.0625f);
              const float2 c1 = make_float2(0.5625f, 0.5625f);
              const float4 q0 = g[0], q1 = g[1], q2 = g[2], q3 = g[3];
              vc = __fmul2_rn(c0, make_float2(q0.x, q0.y));
              vr = __fmul2_rn(c0, make_float2(q0.z, q0.w));
              vc = __ffma2_rn(c1, make_float2(q1.x, q1.y), vc);
              vr = __ffma2_rn(c1, make_float2(q1.z, q1.w), vr);
              vc = __ffma2_rn(c1, make_float2(q2.x, q2.y), vc);
              vr = __ffma2_rn(c1, make_float2(q2.z, q2.w), vr);
              vc = __ffma2_rn(c0, make_float2(q3.x, q3.y), vc);
              vr = __ffma2_rn(c0, make_float2(q3.z, q3.w), vr);
            }
          }
          reinterpret_cast<float4*>(t1)[pp * G::S_T1 + o] = make_float4(vc.x, vc.y, vr.x, vr.y);
        }
      } else {
        const float* g0 = gsm + rl * G::NCX;
        const float* g1 = gsm + G::S_G + rl * G::NCX;
        float vc = 0.f, vr = 0.f;
        if (valid) {
          if (kx >= twoW) {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const int cl = p.cx_base + t - u.CX0;
              vc = fmaf(p.cx[t], g0[cl], vc);
              vr = fmaf(p.cx[t], g1[cl], vr);
            }
          } else if (kx & 1) {
            const int cl = ((kx - 1) >> 1) - u.CX0;
            vc = g0[cl];
            vr = g1[cl];
          } else {
            const int cl = (kx >> 1) - 2 - u.CX0;
            float c = -0.0625f * g0[cl], r = -0.0625f * g1[cl];
            c = fmaf(0.5625f, g0[cl + 1], c);
            r = fmaf(0.5625f, g1[cl + 1], r);
            c = fmaf(0.5625f, g0[cl + 2], c);
            r = fmaf(0.5625f, g1[cl + 2], r);
            vc = fmaf(-0.0625f, g0[cl + 3], c);
            vr = fmaf(-0.0625f, g1[cl + 3], r);
          }
        }
        t1[o] = vc;
        t1[G::S_T1 + o] = vr;
      }
    }
  }

  // gradient row pass and normalisation -> unit gradients of slot s
  __device__ void row_pass(const FusedParams& p, const UnitGeo& u, int s) const {
    const int twoH = 2 * u.H;
    float* hgf = hg0 + s * G::S_HG;
    for (int i = ptid; i < G::HG_R * G::HG_C; i += G::NP) {
      const int kyl = i / G::HG_C, kxl = i % G::HG_C;
      const int ky = u.kb_y + kyl, kx = u.kb_x + kxl;
      const bool valid = ky >= 1 && ky <= u.kmax_y && kx >= 1 && kx <= u.kmax_x;
      float gx[FP], gy[FP];
#pragma unroll
      for (int fr = 0; fr < FP; ++fr) gx[fr] = gy[fr] = 0.f;
      if (valid) {
        if constexpr (FP >= 2) {
#pragma unroll
          for (int pp = 0; pp < FP / 2; ++pp) {
            const float4* c4 = reinterpret_cast<const float4*>(t1) + pp * G::S_T1 + kxl;
            float2 x = make_float2(0.f, 0.f), y = make_float2(0.f, 0.f);
            if (ky >= twoH) {
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                const float4 q = c4[(p.cy_base + t - u.RY0) * G::HG_C];
                const float2 w = make_float2(p.cy[t], p.cy[t]);
                x = __ffma2_rn(w, make_float2(q.x, q.y), x);
                y = __ffma2_rn(w, make_float2(q.z, q.w), y);
              }
            } else if (ky & 1) {
              const float4 q = c4[(((ky - 1) >> 1) - u.RY0) * G::HG_C];
              x = make_float2(q.x, q.y);
              y = make_float2(q.z, q.w);
            } else {
              const float4* c = c4 + ((ky >> 1) - 2 - u.RY0) * G::HG_C;
              const float2 c0 = make_float2(-0.0625f, -0.0625f);
              const float2 c1 = make_float2(0.5625f, 0.5625f);
              const float4 q0 = c[0], q1 = c[G::HG_C], q2 = c[2 * G::HG_C], q3 = c[3 * G::HG_C];
              x = __fmul2_rn(c0, make_float2(q0.x, q0.y));
              y = __fmul2_rn(c0, make_float2(q0.z, q0.w));
              x = __ffma2_rn(c1, make_float2(q1.x, q1.y), x);
              y = __ffma2_rn(c1, make_float2(q1.z, q1.w), y);
              x = __ffma2_rn(c1, make_float2(q2.x, q2.y), x);
              y = __ffma2_rn(c1, make_float2(q2.z, q2.w), y);
              x = __ffma2_rn(c0, make_float2(q3.x, q3.y), x);
              y = __ffma2_rn(c0, make_float2(q3.z, q3.w), y);
            }
            gx[2 * pp] = x.x;
            gx[2 * pp + 1] = x.y;
            gy[2 * pp] = y.x;
            gy[2 * pp + 1] = y.y;
          }
        } else {
          const float* c0 = t1 + kxl;
          const float* c1 = t1 + G::S_T1 + kxl;
          if (ky >= twoH) {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const int rl = p.cy_base + t - u.RY0;
              gx[0] = fmaf(p.cy[t], c0[rl * G::HG_C], gx[0]);
              gy[0] = fmaf(p.cy[t], c1[rl * G::HG_C], gy[0]);
            }
          } else if (ky & 1) {
            const int rl = ((ky - 1) >> 1) - u.RY0;
            gx[0] = c0[rl * G::HG_C];
            gy[0] = c1[rl * G::HG_C];
          } else {
            const int rl = (ky >> 1) - 2 - u.RY0;
            const float* a0 = c0 + rl * G::HG_C;
            const float* a1 = c1 + rl * G::HG_C;
            float x = -0.0625f * a0[0], y = -0.0625f * a1[0];
            x = fmaf(0.5625f, a0[G::HG_C], x);
            y = fmaf(0.5625f, a1[G::HG_C], y);
            x = fmaf(0.5625f, a0[2 * G::HG_C], x);
            y = fmaf(0.5625f, a1[2 * G::HG_C], y);
            gx[0] = fmaf(-0.0625f, a0[3 * G::HG_C], x);
            gy[0] = fmaf(-0.0625f, a1[3 * G::HG_C], y);
          }
        }
      }
      float nxv[FP], nyv[FP];
#pragma unroll
      for (int fr = 0; fr < FP; ++fr) {
        nxv[fr] = nyv[fr] = 0.f;
        const float m2 = fmaf(gx[fr], gx[fr], gy[fr] * gy[fr]);
        if (valid && m2 > 0.f) {
          const float inv = rsqrtf(m2);
          nxv[fr] = gx[fr] * inv;
          nyv[fr] = gy[fr] * inv;
        }
      }
      const int o = (kyl * 2 + (kxl & 1)) * G::HGP + (kxl >> 1);
      if constexpr (FP >= 2) {
#pragma unroll
        for (int pp = 0; pp < FP / 2; ++pp)
          reinterpret_cast<float4*>(hgf)[pp * G::HG_PLANE + o] =
              make_float4(nxv[2 * pp], nxv[2 * pp + 1], nyv[2 * pp], nyv[2 * pp + 1]);
      } else {
        reinterpret_cast<float2*>(hgf)[o] = make_float2(nxv[0], nyv[0]);
      }
    }
  }
};

// Numerator of the horizontal offset of RGC sample (px, ii) from its output's
// centre, 2 M dx = M (cpx + ii - J) - (2 px + 1); its sign is the sign of the
// table's a = dx w / d (zero exactly when dx is).
template <int M, int J>
__host__ __device__ constexpr int dx_num(int px, int ii) {
  return M * ((2 * px + 1) / M + ii - J) - (2 * px + 1);
}

// RGC of one consumer's M outputs for the FP frames of slot hgf.
// Contribution of sample (phase, offset): (dp < 0) ? w - |u| : 0 with
// dp = n.(a, b) and u = n x (a, b) (n the unit gradient).
template <int M, int J, int TY, int FP>
__device__ __forceinline__ void rgc_core(const float* hgf, const float4* tb4, int ty, int py,
                                         int lane, float (&acc)[FP][M]) {
  using G = Geo<M, J, TY, FP>;
  const int cpy = (2 * py + 1) / M;
#pragma unroll
  for (int fr = 0; fr < FP; ++fr)
#pragma unroll
    for (int px = 0; px < M; ++px) acc[fr][px] = 0.f;
  if constexpr (FP == 1) {
    const float2* hg = reinterpret_cast<const float2*>(hgf);
#pragma unroll
    for (int jj = 0; jj < G::W2; ++jj) {
      const int kyl = 2 * ty + cpy + jj;
      const float2* r0 = hg + (kyl * 2 + 0) * G::HGP + lane;
      const float2* r1 = hg + (kyl * 2 + 1) * G::HGP + lane;
      float2 sv[G::NQ];
#pragma unroll
      for (int q = 0; q < G::NQ; ++q) sv[q] = (q & 1) ? r1[q >> 1] : r0[q >> 1];
      const float4* tb = tb4 + (size_t)(py * G::W2 + jj) * G::TBLK;
#pragma unroll
      for (int s4 = 0; s4 < G::NS4; ++s4) {
        const float4 A = tb[s4];
        const float4 B = tb[G::NS4 + s4];
        const float4 Wv = tb[2 * G::NS4 + s4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int sidx = s4 * 4 + e;
          if (sidx < G::NS) {
            const int px = sidx / G::W2;
            const int ii = sidx % G::W2;
            const int cpx = (2 * px + 1) / M;
            const float2 gv = sv[cpx + ii];
            const float a = f4c(A, e), bb = f4c(B, e), w = f4c(Wv, e);
            const float dp = fmaf(gv.x, a, gv.y * bb);
            const float u = fmaf(gv.y, a, -(gv.x * bb));
            const float v = w - fabsf(u);
            acc[0][px] = (dp < 0.f) ? acc[0][px] + v : acc[0][px];
          }
        }
      }
    }
  } else {
    // frame pair in one register pair: gx = (gx0, gx1), gy = (gy0, gy1); every
    // FMA-pipe operation is packed: v = w + (-|u|), acc += [dp < 0] * v
    // (measured 6 % faster than scalar v and predicated scalar adds)
    const float4* hg = reinterpret_cast<const float4*>(hgf);
    constexpr int NPR = FP / 2;  // frame pairs per pass (share every table load)
    float2 acc2[NPR][M];
#pragma unroll
    for (int pp = 0; pp < NPR; ++pp)
#pragma unroll
      for (int px = 0; px < M; ++px) acc2[pp][px] = make_float2(0.f, 0.f);
    // window rows stay a loop: unrolled, the core's code outgrows the
    // instruction cache (measured 2 % slower and with register spills)
#pragma unroll 1
    for (int jj = 0; jj < G::W2; ++jj) {
      const int kyl = 2 * ty + cpy + jj;
      const float4* r0 = hg + (kyl * 2 + 0) * G::HGP + lane;
      const float4* r1 = hg + (kyl * 2 + 1) * G::HGP + lane;
      const float4* tb = tb4 + (size_t)(py * G::W2 + jj) * G::TBLK;
      // gradient-major order: one half-grid sample at a time, applied to every
      // output phase px whose window holds it (fewer live registers than
      // loading the row first; measured 1.3 % faster)
#pragma unroll
      for (int q = 0; q < G::NQ; ++q) {
        float4 g[NPR];
#pragma unroll
        for (int pp = 0; pp < NPR; ++pp)
          g[pp] = (q & 1) ? r1[pp * G::HG_PLANE + (q >> 1)] : r0[pp * G::HG_PLANE + (q >> 1)];
#pragma unroll
        for (int px = 0; px < M; ++px) {
          const int ii = q - (2 * px + 1) / M;
          if (ii < 0 || ii >= G::W2) continue;
          const int sidx = px * G::W2 + ii;
          const float4 T = tb[sidx];
          const float w = T.w;
          const int dxn = dx_num<M, J>(px, ii);  // compile-time after unrolling
          if (dxn != 0) {
            // dp = a (gx + gy rho) and u = a (gy - gx rho), rho = b / a: the
            // sign of a is the sign of dx, a constant of (px, ii), so
            // [dp < 0] is a comparison of t1 = gx + gy rho in a fixed
            // direction, and w - |u| = w + (-|a|) |t2|, t2 = gy - gx rho:
            // 4 packed FMA-pipe operations per sample pair instead of 6
            const float2 rho = make_float2(T.x, T.x), nrho = make_float2(T.y, T.y);
            const float2 nab = make_float2(T.z, T.z);
#pragma unroll
            for (int pp = 0; pp < NPR; ++pp) {
              const float2 gx = make_float2(g[pp].x, g[pp].y), gy = make_float2(g[pp].z, g[pp].w);
              const float2 t1 = __ffma2_rn(gy, rho, gx);
              const float2 t2 = __ffma2_rn(gx, nrho, gy);
              const float2 at2 = make_float2(fabsf(t2.x), fabsf(t2.y));
              const float2 v = __ffma2_rn(nab, at2, make_float2(w, w));
              const float2 msk =
                  dxn > 0 ? make_float2(t1.x < 0.f ? 1.f : 0.f, t1.y < 0.f ? 1.f : 0.f)
                          : make_float2(t1.x > 0.f ? 1.f : 0.f, t1.y > 0.f ? 1.f : 0.f);
              acc2[pp][px] = __ffma2_rn(msk, v, acc2[pp][px]);
            }
          } else {
            // dx = 0: dp = gy b, u = -gx b
            const float2 a = make_float2(T.x, T.x), b = make_float2(T.y, T.y);
            const float2 nb = make_float2(T.z, T.z);
#pragma unroll
            for (int pp = 0; pp < NPR; ++pp) {
              const float2 gx = make_float2(g[pp].x, g[pp].y), gy = make_float2(g[pp].z, g[pp].w);
              const float2 dp = __ffma2_rn(gx, a, __fmul2_rn(gy, b));
              const float2 u = __ffma2_rn(gy, a, __fmul2_rn(gx, nb));
              const float2 nu = make_float2(__int_as_float(__float_as_int(u.x) | 0x80000000),
                                            __int_as_float(__float_as_int(u.y) | 0x80000000));
              const float2 v = __fadd2_rn(make_float2(w, w), nu);
              const float2 msk = make_float2(dp.x < 0.f ? 1.f : 0.f, dp.y < 0.f ? 1.f : 0.f);
              acc2[pp][px] = __ffma2_rn(msk, v, acc2[pp][px]);
            }
          }
        }
      }
    }
#pragma unroll
    for (int pp = 0; pp < NPR; ++pp)
#pragma unroll
      for (int px = 0; px < M; ++px) {
        acc[2 * pp][px] = acc2[pp][px].x;
        acc[2 * pp + 1][px] = acc2[pp][px].y;
      }
  }
}

template <int M, int J, int TY, int FP, int MODE, int NP>
__global__ void __launch_bounds__(32 * TY * M + NP, EsrrfTile<M>::MIN_BLOCKS)
    esrrf_fused_kernel(const __grid_constant__ TmapPack maps, const UnitTable ut) {
  using G = Geo<M, J, TY, FP, NP>;
  extern __shared__ __align__(128) float sm[];
  __shared__ FusedParams sp;
  __shared__ int s_unit;
  __shared__ int s_abort;
  float4* tb4 = reinterpret_cast<float4*>(sm + G::O_TB);
  float* rw = sm + G::O_RW;
  float* cw = sm + G::O_CW;
  float* tw = sm + G::O_TW;  // tw[px * NTC + tid]
  float* tk = sm + G::O_TK;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + G::o_bar(MODE, ut.ns_cap));
  uint64_t* full = bars;                    // [NSLOT] slot prepared (NP arrivals)
  uint64_t* empty = bars + G::NSLOT;        // [NSLOT] slot released (NTC arrivals)
  uint64_t* pbar = bars + 2 * G::NSLOT;     // producer-group barrier (NP arrivals)
  uint64_t* tbar = bars + 2 * G::NSLOT + 1; // [2 FP] TMA input tiles

  const int tid = threadIdx.x;
  const bool producer = tid >= G::NTC;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int ty = warp % TY;  // consumers
  const int py = warp / TY;
  Producer<M, J, TY, FP, NP> prod{sm + G::O_INB, sm + G::O_G, sm + G::O_T1, sm + G::O_HG,
                              sm + G::O_RI, rw, tid - G::NTC};

  if (tid == 0) {
    for (int k = 0; k < G::NSLOT; ++k) {
      mbar_init(&full[k], G::NP);
      mbar_init(&empty[k], G::NTC);
    }
    mbar_init(pbar, G::NP);
    for (int k = 0; k < 2 * FP; ++k) mbar_init(&tbar[k], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();
  unsigned gp = 0;      // frame passes since launch: slot gp % NSLOT, use gp / NSLOT (all threads)
  unsigned tphase = 0;  // producers: bit k = parity of the next completion of tbar[k]
  unsigned tpend = 0;   // producers: bit k = a TMA load into input buffer k is in flight
  unsigned pphase = 0;  // producers: parity of the next completion of pbar
  int cur_item = -1;

  for (int iter = 0;; ++iter) {
  int unit;
  if (ut.counter) {
    if (tid == 0) s_unit = (int)atomicAdd(ut.counter, 1u);
    __syncthreads();
    unit = s_unit;
  } else {
    unit = blockIdx.x + iter * gridDim.x;
  }
  if (unit >= ut.total_units) break;
  int item = 0;
  if (ut.items) {
    int lo = 0, hi = ut.n_items - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(ut.unit_start + mid) <= unit) lo = mid;
      else hi = mid - 1;
    }
    item = lo;
  }
  if (item != cur_item) {
    if (tid == 0) sp = ut.items ? ut.items[item] : ut.single;
    __syncthreads();
    if constexpr (FP == 1) {
      const float4* src = reinterpret_cast<const float4*>(sp.tbl);
      for (int i = tid; i < M * G::W2 * 3 * G::NS4; i += G::NT) tb4[i] = src[i];
    } else {
      // plan layout [py][jj]{a, b, w}[NS4 * 4] -> one float4 per sample:
      //   dx != 0: (rho, -rho, -|a|, w) with rho = b / a (see rgc_core);
      //   dx == 0: (a, b, -b, w) (a = 0);  outside the window: zeros
      constexpr int N4 = G::NS4 * 4;
      const float* src = sp.tbl;
      for (int i = tid; i < M * G::W2 * N4; i += G::NT) {
        const int blk = i / N4, s = i % N4;
        const float a = src[(blk * 3 + 0) * N4 + s];
        const float b = src[(blk * 3 + 1) * N4 + s];
        const float w = src[(blk * 3 + 2) * N4 + s];
        const int px = s / G::W2, ii = s % G::W2;
        float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
        if (s < G::NS && w != 0.f) {
          if (dx_num<M, J>(px, ii) == 0) {
            e = make_float4(a, b, -b, w);
          } else if (a != 0.f) {
            const float rho = __fdiv_rn(b, a);
            e = make_float4(rho, -rho, -fabsf(a), w);
          }
        }
        tb4[blk * G::TBLK + s] = e;
      }
    }
    cur_item = item;
  }
  const FusedParams& p = sp;
  const unsigned long long lim = p.wait_ns ? p.wait_ns : kWaitLimitNs;
  const int local = unit - (ut.items ? __ldg(ut.unit_start + item) : 0);
  const int tiles = p.tiles_x * p.tiles_y;
  const int tile = local % tiles;
  const int tp = (local / tiles) / p.chunks;
  const int chunk = (local / tiles) % p.chunks;

  // frames of this unit
  const int tp_f0 = tp * p.fpt;
  const int tp_nf = min(p.fpt, p.T - tp_f0);
  const int nch = min(p.chunks, tp_nf);
  int npass = 0;
  if (chunk < nch) {  // uniform across the CTA
  UnitGeo u;
  u.nx0 = (tile % p.tiles_x) * G::TX;
  u.ny0 = (tile / p.tiles_x) * TY;
  u.H = p.H;
  u.W = p.W;
  u.f0 = tp_f0 + (int)((long long)chunk * tp_nf / nch);
  u.f1 = tp_f0 + (int)((long long)(chunk + 1) * tp_nf / nch);
  u.kb_y = 2 * u.ny0 - J;
  u.kb_x = 2 * u.nx0 - J;
  u.RY0 = u.ny0 - G::RLO;
  u.CX0 = u.nx0 - G::CLO;
  u.y_start = u.ny0 - G::IY;
  u.x_start = u.nx0 - G::IX;
  u.kmax_y = 2 * p.rowsM - 2;
  u.kmax_x = 2 * p.colsM - 2;
  const int f0 = u.f0, f1 = u.f1;
  npass = (f1 - f0 + FP - 1) / FP;

  // ---- per-CTA constants: intensity interpolation weights -----------------
  for (int i = tid; i < G::OY; i += G::NT) {
    const int yM = u.ny0 * M + i;
    const int nyp = u.ny0 + i / M;
    const float ry = __fdiv_rn((float)yM, (float)M);
    const int rb = (int)floorf(ry - 0.5f);
    float w5[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int nb = rb - 1 + t;
      const int k = nb - (nyp - 2);
      const float w = cr_cubic(ry - ((float)nb + 0.5f));
#pragma unroll
      for (int kk = 0; kk < 5; ++kk) w5[kk] = (k == kk) ? w : w5[kk];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) rw[i * 5 + k] = w5[k];
  }
  for (int i = tid; i < G::OX; i += G::NT) {
    const int xM = u.nx0 * M + i;
    const int nxp = u.nx0 + i / M;
    const float rx = __fdiv_rn((float)xM, (float)M);
    const int cb = (int)floorf(rx - 0.5f);
    float w5[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int nb = cb - 1 + t;
      const int k = nb - (nxp - 2);
      const float w = cr_cubic(rx - ((float)nb + 0.5f));
#pragma unroll
      for (int kk = 0; kk < 5; ++kk) w5[kk] = (k == kk) ? w : w5[kk];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) cw[i * 5 + k] = w5[k];
  }

  // ---- consumer constants --------------------------------------------------
  const int ny = u.ny0 + ty;
  const int nx = u.nx0 + lane;
  const int yM = ny * M + py;
  unsigned omask = 0;  // bit px: output forced to 0 / not written; bit 31: outside the image
  if (!producer) {
    const int cpy = (2 * py + 1) / M;
    const int ky_lo = 2 * ny + cpy - J, ky_hi = 2 * ny + cpy + J;
    const bool by = (ky_lo < 1) || (ky_hi > u.kmax_y);
#pragma unroll
    for (int px = 0; px < M; ++px) {
      const int cpx = (2 * px + 1) / M;
      const int xM = nx * M + px;
      const int kx_lo = 2 * nx + cpx - J, kx_hi = 2 * nx + cpx + J;
      float iw = p.inv_wsum[py * M + px];
      if (by || kx_lo < 1 || kx_hi > u.kmax_x) {
        // window reaches invalid half-grid samples: they count in neither sum
        const float* wf = p.wfull + (size_t)(py * M + px) * G::W2 * G::W2;
        float s = 0.f;
        for (int jj = 0; jj < G::W2; ++jj) {
          const int ky = ky_lo + jj;
          if (ky < 1 || ky > u.kmax_y) continue;
          for (int ii = 0; ii < G::W2; ++ii) {
            const int kx = kx_lo + ii;
            if (kx < 1 || kx > u.kmax_x) continue;
            s += wf[jj * G::W2 + ii];
          }
        }
        iw = s > 0.f ? 1.f / s : 0.f;
      }
      tw[px * G::NTC + tid] = iw;
      const bool outside = (ny >= u.H) || (nx >= u.W);
      const bool in_margin = (yM < p.margin) || (yM >= p.rowsM - p.margin) ||
                             (xM < p.margin) || (xM >= p.colsM - p.margin);
      if (outside) omask |= (1u << px) | (1u << 31);
      else if (in_margin) omask |= (1u << px);
    }
  }
  __syncthreads();

  if (producer) {
    // ======================= producer warpgroup =============================
    constexpr unsigned kTileBytes = unsigned(G::BH * G::BW * 4);
    const bool use_tma = p.tmap >= 0;
    const CUtensorMap* tmap = use_tma ? &maps.m[p.tmap] : nullptr;
    const bool leader = prod.ptid == 0;
    if (use_tma && leader) {
      // input buffer k = set * FP + fr holds frame f0 + k for the first two sets
      fence_proxy_async_smem();
      for (int k = 0; k < 2 * FP; ++k) {
        if (f0 + k < f1) {
          mbar_arrive_expect_tx(&tbar[k], kTileBytes);
          tma_load_3d(prod.inb + k * G::S_INB, tmap, &tbar[k], u.x_start, u.y_start, f0 + k);
          tpend |= 1u << k;
        }
      }
    }
    for (int j = 0; j < npass; ++j) {
      const unsigned g = gp + j;
      const int s = (int)(g % G::NSLOT);
      const unsigned use = g / G::NSLOT;
      const int fa = f0 + j * FP;
      const int set = j & 1;
      const int nf = min(FP, f1 - fa);
      const float* tin[FP];
#pragma unroll
      for (int fr = 0; fr < FP; ++fr)
        tin[fr] = prod.inb + (set * FP + (fr < nf ? fr : 0)) * G::S_INB;
      // slot s is free once the consumers released its previous use
      bool ok = use == 0 || mbar_wait_or_abort(&empty[s], (use - 1) & 1u, &s_abort, lim);
      if (ok && use_tma) {
#pragma unroll
        for (int fr = 0; fr < FP; ++fr) {
          const int k = set * FP + fr;
          if (fr < nf && ok) {
            ok = mbar_wait_or_abort(&tbar[k], (tphase >> k) & 1u, &s_abort, lim);
            if (ok) {
              tphase ^= 1u << k;
              tpend &= ~(1u << k);
            }
          }
        }
      } else if (ok) {
        for (int fr = 0; fr < nf; ++fr) {
          const float* src = p.in + (size_t)(fa + fr) * u.H * u.W;
          float* dst = prod.inb + (set * FP + fr) * G::S_INB;
          for (int i = prod.ptid; i < G::BH * G::BW; i += G::NP) {
            const int r = u.y_start + i / G::BW;
            const int c = u.x_start + i % G::BW;
            dst[i] = (r >= 0 && r < u.H && c >= 0 && c < u.W) ? __ldg(src + (size_t)r * u.W + c)
                                                               : 0.f;
          }
        }
        mbar_arrive(pbar);
        ok = mbar_wait_or_abort(pbar, pphase & 1u, &s_abort, lim);
        pphase ^= 1u;
      }
      if (!ok) {
        *(volatile int*)&s_abort = 1;
        break;
      }
      prod.roberts_and_rows(p, u, tin, s);
      mbar_arrive(pbar);
      ok = mbar_wait_or_abort(pbar, pphase & 1u, &s_abort, lim);
      pphase ^= 1u;
      if (!ok) {
        *(volatile int*)&s_abort = 1;
        break;
      }
      if (use_tma && leader) {
        // this set's input buffers are free: fetch the frames two passes ahead
        fence_proxy_async_smem();
#pragma unroll
        for (int fr = 0; fr < FP; ++fr) {
          const int fn = fa + 2 * FP + fr;
          const int k = set * FP + fr;
          if (fn < f1) {
            mbar_arrive_expect_tx(&tbar[k], kTileBytes);
            tma_load_3d(prod.inb + k * G::S_INB, tmap, &tbar[k], u.x_start, u.y_start, fn);
            tpend |= 1u << k;
          }
        }
      }
      prod.column_pass(p, u);
      mbar_arrive(pbar);
      ok = mbar_wait_or_abort(pbar, pphase & 1u, &s_abort, lim);
      pphase ^= 1u;
      if (!ok) {
        *(volatile int*)&s_abort = 1;
        break;
      }
      prod.row_pass(p, u, s);
      if (!(p.test_withhold_full && iter == 0 && j == 0)) mbar_arrive(&full[s]);
    }
  } else {
    // ======================= consumers ======================================
    const size_t plane = (size_t)p.rowsM * p.colsM;
    for (int j = 0; j < npass; ++j) {
      const unsigned g = gp + j;
      const int s = (int)(g % G::NSLOT);
      const unsigned use = g / G::NSLOT;
      const int fa = f0 + j * FP;
      const int nf = min(FP, f1 - fa);
      if (!mbar_wait_or_abort(&full[s], use & 1u, &s_abort, lim)) {
        *(volatile int*)&s_abort = 1;
        break;
      }
      float acc[FP][M];
      rgc_core<M, J, TY, FP>(sm + G::O_HG + s * G::S_HG, tb4, ty, py, lane, acc);

      // ---- normalise, ^sensitivity, intensity, margin, temporal ------------
      // magnified intensity of this thread's outputs: column pass of the
      // Catmull-Rom interpolation from the row-pass values (5 taps per output)
      const float* ri = sm + G::O_RI + s * FP * G::S_RI;
      float rv[FP][5];
      if (p.iw) {
#pragma unroll
        for (int fr = 0; fr < FP; ++fr)
#pragma unroll
          for (int k = 0; k < 5; ++k) rv[fr][k] = ri[fr * G::S_RI + (ty * M + py) * G::RIW + lane + k];
      }
      mbar_arrive(&empty[s]);  // slot s fully read
      const bool first = (fa == f0);
      // frame fa + fr is frame k = fa - f0 + fr of this unit's series; 1 / (k + 1)
      // by the fast reciprocal (the increment it scales is a deviation-sized term,
      // so its ~1 ulp error does not show; the IEEE reciprocal cost 2 % of the kernel)
      float inv_n[FP];
#pragma unroll
      for (int fr = 0; fr < FP; ++fr) inv_n[fr] = __fdividef(1.0f, (float)(fa - f0 + fr + 1));
#pragma unroll
      for (int px = 0; px < M; ++px) {
        const float twv = tw[px * G::NTC + tid];
        const bool zero = (omask & (1u << px)) != 0;
        float base[FP], ival[FP];
#pragma unroll
        for (int fr = 0; fr < FP; ++fr) {
          base[fr] = acc[fr][px] * twv;
          base[fr] = (base[fr] < 0.f) ? 0.f : base[fr];
          ival[fr] = 1.f;
        }
        if (p.iw) {
          float w5[5];
#pragma unroll
          for (int k = 0; k < 5; ++k) w5[k] = cw[(lane * M + px) * 5 + k];
          if constexpr (FP >= 2) {
#pragma unroll
            for (int pp = 0; pp < FP / 2; ++pp) {
              float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
              for (int k = 0; k < 5; ++k)
                s2 = __ffma2_rn(make_float2(w5[k], w5[k]),
                                make_float2(rv[2 * pp][k], rv[2 * pp + 1][k]), s2);
              ival[2 * pp] = s2.x;
              ival[2 * pp + 1] = s2.y;
            }
          } else {
            float s1 = 0.f;
#pragma unroll
            for (int k = 0; k < 5; ++k) s1 = fmaf(w5[k], rv[0][k], s1);
            ival[0] = s1;
          }
        }
        if (MODE == kModeSum) {
          // unrolled over the sensitivity slots (a runtime-bounded loop here
          // made the compiler re-materialise addresses in the RGC core: +14 %
          // instructions); running mean per sensitivity (Welford)
#pragma unroll
          for (int k = 0; k < kMaxSens; ++k) {
            if (k >= p.n_sens) break;
            float* ks = tk + (k * M + px) * G::NTC + tid;
            float mu = first ? 0.f : *ks;
#pragma unroll
            for (int fr = 0; fr < FP; ++fr) {
              if (fr < nf) {
                float r = apply_sens(base[fr], p.sens_mode_k[k], p.sens_int_k[k], p.sens_k[k]);
                r = zero ? 0.f : r * ival[fr];
                mu = (first && fr == 0) ? r : fmaf(r - mu, inv_n[fr], mu);
              }
            }
            *ks = mu;
          }
        } else if (MODE == kModeStack) {
#pragma unroll
          for (int fr = 0; fr < FP; ++fr) {
            if (fr < nf) {
              float r = apply_sens(base[fr], p.sens_mode_k[0], p.sens_int_k[0], p.sens_k[0]);
              r = zero ? 0.f : r * ival[fr];
              if (!(omask >> 31))
                p.out[(size_t)(fa + fr) * plane + (size_t)yM * p.colsM + (size_t)nx * M + px] = r;
            }
          }
        } else {
          float4* st = reinterpret_cast<float4*>(tk) + px * G::NTC + tid;
          float* stl = tk + 4 * M * G::NTC + px * G::NTC + tid;
          Moments mo{0.f, 0.f, 0.f, 0.f, 0.f};
          if (!first) {
            const float4 t = *st;
            mo = Moments{t.x, t.y, t.z, t.w, *stl};
          }
#pragma unroll
          for (int fr = 0; fr < FP; ++fr) {
            if (fr < nf) {
              float r = apply_sens(base[fr], p.sens_mode_k[0], p.sens_int_k[0], p.sens_k[0]);
              r = zero ? 0.f : r * ival[fr];
              if (first && fr == 0) mo = moments_start(r);
              else moments_push(mo, r, inv_n[fr]);
            }
          }
          *st = make_float4(mo.mean, mo.m2, mo.c, mo.a);
          *stl = mo.b;
        }
      }
    }
  }
  if (!producer && s_abort == 0 && MODE != kModeStack && !(omask >> 31)) {
    const size_t plane = (size_t)p.rowsM * p.colsM;
    float* rec = p.out + (size_t)(tp * p.chunks + chunk) * p.F * plane +
                 (size_t)yM * p.colsM + (size_t)nx * M;
    if (MODE == kModeSum) {
      for (int k = 0; k < p.n_sens; ++k) {
#pragma unroll
        for (int px = 0; px < M; ++px) rec[k * plane + px] = tk[(k * M + px) * G::NTC + tid];
      }
    } else {
#pragma unroll
      for (int px = 0; px < M; ++px) {
        const float4 t = reinterpret_cast<const float4*>(tk)[px * G::NTC + tid];
        rec[px] = t.x;
        rec[plane + px] = t.y;
        rec[2 * plane + px] = t.z;
        rec[3 * plane + px] = t.w;
        rec[4 * plane + px] = tk[4 * M * G::NTC + px * G::NTC + tid];
      }
    }
  }
  }  // chunk < nch
  __syncthreads();  // the unit's shared state is free for the next unit
  if (s_abort) {
    // a wait ran out: the producer leader waits (bounded) for its TMA copies
    // still in flight, then every thread leaves without writing more
    if (producer && prod.ptid == 0 && p.status) atomicOr(p.status, kDevTmaTimeout);
    if (producer && prod.ptid == 0) {
      for (int k = 0; k < 2 * FP; ++k)
        if (tpend & (1u << k)) (void)mbar_wait_bounded(&tbar[k], (tphase >> k) & 1u);
    }
    return;
  }
  gp += npass;
  }  // unit loop
}

template <int M, int J, int MODE, int V = 0>
size_t fused_smem_bytes(int ns_cap) {
  return FusedCfg<M, J, MODE, V>::G::smem_bytes(MODE, ns_cap);
}

template <int M, int J, int MODE, int V = 0>
cudaError_t launch_fused(const UnitTable& ut, const TmapPack& maps, int grid,
                         cudaStream_t stream) {
  using C = FusedCfg<M, J, MODE, V>;
  using G = typename C::G;
  auto kern = esrrf_fused_kernel<M, J, C::TY, C::FP, MODE, C::NP>;
  const size_t smem = G::smem_bytes(MODE, MODE == kModeSum ? ut.ns_cap : 1);
  if (smem > kSmemBudget) return cudaErrorInvalidValue;
  static int attr_done = -1;  // device the attributes were last set for
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (attr_done != dev) {
    const size_t cap = std::min(kSmemBudget, G::smem_bytes(MODE, C::NSC));
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    attr_done = dev;
  }
  if (grid < 1) return cudaSuccess;
  kern<<<grid, G::NT, smem, stream>>>(maps, ut);
  return cudaGetLastError();
}

// resident CTAs per SM of one instantiation (for persistent grids)
template <int M, int J, int MODE, int V = 0>
int fused_occupancy(int ns_cap) {
  using C = FusedCfg<M, J, MODE, V>;
  using G = typename C::G;
  auto kern = esrrf_fused_kernel<M, J, C::TY, C::FP, MODE, C::NP>;
  const size_t smem = G::smem_bytes(MODE, MODE == kModeSum ? ns_cap : 1);
  if (smem > kSmemBudget) return 0;
  // cached per device and sensitivity count (queried once; launches ask per call)
  static int cache[16][kMaxSens + 1] = {};
  int dev = 0;
  const bool cacheable = cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 16 &&
                         ns_cap >= 0 && ns_cap <= kMaxSens;
  if (cacheable && cache[dev][ns_cap] > 0) return cache[dev][ns_cap];
  int n = 0;
  const size_t cap = std::min(kSmemBudget, G::smem_bytes(MODE, C::NSC));
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap) !=
      cudaSuccess)
    return 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, G::NT, smem) != cudaSuccess)
    return 1;
  n = n > 0 ? n : 1;
  if (cacheable) cache[dev][ns_cap] = n;
  return n;
}

// geometry the host needs to build the tensor map for a given (M, J); the
// tile shape does not depend on the mode or on FP
struct FusedGeometry {
  int TY, IX, IY, BW, BH;
};

template <int M, int J, int V = 0>
FusedGeometry fused_geometry() {
  using G = Geo<M, J, EsrrfTile<M, V>::TY, 1>;
  return FusedGeometry{EsrrfTile<M, V>::TY, G::IX, G::IY, G::BW, G::BH};
}

}  // namespace nx
