// C-ABI of the eSRRF / SRRF engine: plans, workspace sizing, dispatch.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "nanopyx_gb300.h"

namespace nx {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* what) {
  set_error("%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? NX_ERR_OUT_OF_MEMORY : NX_ERR_CUDA;
}

static int invalid(const char* msg) {
  set_error("%s", msg);
  return NX_ERR_INVALID_ARG;
}

// ---------------------------------------------------------------------------
// fused-kernel registry
// ---------------------------------------------------------------------------
const FusedEntry* fused_entry(int M, int J, int variant) {
  if (variant == 1) {
    switch (M) {
      case 2: return fused_entry_m2_alt(J);
      case 4: return fused_entry_m4_alt(J);
      case 5: return fused_entry_m5_alt(J);
      default: return nullptr;
    }
  }
  if (variant != 0) return nullptr;
  switch (M) {
    case 1: return fused_entry_m1(J);
    case 2: return fused_entry_m2(J);
    case 3: return fused_entry_m3(J);
    case 4: return fused_entry_m4(J);
    case 5: return fused_entry_m5(J);
    case 6: return fused_entry_m6(J);
    case 8: return fused_entry_m8(J);
    default: return nullptr;
  }
}

// ---------------------------------------------------------------------------
// TMA descriptor encoding through the driver entry point (no libcuda link)
// ---------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// 3-D (W, H, T) float32 map with a (BW, BH, 1) box, zero fill out of bounds.
static bool make_frame_tmap(CUtensorMap* map, const float* base, int T, int H, int W, int BW,
                            int BH) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false;
  if (((size_t)W * 4) % 16 != 0) return false;
  if (BW > 256 || BH > 256 || (BW * 4) % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)T};
  const cuuint64_t strides[2] = {(cuuint64_t)W * 4, (cuuint64_t)W * H * 4};
  const cuuint32_t box[3] = {(cuuint32_t)BW, (cuuint32_t)BH, 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

static int g_force_no_tma = -1;
static bool tma_disabled() {
  if (g_force_no_tma < 0) {
    const char* e = getenv("NANOPYX_GB300_NO_TMA");
    g_force_no_tma = (e && *e && *e != '0') ? 1 : 0;
  }
  return g_force_no_tma == 1;
}

static int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
  return sms > 0 ? sms : 148;
}

}  // namespace nx

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------
struct nx_esrrf_plan {
  int H, W, M;
  float radius, sensitivity;
  int iw;
  int rowsM, colsM;
  int JW;           // half-width of the (symmetric) window used by the fused kernel
  nx::RgcScalars sc;
  const nx::FusedEntry* fused;
  int tile_variant;  // which instantiation `fused` is (0: default tiling)
  int cy_base, cx_base;
  float cy[4], cx[4];
  int device;
  float* d_tbl;     // device: [tbl | inv_wsum | wfull]
  size_t n_tbl, n_inv, n_wfull;
};

namespace nx {

// Catmull-Rom taps (double, as _c_cubic) of the 2m-grid index 2*m*n-1 along an
// axis of n input pixels: the position the reference RGC clamps to.
static void clamp_taps(int n, int M, int* base, float w[4]) {
  const float mag = (float)(2 * M);
  const float r = (float)(2 * M * n - 1) / mag;  // float division, as ShiftAndMagnify
  const int r_int = (int)std::floor((float)((double)r - 0.5));
  *base = r_int - 1;
  for (int t = 0; t < 4; ++t) {
    const int nb = r_int - 1 + t;
    double v = std::fabs((double)r - ((double)nb + 0.5));
    double z = 0.0;
    if (v < 1) z = v * v * (v * (-0.5 + 2) + (0.5 - 3)) + 1;
    else if (v < 2) z = -0.5 * v * v * v + 5 * 0.5 * v * v - 8 * 0.5 * v + 4 * 0.5;
    w[t] = (nb >= 0 && nb < n) ? (float)z : 0.f;
  }
}

// Phase tables of the RGC sample weights (FP64, rounded once to float).
//   per output sub-pixel phase (py, px) and window offset (j, i):
//   dx, dy: offset of the half-grid sample from the output centre,
//   d = |(dx, dy)|, w = (d exp(-d^2 / tSS))^4 if 0 < d <= tSO, else 0,
//   a = dx * w / d, b = dy * w / d.
static void build_tables(nx_esrrf_plan* p, std::vector<float>& tbl, std::vector<float>& inv,
                         std::vector<float>& wfull) {
  const int M = p->M;
  const int JW = p->JW;
  const int W2 = 2 * JW + 1;
  const int NS = M * W2;
  const int NS4 = (NS + 3) / 4;
  tbl.assign((size_t)M * W2 * 3 * NS4 * 4, 0.f);
  inv.assign((size_t)M * M, 0.f);
  wfull.assign((size_t)M * M * W2 * W2, 0.f);
  const double tSS = p->sc.tSS;
  std::vector<double> wsum((size_t)M * M, 0.0);
  for (int py = 0; py < M; ++py) {
    const int cpy = (2 * py + 1) / M;
    for (int jj = 0; jj < W2; ++jj) {
      const int j = jj - JW;
      const double dy = (cpy + j) / 2.0 - (py + 0.5) / M;
      float* blk = tbl.data() + (size_t)(py * W2 + jj) * 3 * NS4 * 4;
      for (int px = 0; px < M; ++px) {
        const int cpx = (2 * px + 1) / M;
        for (int ii = 0; ii < W2; ++ii) {
          const int i = ii - JW;
          const double dx = (cpx + i) / 2.0 - (px + 0.5) / M;
          const float d = (float)std::sqrt(dx * dx + dy * dy);
          const bool in_win = j >= p->sc.start && j < p->sc.end && i >= p->sc.start &&
                              i < p->sc.end;
          float w = 0.f, a = 0.f, b = 0.f;
          if (in_win && d != 0.f && d <= p->sc.tSO) {
            const double dd = d;
            const double e = dd * std::exp(-(dd * dd) / tSS);
            w = (float)(e * e * e * e);
            const double wd = (double)w / dd;
            a = (float)(dx * wd);
            b = (float)(dy * wd);
          }
          const int sidx = px * W2 + ii;
          blk[0 * NS4 * 4 + sidx] = a;
          blk[1 * NS4 * 4 + sidx] = b;
          blk[2 * NS4 * 4 + sidx] = w;
          wfull[((size_t)(py * M + px) * W2 + jj) * W2 + ii] = w;
          wsum[py * M + px] += (double)w;
        }
      }
    }
  }
  for (int k = 0; k < M * M; ++k) inv[k] = wsum[k] > 0 ? (float)(1.0 / (double)(float)wsum[k]) : 0.f;
}

static int check_plan(const nx_esrrf_plan* p) {
  if (!p) return invalid("plan is NULL");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->device) {
    set_error("plan was created on device %d but device %d is current", p->device, dev);
    return NX_ERR_INVALID_ARG;
  }
  return NX_OK;
}

// chunking of each timepoint's frames across CTAs (deterministic in its inputs)
// Frame chunks per timepoint of a launch over `tiles` x `n_tp` units.  The
// resident CTAs stride over (tile, timepoint, chunk) units, so a CTA runs
// about ceil(units / resident) units, each costing its frame passes plus a
// start-up of ~0.65 pass (the unit's first pass is not overlapped with the
// producer warps' preparation).  The chunk count with the smallest estimate
// wins: few chunks for large stacks, enough to fill every SM for small ones,
// and >= 4 frames per chunk.
static int best_chunks(long long tiles, int n_tp, int fpt, int min_nf, long long resident) {
  int best = 1;
  double best_cost = 1e300;
  const int cmax = std::max(1, std::min(min_nf / 4, 64));
  for (int c = 1; c <= cmax; ++c) {
    const long long units = tiles * n_tp * c;
    const double per_cta = (double)((units + resident - 1) / resident);
    const double passes = std::ceil((double)fpt / c / 2.0);
    const double cost = per_cta * (passes + 0.65);
    if (cost < best_cost * 0.999) {
      best_cost = cost;
      best = c;
    }
  }
  return best;
}

static int plan_chunks(const nx_esrrf_plan* p, int T, int fpt, int n_tp) {
  if (!p->fused) return 1;
  const int TY = p->fused->geo.TY;
  const long long tiles = (long long)((p->W + 31) / 32) * ((p->H + TY - 1) / TY);
  const int min_nf = std::min(fpt, T - (n_tp - 1) * fpt);
  const long long resident =
      (long long)std::max(1, p->fused->occupancy[kModeFull](1)) * device_sms();
  return best_chunks(tiles, n_tp, fpt, min_nf, resident);
}

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

static const size_t kStatusBytes = 256;

static int corr_count(int mask) {
  return ((mask & NX_CORR_AVG) ? 1 : 0) + ((mask & NX_CORR_VAR) ? 1 : 0) +
         ((mask & NX_CORR_TAC2) ? 1 : 0);
}

static int fields_for(int corr_mask) {
  return (corr_mask & (NX_CORR_VAR | NX_CORR_TAC2)) ? 5 : 1;
}

static void fill_params(const nx_esrrf_plan* p, FusedParams& fp, const float* in, int T, int fpt,
                        int n_tp, int chunks, float* out, unsigned* status) {
  memset(&fp, 0, sizeof(fp));
  fp.in = in;
  fp.T = T;
  fp.H = p->H;
  fp.W = p->W;
  fp.rowsM = p->rowsM;
  fp.colsM = p->colsM;
  fp.tiles_x = (p->W + 31) / 32;
  fp.tiles_y = (p->H + p->fused->geo.TY - 1) / p->fused->geo.TY;
  fp.fpt = fpt;
  fp.n_tp = n_tp;
  fp.chunks = chunks;
  fp.margin = p->sc.margin;
  fp.iw = p->iw;
  fp.n_sens = 1;
  fp.sens_mode_k[0] = p->sc.sens_mode;
  fp.sens_int_k[0] = p->sc.sens_int;
  fp.sens_k[0] = p->sc.sens;
  fp.cy_base = p->cy_base;
  fp.cx_base = p->cx_base;
  for (int t = 0; t < 4; ++t) {
    fp.cy[t] = p->cy[t];
    fp.cx[t] = p->cx[t];
  }
  fp.tbl = p->d_tbl;
  fp.inv_wsum = p->d_tbl + p->n_tbl;
  fp.wfull = p->d_tbl + p->n_tbl + p->n_inv;
  fp.out = out;
  fp.status = status;
  fp.tmap = -1;
  fp.F = 0;
}

static long long fused_units(const FusedParams& fp) {
  return (long long)fp.tiles_x * fp.tiles_y * fp.n_tp * fp.chunks;
}

static int launch_fused_mode(const nx_esrrf_plan* p, int mode, const float* d_in, int T, int fpt,
                             int n_tp, int chunks, float* out, unsigned* status,
                             cudaStream_t s, unsigned long long wait_ns = 0,
                             int withhold_full = 0) {
  UnitTable ut;
  memset(&ut, 0, sizeof(ut));
  fill_params(p, ut.single, d_in, T, fpt, n_tp, chunks, out, status);
  ut.single.F = mode_fields(mode);
  ut.single.wait_ns = wait_ns;
  ut.single.test_withhold_full = withhold_full;
  TmapPack pack;
  memset(&pack, 0, sizeof(pack));
  if (!tma_disabled() && make_frame_tmap(&pack.m[0], d_in, T, p->H, p->W, p->fused->geo.BW,
                                         p->fused->geo.BH))
    ut.single.tmap = 0;
  const long long units = fused_units(ut.single);
  if (units > 0x7fffffffLL) return invalid("work too large for one launch");
  ut.n_items = 1;
  ut.ns_cap = 1;
  ut.total_units = (int)units;
  // persistent grid: the resident CTAs stride over the units (setup and the
  // phase-table copy once per CTA instead of once per unit)
  const long long resident = (long long)p->fused->occupancy[mode](1) * device_sms();
  const int grid = (int)std::min<long long>(units, std::max<long long>(1, resident));
  cudaError_t e = p->fused->launch[mode](ut, pack, grid, s);
  if (e != cudaSuccess) return cuda_status(e, "fused eSRRF launch");
  return NX_OK;
}

// ---------------------------------------------------------------------------
// general (unfused) pipeline for (m, R) without a fused instantiation: the
// reference's own sequence CR(m) -> RobX -> CR(2m) x 2 -> RGC, one frame at a
// time, reading only what the reference reads.
// ---------------------------------------------------------------------------
static size_t generic_frame_floats(const nx_esrrf_plan* p) {
  const size_t planeM = (size_t)p->rowsM * p->colsM;
  const size_t plane = (size_t)p->H * p->W;
  return planeM /*mag*/ + 2 * plane /*gc, gr*/ + 2 * 4 * planeM /*gci, gri*/ + planeM /*rgc*/ +
         2 * 64 /*shift arrays*/;
}

static int generic_frame(const nx_esrrf_plan* p, const float* frame, float* out_frame,
                         float* scratch, cudaStream_t s) {
  const size_t planeM = (size_t)p->rowsM * p->colsM;
  const size_t plane = (size_t)p->H * p->W;
  float* mag = scratch;
  float* gc = mag + planeM;
  float* gr = gc + plane;
  float* gci = gr + plane;
  float* gri = gci + 4 * planeM;
  float* zeros = gri + 4 * planeM + planeM;
  cudaError_t e = cudaMemsetAsync(zeros, 0, 64 * sizeof(float), s);
  if (e != cudaSuccess) return cuda_status(e, "memset");
  const int M = p->M;
  e = launch_cr_shift_magnify(frame, 1, p->H, p->W, zeros, zeros, (float)M, (float)M, p->rowsM,
                              p->colsM, mag, s);
  if (e == cudaSuccess) e = launch_roberts_cross(frame, 1, p->H, p->W, gc, gr, s);
  if (e == cudaSuccess)
    e = launch_cr_shift_magnify(gc, 1, p->H, p->W, zeros, zeros, (float)(2 * M), (float)(2 * M),
                                2 * p->rowsM, 2 * p->colsM, gci, s);
  if (e == cudaSuccess)
    e = launch_cr_shift_magnify(gr, 1, p->H, p->W, zeros, zeros, (float)(2 * M), (float)(2 * M),
                                2 * p->rowsM, 2 * p->colsM, gri, s);
  if (e == cudaSuccess)
    e = launch_rgc(gci, gri, mag, 1, p->rowsM, p->colsM, M, p->sc, p->iw, out_frame, s);
  if (e != cudaSuccess) return cuda_status(e, "unfused eSRRF frame");
  return NX_OK;
}

}  // namespace nx

using namespace nx;

extern "C" {

int nx_abi_version(void) { return NX_ABI_VERSION; }

const char* nx_last_error(void) { return g_err; }

int nx_esrrf_plan_create(nx_esrrf_plan** out, int H, int W, int magnification, float radius,
                         float sensitivity, int do_intensity_weighting) {
  if (!out) return invalid("plan out-pointer is NULL");
  *out = nullptr;
  if (H < 1 || W < 1) return invalid("image must have H, W >= 1");
  if (magnification < 1 || magnification > 64) return invalid("magnification must be in [1, 64]");
  if (!(radius > 0.f) || !(radius < 64.f)) return invalid("radius must be in (0, 64)");
  if ((long long)H * magnification * 2 >= (1LL << 24) || (long long)W * magnification * 2 >= (1LL << 24))
    return invalid("magnified image too large for float32 coordinates");
  nx_esrrf_plan* p = new nx_esrrf_plan();
  p->H = H;
  p->W = W;
  p->M = magnification;
  p->radius = radius;
  p->sensitivity = sensitivity;
  p->iw = do_intensity_weighting ? 1 : 0;
  p->rowsM = H * magnification;
  p->colsM = W * magnification;
  p->sc = rgc_scalars(magnification, radius, sensitivity, 0);
  p->JW = std::max(-p->sc.start, p->sc.end - 1);
  p->fused = (p->JW >= 1 && p->JW <= 6) ? fused_entry(magnification, p->JW) : nullptr;
  p->tile_variant = 0;
  if (p->fused) {
    // instantiations whose shared-memory layout does not fit a CTA use the general path
    const size_t lim = kSmemBudget;
    for (int mode = 0; mode < 3; ++mode)
      if (p->fused->smem[mode](1) > lim) p->fused = nullptr;
  }
  clamp_taps(H, magnification, &p->cy_base, p->cy);
  clamp_taps(W, magnification, &p->cx_base, p->cx);
  cudaGetDevice(&p->device);
  p->d_tbl = nullptr;
  if (p->fused) {
    std::vector<float> tbl, inv, wfull;
    build_tables(p, tbl, inv, wfull);
    p->n_tbl = tbl.size();
    p->n_inv = inv.size();
    p->n_wfull = wfull.size();
    std::vector<float> all;
    all.reserve(tbl.size() + inv.size() + wfull.size());
    all.insert(all.end(), tbl.begin(), tbl.end());
    all.insert(all.end(), inv.begin(), inv.end());
    all.insert(all.end(), wfull.begin(), wfull.end());
    cudaError_t e = cudaMalloc(&p->d_tbl, all.size() * sizeof(float));
    if (e != cudaSuccess) {
      delete p;
      return cuda_status(e, "plan table allocation");
    }
    e = cudaMemcpy(p->d_tbl, all.data(), all.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(p->d_tbl);
      delete p;
      return cuda_status(e, "plan table upload");
    }
  }
  *out = p;
  return NX_OK;
}

int nx_esrrf_plan_set_tile_variant(nx_esrrf_plan* p, int variant) {
  if (!p) return invalid("plan is NULL");
  if (!p->fused) {
    set_error("this plan runs the general (unfused) path: no tilings to choose from");
    return NX_ERR_UNSUPPORTED;
  }
  if (variant < 0 || variant >= kTileVariants) return invalid("tile variant must be 0 or 1");
  const FusedEntry* e = fused_entry(p->M, p->JW, variant);
  if (!e) {
    set_error("magnification %d, window %d has no tile variant %d", p->M, p->JW, variant);
    return NX_ERR_UNSUPPORTED;
  }
  for (int mode = 0; mode < 3; ++mode)
    if (e->smem[mode](1) > kSmemBudget) {
      set_error("tile variant %d does not fit a CTA's shared memory at this window", variant);
      return NX_ERR_UNSUPPORTED;
    }
  p->fused = e;
  p->tile_variant = variant;
  return NX_OK;
}

int nx_esrrf_plan_tile_variant(const nx_esrrf_plan* p) {
  if (!p) return invalid("plan is NULL");
  return p->fused ? p->tile_variant : NX_ERR_UNSUPPORTED;
}

int nx_esrrf_weight_table(int magnification, float radius, float* h_out, size_t cap) {
  if (magnification < 1 || magnification > 64) return invalid("magnification must be in [1, 64]");
  if (!(radius > 0.f) || !(radius < 64.f)) return invalid("radius must be in (0, 64)");
  nx_esrrf_plan tmp{};
  tmp.M = magnification;
  tmp.radius = radius;
  tmp.sc = rgc_scalars(magnification, radius, 1.f, 0);
  tmp.JW = std::max(-tmp.sc.start, tmp.sc.end - 1);
  const size_t W2 = 2 * (size_t)tmp.JW + 1;
  const size_t need = (size_t)magnification * magnification * W2 * W2;
  if (h_out && cap >= need) {
    std::vector<float> tbl, inv, wfull;
    build_tables(&tmp, tbl, inv, wfull);
    std::memcpy(h_out, wfull.data(), need * sizeof(float));
  }
  return tmp.JW;
}

int nx_esrrf_plan_destroy(nx_esrrf_plan* p) {
  if (!p) return NX_OK;
  if (p->d_tbl) cudaFree(p->d_tbl);
  delete p;
  return NX_OK;
}

size_t nx_esrrf_st_workspace_bytes(const nx_esrrf_plan* p, int T) {
  (void)T;
  if (!p) return 0;
  size_t b = kStatusBytes;
  if (!p->fused) b += align256(generic_frame_floats(p) * sizeof(float));
  return b;
}

int nx_esrrf_st(const nx_esrrf_plan* p, const float* d_in, int T, float* d_out, void* d_ws,
                size_t ws_bytes, void* stream) {
  int rc = check_plan(p);
  if (rc) return rc;
  if (T < 0) return invalid("T must be >= 0");
  if (T == 0) return NX_OK;
  if (!d_in || !d_out) return invalid("NULL input/output");
  if (!d_ws || ws_bytes < nx_esrrf_st_workspace_bytes(p, T)) {
    set_error("workspace too small: need %zu bytes", nx_esrrf_st_workspace_bytes(p, T));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* status = (unsigned*)d_ws;
  NX_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), s));
  if (p->fused) return launch_fused_mode(p, kModeStack, d_in, T, T, 1, 1, d_out, status, s);
  float* scratch = (float*)((char*)d_ws + kStatusBytes);
  const size_t planeM = (size_t)p->rowsM * p->colsM;
  for (int t = 0; t < T; ++t) {
    rc = generic_frame(p, d_in + (size_t)t * p->H * p->W, d_out + (size_t)t * planeM, scratch, s);
    if (rc) return rc;
  }
  return NX_OK;
}

int nx_selftest_fused_abort(const nx_esrrf_plan* p, const float* d_in, int T, float* d_out,
                            void* d_ws, size_t ws_bytes, unsigned long long limit_ns,
                            void* stream) {
  int rc = check_plan(p);
  if (rc) return rc;
  if (!p->fused) return invalid("the self-test needs a plan with a fused kernel");
  if (T < 1 || !d_in || !d_out) return invalid("need frames and buffers");
  if (limit_ns < 1000000ull || limit_ns > 1000000000ull)
    return invalid("limit_ns must be in [1 ms, 1 s]");  // keep the self-test short
  if (!d_ws || ws_bytes < nx_esrrf_st_workspace_bytes(p, T)) {
    set_error("workspace too small: need %zu bytes", nx_esrrf_st_workspace_bytes(p, T));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* status = (unsigned*)d_ws;
  NX_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), s));
  return launch_fused_mode(p, kModeStack, d_in, T, T, 1, 1, d_out, status, s, limit_ns, 1);
}

size_t nx_esrrf_workspace_bytes(const nx_esrrf_plan* p, int T, int fpt, int corr_mask) {
  if (!p || T < 1) return kStatusBytes;
  if (fpt <= 0 || fpt > T) fpt = T;
  const int n_tp = (T + fpt - 1) / fpt;
  const size_t planeM = (size_t)p->rowsM * p->colsM;
  const int F = fields_for(corr_mask);
  size_t b = kStatusBytes;
  if (p->fused) {
    const int chunks = plan_chunks(p, T, fpt, n_tp);
    b += align256((size_t)n_tp * chunks * F * planeM * sizeof(float));
  } else {
    b += align256((size_t)n_tp * 5 * planeM * sizeof(float));
    b += align256(generic_frame_floats(p) * sizeof(float));
  }
  b += nx_macro_pixel_workspace_bytes(corr_count(corr_mask) * n_tp, p->M);
  return b;
}

static int esrrf_validate(const nx_esrrf_plan* p, int T, int& fpt, int corr_mask, void* d_ws,
                          size_t ws_bytes) {
  int rc = check_plan(p);
  if (rc) return rc;
  if (T < 1) return invalid("need at least one frame");
  if (corr_mask <= 0 || corr_mask > 7) return invalid("Type of correlation must be AVG, VAR or TAC2");
  if (fpt <= 0 || fpt > T) fpt = T;
  const size_t need = nx_esrrf_workspace_bytes(p, T, fpt, corr_mask);
  if (!d_ws || ws_bytes < need) {
    set_error("workspace too small: need %zu bytes", need);
    return NX_ERR_WORKSPACE;
  }
  return NX_OK;
}

int nx_esrrf_run_stage1(const nx_esrrf_plan* p, const float* d_in, int T, int fpt, int corr_mask,
                        void* d_ws, size_t ws_bytes, void* stream) {
  int rc = esrrf_validate(p, T, fpt, corr_mask, d_ws, ws_bytes);
  if (rc) return rc;
  if (!d_in) return invalid("NULL input");
  cudaStream_t s = (cudaStream_t)stream;
  const int n_tp = (T + fpt - 1) / fpt;
  const long long planeM = (long long)p->rowsM * p->colsM;
  const int F = fields_for(corr_mask);
  unsigned* status = (unsigned*)d_ws;
  char* cur = (char*)d_ws + kStatusBytes;
  NX_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), s));
  float* rec = (float*)cur;
  if (p->fused) {
    const int chunks = plan_chunks(p, T, fpt, n_tp);
    return launch_fused_mode(p, F == 5 ? kModeFull : kModeSum, d_in, T, fpt, n_tp, chunks, rec,
                             status, s);
  }
  cur += align256((size_t)n_tp * 5 * planeM * sizeof(float));
  float* scratch = (float*)cur;
  float* rgc_frame = scratch + (size_t)planeM + 2 * (size_t)p->H * p->W + 8 * (size_t)planeM;
  for (int t = 0; t < T; ++t) {
    const int tp = t / fpt;
    rc = generic_frame(p, d_in + (size_t)t * p->H * p->W, rgc_frame, scratch, s);
    if (rc) return rc;
    cudaError_t e = launch_record_push_frame(rgc_frame, planeM, rec + (size_t)tp * 5 * planeM,
                                             t - tp * fpt, s);
    if (e != cudaSuccess) return cuda_status(e, "record push");
  }
  return NX_OK;
}

int nx_esrrf_run_stage2(const nx_esrrf_plan* p, int T, int fpt, int corr_mask, int mpc,
                        float* d_out, void* d_ws, size_t ws_bytes, void* stream) {
  int rc = esrrf_validate(p, T, fpt, corr_mask, d_ws, ws_bytes);
  if (rc) return rc;
  if (!d_out) return invalid("NULL output");
  cudaStream_t s = (cudaStream_t)stream;
  const int n_tp = (T + fpt - 1) / fpt;
  const long long planeM = (long long)p->rowsM * p->colsM;
  const int F = fields_for(corr_mask);
  const int ncorr = corr_count(corr_mask);
  char* cur = (char*)d_ws + kStatusBytes;
  float* rec = (float*)cur;
  int chunks = 1, Fr = 5;
  if (p->fused) {
    chunks = plan_chunks(p, T, fpt, n_tp);
    Fr = F;
    cur += align256((size_t)n_tp * chunks * F * planeM * sizeof(float));
  } else {
    cur += align256((size_t)n_tp * 5 * planeM * sizeof(float));
    cur += align256(generic_frame_floats(p) * sizeof(float));
  }
  float* map = (float*)cur;
  for (int tp = 0; tp < n_tp; ++tp) {
    const int nf = std::min(fpt, T - tp * fpt);
    const int nch = std::min(chunks, nf);
    cudaError_t e = launch_finalize(rec + (size_t)tp * chunks * Fr * planeM, Fr, nch, nf, planeM,
                                    corr_mask, d_out + (size_t)tp * planeM,
                                    (long long)n_tp * planeM, Fr == 5, s);
    if (e != cudaSuccess) return cuda_status(e, "temporal finalize");
  }
  if (mpc) {
    cudaError_t e = launch_mpc(d_out, ncorr * n_tp, p->rowsM, p->colsM, p->M, map, s);
    if (e != cudaSuccess) return cuda_status(e, "macro-pixel correction");
  }
  return NX_OK;
}

int nx_esrrf_run(const nx_esrrf_plan* p, const float* d_in, int T, int fpt, int corr_mask,
                 int mpc, float* d_out, void* d_ws, size_t ws_bytes, void* stream) {
  if (!d_out) return invalid("NULL output");
  int rc = nx_esrrf_run_stage1(p, d_in, T, fpt, corr_mask, d_ws, ws_bytes, stream);
  if (rc) return rc;
  return nx_esrrf_run_stage2(p, T, fpt, corr_mask, mpc, d_out, d_ws, ws_bytes, stream);
}

size_t nx_esrrf_accum_bytes(const nx_esrrf_plan* p) {
  if (!p) return 0;
  return align256((size_t)5 * p->rowsM * p->colsM * sizeof(float));
}

size_t nx_esrrf_push_workspace_bytes(const nx_esrrf_plan* p, int T_block) {
  if (!p || T_block < 1) return kStatusBytes;
  return nx_esrrf_workspace_bytes(p, T_block, T_block, NX_CORR_VAR | NX_CORR_TAC2);
}

int nx_esrrf_accum_push(const nx_esrrf_plan* p, const float* d_block, int T_block,
                        int frames_before, void* d_accum, void* d_ws, size_t ws_bytes,
                        void* stream) {
  int rc = check_plan(p);
  if (rc) return rc;
  if (T_block < 1 || frames_before < 0) return invalid("bad block size / frame offset");
  if (!d_block || !d_accum) return invalid("NULL block/accumulator");
  const size_t need = nx_esrrf_push_workspace_bytes(p, T_block);
  if (!d_ws || ws_bytes < need) {
    set_error("workspace too small: need %zu bytes", need);
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const long long planeM = (long long)p->rowsM * p->colsM;
  unsigned* status = (unsigned*)d_ws;
  float* rec = (float*)((char*)d_ws + kStatusBytes);
  float* acc = (float*)d_accum;
  // block records: chunks merged in order into rec chunk 0 ... then into acc
  int chunks = 1;
  if (p->fused) {
    chunks = plan_chunks(p, T_block, T_block, 1);
    rc = launch_fused_mode(p, kModeFull, d_block, T_block, T_block, 1, chunks, rec, status, s);
    if (rc) return rc;
  } else {
    float* scratch = rec + align256((size_t)5 * planeM * sizeof(float)) / sizeof(float);
    float* rgc_frame = scratch + (size_t)planeM + 2 * (size_t)p->H * p->W + 8 * (size_t)planeM;
    for (int t = 0; t < T_block; ++t) {
      rc = generic_frame(p, d_block + (size_t)t * p->H * p->W, rgc_frame, scratch, s);
      if (rc) return rc;
      cudaError_t e = launch_record_push_frame(rgc_frame, planeM, rec, t, s);
      if (e != cudaSuccess) return cuda_status(e, "record push");
    }
  }
  int n_acc = frames_before;
  for (int c = 0; c < chunks; ++c) {
    const int nc = (int)((long long)(c + 1) * T_block / chunks - (long long)c * T_block / chunks);
    cudaError_t e;
    if (n_acc == 0) {
      e = cudaMemcpyAsync(acc, rec + (size_t)c * 5 * planeM, (size_t)5 * planeM * sizeof(float),
                          cudaMemcpyDeviceToDevice, s);
    } else {
      e = launch_record_merge(acc, rec + (size_t)c * 5 * planeM, planeM, n_acc, nc, s);
    }
    if (e != cudaSuccess) return cuda_status(e, "accumulator merge");
    n_acc += nc;
  }
  return NX_OK;
}

int nx_esrrf_accum_finalize(const nx_esrrf_plan* p, const void* d_accum, int total_frames,
                            int corr_mask, int mpc, float* d_out, void* d_ws, size_t ws_bytes,
                            void* stream) {
  int rc = check_plan(p);
  if (rc) return rc;
  if (total_frames < 1) return invalid("no frames were pushed");
  if (corr_mask <= 0 || corr_mask > 7) return invalid("Type of correlation must be AVG, VAR or TAC2");
  const int ncorr = corr_count(corr_mask);
  const size_t need = kStatusBytes + nx_macro_pixel_workspace_bytes(ncorr, p->M);
  if (!d_ws || ws_bytes < need) {
    set_error("workspace too small: need %zu bytes", need);
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const long long planeM = (long long)p->rowsM * p->colsM;
  cudaError_t e = launch_finalize((const float*)d_accum, 5, 1, total_frames, planeM, corr_mask,
                                  d_out, planeM, true, s);
  if (e != cudaSuccess) return cuda_status(e, "temporal finalize");
  if (mpc) {
    float* map = (float*)((char*)d_ws + kStatusBytes);
    e = launch_mpc(d_out, ncorr, p->rowsM, p->colsM, p->M, map, s);
    if (e != cudaSuccess) return cuda_status(e, "macro-pixel correction");
  }
  return NX_OK;
}

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
}  // extern "C"

struct nx_esrrf_batch {
  struct Item {
    nx_esrrf_item desc;
    int mode;            // kModeSum / kModeFull
    int n_out;           // outputs per timepoint (n_corr or n_sens)
    int fpt, n_tp, chunks;
    size_t rec_off;      // byte offsets in the workspace
    size_t mpc_off;
    nx::FusedParams fp;  // device pointers filled at bind()
    int cls;
  };
  struct Class {
    const nx::FusedEntry* entry;
    int mode;
    int ns_cap;
    std::vector<int> items;
    std::vector<int> unit_start;  // prefix sums, size n + 1
    size_t params_off, starts_off;
    size_t jobs_off;      // the class's temporal finalisations (FinalizeJob list)
    int n_jobs, job_blocks;
    int grid;
    nx::TmapPack maps;
  };
  std::vector<Item> items;
  std::vector<Class> classes;
  size_t ws_bytes = 0;
  size_t counters_off = 0;
  void* d_ws = nullptr;
  int device = -1;
  // one side stream per class after the first, and the events that fork them
  // from / join them back into the caller's stream (created at bind)
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> events;  // [0]: fork, [1 + c]: class c done
  ~nx_esrrf_batch() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    for (cudaStream_t st : side) cudaStreamDestroy(st);
  }
};

namespace nx {

static int batch_item_mode(const nx_esrrf_item& it) {
  return (it.n_sens > 0 || it.corr_mask == NX_CORR_AVG) ? kModeSum : kModeFull;
}

}  // namespace nx

extern "C" {

int nx_esrrf_batch_create(nx_esrrf_batch** out, const nx_esrrf_item* items, int n) {
  if (!out) return invalid("batch out-pointer is NULL");
  *out = nullptr;
  if (n < 1 || !items) return invalid("empty batch");
  int dev = -1;
  NX_CUDA_TRY(cudaGetDevice(&dev));
  auto* b = new nx_esrrf_batch();
  b->device = dev;
  const int sms = device_sms();
  for (int i = 0; i < n; ++i) {
    const nx_esrrf_item& it = items[i];
    const nx_esrrf_plan* p = it.plan;
    int rc = check_plan(p);
    if (rc) { delete b; return rc; }
    if (!p->fused) {
      delete b;
      set_error("batch item %d: magnification %d / radius %g has no fused kernel", i, p->M,
                (double)p->radius);
      return NX_ERR_UNSUPPORTED;
    }
    if (it.T < 1 || !it.d_in || !it.d_out) { delete b; return invalid("batch item without frames or buffers"); }
    if (it.n_sens < 0 || it.n_sens > kMaxSens) { delete b; return invalid("n_sens must be 0..4"); }
    if (it.corr_mask <= 0 || it.corr_mask > 7) { delete b; return invalid("Type of correlation must be AVG, VAR or TAC2"); }
    if (it.n_sens > 0 && it.corr_mask != NX_CORR_AVG) { delete b; return invalid("sensitivity sweeps are AVG only"); }
    nx_esrrf_batch::Item bi;
    bi.desc = it;
    bi.mode = batch_item_mode(it);
    bi.n_out = it.n_sens > 0 ? it.n_sens : corr_count(it.corr_mask);
    bi.fpt = (it.frames_per_timepoint <= 0 || it.frames_per_timepoint > it.T) ? it.T
                                                                                : it.frames_per_timepoint;
    bi.n_tp = (it.T + bi.fpt - 1) / bi.fpt;
    const int min_nf = std::min(bi.fpt, it.T - (bi.n_tp - 1) * bi.fpt);
    int fpu = it.frames_per_unit;
    if (fpu <= 0) {
      // heuristic: the chunking that balances this item alone over the resident CTAs
      const long long tiles = (long long)((p->W + 31) / 32) * ((p->H + p->fused->geo.TY - 1) / p->fused->geo.TY);
      const long long resident =
          (long long)std::max(1, p->fused->occupancy[bi.mode](std::max(1, it.n_sens))) * sms;
      const int c = best_chunks(tiles, bi.n_tp, bi.fpt, min_nf, resident);
      fpu = std::max(1, (min_nf + c - 1) / c);
    }
    bi.chunks = std::max(1, std::min(min_nf, (min_nf + fpu - 1) / fpu));
    bi.cls = -1;
    // class by (kernel entry, mode)
    for (size_t c = 0; c < b->classes.size(); ++c)
      if (b->classes[c].entry == p->fused && b->classes[c].mode == bi.mode) bi.cls = (int)c;
    if (bi.cls < 0) {
      nx_esrrf_batch::Class cl;
      cl.entry = p->fused;
      cl.mode = bi.mode;
      cl.grid = 0;
      memset(&cl.maps, 0, sizeof(cl.maps));
      b->classes.push_back(cl);
      bi.cls = (int)b->classes.size() - 1;
    }
    b->classes[bi.cls].items.push_back(i);
    b->items.push_back(bi);
  }
  // workspace layout
  size_t off = kStatusBytes;
  b->counters_off = off;
  off += align256(b->classes.size() * sizeof(unsigned));
  for (auto& cl : b->classes) {
    cl.params_off = off;
    off += align256(cl.items.size() * sizeof(FusedParams));
    cl.starts_off = off;
    off += align256((cl.items.size() + 1) * sizeof(int));
    cl.unit_start.assign(1, 0);
    for (int idx : cl.items) {
      const auto& bi = b->items[idx];
      const nx_esrrf_plan* p = bi.desc.plan;
      const long long tiles = (long long)((p->W + 31) / 32) * ((p->H + p->fused->geo.TY - 1) / p->fused->geo.TY);
      const long long u = (long long)cl.unit_start.back() + tiles * bi.n_tp * bi.chunks;
      if (u > 0x7fffffffLL) { delete b; return invalid("batch too large for one launch"); }
      cl.unit_start.push_back((int)u);
    }
    cl.ns_cap = 1;
    for (int idx : cl.items) cl.ns_cap = std::max(cl.ns_cap, b->items[idx].desc.n_sens);
    const int occ = cl.entry->occupancy[cl.mode](cl.ns_cap);
    if (occ < 1) {
      delete b;
      set_error("a batch class needs more shared memory than a CTA can hold "
                "(too many sensitivities at this magnification)");
      return NX_ERR_UNSUPPORTED;
    }
    cl.grid = std::min(cl.unit_start.back(), occ * sms);
    // one finalisation job per item, timepoint and (AVG sweep) sensitivity
    cl.n_jobs = 0;
    long long blocks = 0;
    for (int idx : cl.items) {
      const auto& bi = b->items[idx];
      const long long planeM = (long long)bi.desc.plan->rowsM * bi.desc.plan->colsM;
      const int per_tp = bi.mode == kModeFull ? 1 : bi.n_out;
      cl.n_jobs += bi.n_tp * per_tp;
      blocks += (long long)bi.n_tp * per_tp * ((planeM + 255) / 256);
    }
    if (blocks > 0x7fffffffLL) { delete b; return invalid("batch too large for one launch"); }
    cl.job_blocks = (int)blocks;
    cl.jobs_off = off;
    off += align256((size_t)cl.n_jobs * sizeof(FinalizeJob));
  }
  for (auto& bi : b->items) {
    const nx_esrrf_plan* p = bi.desc.plan;
    const size_t planeM = (size_t)p->rowsM * p->colsM;
    const int F = bi.mode == kModeFull ? 5 : bi.n_out;
    bi.rec_off = off;
    off += align256((size_t)bi.n_tp * bi.chunks * F * planeM * sizeof(float));
    bi.mpc_off = off;
    off += nx_macro_pixel_workspace_bytes(bi.n_out * bi.n_tp, p->M);
  }
  b->ws_bytes = off;
  *out = b;
  return NX_OK;
}

size_t nx_esrrf_batch_workspace_bytes(const nx_esrrf_batch* b) { return b ? b->ws_bytes : 0; }

int nx_esrrf_batch_bind(nx_esrrf_batch* b, void* d_ws, size_t ws_bytes, void* stream) {
  if (!b) return invalid("batch is NULL");
  if (!d_ws || ws_bytes < b->ws_bytes) {
    set_error("workspace too small: need %zu bytes", b->ws_bytes);
    return NX_ERR_WORKSPACE;
  }
  int dev = -1;
  NX_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != b->device) return invalid("batch bound on another device than it was created on");
  cudaStream_t s = (cudaStream_t)stream;
  char* base = (char*)d_ws;
  unsigned* status = (unsigned*)base;
  while (b->side.size() + 1 < b->classes.size()) {
    cudaStream_t st = nullptr;
    NX_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    b->side.push_back(st);
  }
  while (b->events.size() < b->classes.size() + 1) {
    cudaEvent_t e = nullptr;
    NX_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->events.push_back(e);
  }
  for (size_t c = 0; c < b->classes.size(); ++c) {
    auto& cl = b->classes[c];
    std::vector<FusedParams> params(cl.items.size());
    int nmaps = 0;
    for (size_t k = 0; k < cl.items.size(); ++k) {
      auto& bi = b->items[cl.items[k]];
      const nx_esrrf_plan* p = bi.desc.plan;
      FusedParams& fp = params[k];
      fill_params(p, fp, bi.desc.d_in, bi.desc.T, bi.fpt, bi.n_tp, bi.chunks,
                  (float*)(base + bi.rec_off), status);
      if (bi.mode == kModeSum) {
        const int ns = bi.desc.n_sens > 0 ? bi.desc.n_sens : 1;
        fp.n_sens = ns;
        fp.F = ns;
        for (int k2 = 0; k2 < ns && bi.desc.n_sens > 0; ++k2) {
          const RgcScalars sc = rgc_scalars(p->M, p->radius, bi.desc.sens[k2], 0);
          fp.sens_mode_k[k2] = sc.sens_mode;
          fp.sens_int_k[k2] = sc.sens_int;
          fp.sens_k[k2] = sc.sens;
        }
      } else {
        fp.F = 5;
      }
      if (nmaps < kMaxTmaps && !tma_disabled() &&
          make_frame_tmap(&cl.maps.m[nmaps], bi.desc.d_in, bi.desc.T, p->H, p->W,
                          p->fused->geo.BW, p->fused->geo.BH))
        fp.tmap = nmaps++;
      bi.fp = fp;
    }
    NX_CUDA_TRY(cudaMemcpyAsync(base + cl.params_off, params.data(),
                                params.size() * sizeof(FusedParams), cudaMemcpyHostToDevice, s));
    NX_CUDA_TRY(cudaMemcpyAsync(base + cl.starts_off, cl.unit_start.data(),
                                cl.unit_start.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    std::vector<FinalizeJob> jobs;
    jobs.reserve(cl.n_jobs);
    int block0 = 0;
    for (int idx : cl.items) {
      const auto& bi = b->items[idx];
      const nx_esrrf_plan* p = bi.desc.plan;
      const long long planeM = (long long)p->rowsM * p->colsM;
      const bool full = bi.mode == kModeFull;
      const int F = full ? 5 : bi.n_out;
      const float* rec = (const float*)(base + bi.rec_off);
      const long long stride = (long long)bi.n_tp * planeM;
      const int nblk = (int)((planeM + 255) / 256);
      for (int tp = 0; tp < bi.n_tp; ++tp) {
        const int nf = std::min(bi.fpt, bi.desc.T - tp * bi.fpt);
        const int nch = std::min(bi.chunks, nf);
        const float* rtp = rec + (size_t)tp * bi.chunks * F * planeM;
        float* out = bi.desc.d_out + (size_t)tp * planeM;
        for (int k = 0; k < (full ? 1 : bi.n_out); ++k) {
          FinalizeJob j;
          j.rec = full ? rtp : rtp + (size_t)k * planeM;
          j.out = full ? out : out + (size_t)k * stride;
          j.n = planeM;
          j.out_stride = stride;
          j.F = F;
          j.nchunks = nch;
          j.nf = nf;
          j.corr_mask = full ? bi.desc.corr_mask : NX_CORR_AVG;
          j.full = full ? 1 : 0;
          j.block0 = block0;
          block0 += nblk;
          jobs.push_back(j);
        }
      }
    }
    if (!jobs.empty())
      NX_CUDA_TRY(cudaMemcpyAsync(base + cl.jobs_off, jobs.data(), jobs.size() * sizeof(FinalizeJob),
                                  cudaMemcpyHostToDevice, s));
  }
  NX_CUDA_TRY(cudaStreamSynchronize(s));
  b->d_ws = d_ws;
  return NX_OK;
}

int nx_esrrf_batch_launch(const nx_esrrf_batch* b, void* stream) {
  if (!b || !b->d_ws) return invalid("batch is not bound to a workspace");
  cudaStream_t s = (cudaStream_t)stream;
  char* base = (char*)b->d_ws;
  NX_CUDA_TRY(cudaMemsetAsync(base, 0, kStatusBytes + align256(b->classes.size() * sizeof(unsigned)),
                              s));
  // class 0 runs on the caller's stream, class c > 0 on side stream c - 1,
  // forked after the memset and joined back at the end: one class's wave tail,
  // finalisation and macro-pixel correction overlap the next class's kernel
  const size_t nc = b->classes.size();
  if (nc > 1) {
    NX_CUDA_TRY(cudaEventRecord(b->events[0], s));
    for (size_t c = 1; c < nc; ++c) NX_CUDA_TRY(cudaStreamWaitEvent(b->side[c - 1], b->events[0], 0));
  }
  for (size_t c = 0; c < nc; ++c) {
    const auto& cl = b->classes[c];
    cudaStream_t cs = c == 0 ? s : b->side[c - 1];
    UnitTable ut;
    memset(&ut, 0, sizeof(ut));
    ut.items = (const FusedParams*)(base + cl.params_off);
    ut.unit_start = (const int*)(base + cl.starts_off);
    ut.n_items = (int)cl.items.size();
    ut.total_units = cl.unit_start.back();
    ut.counter = (unsigned*)(base + b->counters_off) + c;
    ut.ns_cap = cl.ns_cap;
    cudaError_t e = cl.entry->launch[cl.mode](ut, cl.maps, cl.grid, cs);
    if (e != cudaSuccess) return cuda_status(e, "batched eSRRF launch");
    // every item's temporal finalisation of this class in one launch
    e = launch_finalize_jobs((const FinalizeJob*)(base + cl.jobs_off), cl.n_jobs, cl.job_blocks,
                             cs);
    if (e != cudaSuccess) return cuda_status(e, "batched temporal finalize");
    for (int idx : cl.items) {
      const auto& bi = b->items[idx];
      const nx_esrrf_plan* p = bi.desc.plan;
      if (bi.desc.macro_pixel_correction) {
        e = launch_mpc(bi.desc.d_out, bi.n_out * bi.n_tp, p->rowsM, p->colsM, p->M,
                       (float*)(base + bi.mpc_off), cs);
        if (e != cudaSuccess) return cuda_status(e, "batched macro-pixel correction");
      }
    }
    if (c > 0) NX_CUDA_TRY(cudaEventRecord(b->events[c + 1], cs));
  }
  for (size_t c = 1; c < nc; ++c) NX_CUDA_TRY(cudaStreamWaitEvent(s, b->events[c + 1], 0));
  return NX_OK;
}

int nx_esrrf_batch_destroy(nx_esrrf_batch* b) {
  delete b;
  return NX_OK;
}

int nx_workspace_status(const void* d_ws, void* stream) {
  if (!d_ws) return invalid("NULL workspace");
  unsigned st = 0;
  cudaStream_t s = (cudaStream_t)stream;
  NX_CUDA_TRY(cudaMemcpyAsync(&st, d_ws, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  NX_CUDA_TRY(cudaStreamSynchronize(s));
  if (st & kDevTmaTimeout) {
    set_error("a TMA tile wait timed out on the device (status 0x%x)", st);
    return NX_ERR_DEVICE_TIMEOUT;
  }
  if (st) {
    set_error("device status 0x%x", st);
    return NX_ERR_CUDA;
  }
  return NX_OK;
}

int nx_cr_shift_magnify(const float* d_in, int T, int H, int W, const float* d_shift_row,
                        const float* d_shift_col, float mag_row, float mag_col, float* d_out,
                        void* stream) {
  if (T < 0 || H < 1 || W < 1) return invalid("bad image shape");
  if (!(mag_row > 0.f) || !(mag_col > 0.f)) return invalid("magnification must be > 0");
  const int rowsM = (int)((float)H * mag_row);
  const int colsM = (int)((float)W * mag_col);
  cudaError_t e = launch_cr_shift_magnify(d_in, T, H, W, d_shift_row, d_shift_col, mag_row,
                                          mag_col, rowsM, colsM, d_out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "ShiftAndMagnify");
  return NX_OK;
}

int nx_roberts_cross(const float* d_in, int T, int H, int W, float* d_gc, float* d_gr,
                     void* stream) {
  if (T < 0 || H < 1 || W < 1) return invalid("bad image shape");
  cudaError_t e = launch_roberts_cross(d_in, T, H, W, d_gc, d_gr, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "GradientRobertsCross");
  return NX_OK;
}

int nx_rgc(const float* d_gc, const float* d_gr, const float* d_img, int T, int rowsM, int colsM,
           int magnification, float radius, float sensitivity, int iw, int pad_edges,
           float* d_out, void* stream) {
  if (T < 0 || rowsM < 1 || colsM < 1) return invalid("bad image shape");
  if (magnification < 1) return invalid("magnification must be >= 1");
  if (!(radius > 0.f)) return invalid("radius must be > 0");
  const RgcScalars sc = rgc_scalars(magnification, radius, sensitivity, pad_edges);
  cudaError_t e = launch_rgc(d_gc, d_gr, d_img, T, rowsM, colsM, magnification, sc, iw ? 1 : 0,
                             d_out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "RadialGradientConvergence");
  return NX_OK;
}

size_t nx_radiality_workspace_bytes(int T, int h, int w) {
  return align256((size_t)2 * T * h * w * sizeof(float));
}

int nx_radiality(const float* d_img, const float* d_img_interp, int T, int h, int w,
                 int magnification, float ring_radius, int border, int positivity, int iw,
                 float* d_out, void* d_ws, size_t ws_bytes, void* stream) {
  if (T < 0 || h < 1 || w < 1) return invalid("bad image shape");
  if (magnification < 1) return invalid("magnification must be >= 1");
  if (!d_ws || ws_bytes < nx_radiality_workspace_bytes(T, h, w)) {
    set_error("workspace too small: need %zu bytes", nx_radiality_workspace_bytes(T, h, w));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const RingCoords rc = ring_coords(magnification, ring_radius);
  cudaError_t e = launch_srrf_fused(d_img, d_img_interp, T, h, w, magnification, rc, ring_radius,
                                    border, positivity ? 1 : 0, iw ? 1 : 0, d_out, s);
  if (e == cudaSuccess) return NX_OK;
  if (e != cudaErrorNotSupported) return cuda_status(e, "Radiality");
  (void)cudaGetLastError();
  float* gx = (float*)d_ws;
  float* gy = gx + (size_t)T * h * w;
  e = launch_gradient_radiality(d_img, T, h, w, gx, gy, s);
  if (e == cudaSuccess)
    e = launch_radiality(gx, gy, d_img_interp, T, h, w, magnification,
                         ring_coords(magnification, ring_radius), border, positivity ? 1 : 0,
                         iw ? 1 : 0, d_out, s);
  if (e != cudaSuccess) return cuda_status(e, "Radiality");
  return NX_OK;
}

int nx_temporal_correlation(const float* d_stack, int T, long long n, int corr, float* d_out,
                            void* stream) {
  if (T < 1 || n < 0) return invalid("bad stack shape");
  if (corr != NX_CORR_AVG && corr != NX_CORR_VAR && corr != NX_CORR_TAC2)
    return invalid("Type of correlation must be AVG, VAR or TAC2");
  cudaError_t e = launch_temporal_stack(d_stack, T, n, corr, d_out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "temporal correlation");
  return NX_OK;
}

int nx_srrf_temporal_correlation(const float* d_stack, int T, long long n, int order,
                                 float* d_out, void* stream) {
  if (T < 1 || n < 0) return invalid("bad stack shape");
  if (order > 4 || order < -1) return invalid("order must be -1, 0, 1, 2, 3 or 4");
  cudaError_t e = launch_srrf_temporal(d_stack, T, n, order, d_out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "SRRF temporal correlation");
  return NX_OK;
}

}  // extern "C"

namespace nx {

// Loop control of the reference's ACRF with lag-time integration
// (sr_temporal_correlations.py:159-200) replayed on the host in its own
// arithmetic: the level count is a Python int (T) at the first level and a
// float (T / order^k) after, compared with integer t; the binning of frame t
// reads frames t*order .. t*order + order-2 when t*order < n_binned.
static int acrf_schedule(int T, int order, AcrfSchedule* sch) {
  memset(sch, 0, sizeof(*sch));
  double nb = (double)T;
  while (nb > (double)order) {
    if (sch->n_levels >= kMaxAcrfLevels) return invalid("too many lag-time levels");
    long long t = 0, n_bin = 0;
    while ((double)t < nb - (double)order) {
      if ((double)(t * order) < nb) {
        if (t * order + order - 2 >= T) {
          set_error("index %lld is out of bounds for axis 0 with size %d", t * order + order - 2,
                    T);
          return NX_ERR_INDEX;
        }
        n_bin = t + 1;
      }
      ++t;
    }
    const int L = sch->n_levels++;
    sch->n_iter[L] = (int)t;
    sch->n_bin[L] = (int)n_bin;
    sch->n_binned[L] = (float)nb;
    nb = nb / (double)order;
  }
  return NX_OK;
}

}  // namespace nx

extern "C" {

size_t nx_srrf_acrf_workspace_bytes(int T, long long n) {
  if (T < 1 || n < 0) return 0;
  return align256((size_t)T * (size_t)n * sizeof(float));
}

int nx_srrf_acrf_integrated(const float* d_stack, int T, long long n, int order, float* d_out,
                            void* d_ws, size_t ws_bytes, void* stream) {
  if (T < 1 || n < 0) return invalid("bad stack shape");
  if (order < 2 || order > 4) return invalid("lag-time integration applies to orders 2, 3 and 4");
  AcrfSchedule sch;
  int rc = acrf_schedule(T, order, &sch);
  if (rc) return rc;
  if (n == 0) return NX_OK;
  if (!d_stack || !d_out) return invalid("NULL stack/output");
  if (!d_ws || ws_bytes < nx_srrf_acrf_workspace_bytes(T, n)) {
    set_error("workspace too small: need %zu bytes", nx_srrf_acrf_workspace_bytes(T, n));
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  float* im = (float*)d_ws;
  NX_CUDA_TRY(cudaMemcpyAsync(im, d_stack, (size_t)T * n * sizeof(float), cudaMemcpyDeviceToDevice,
                              s));
  cudaError_t e = launch_srrf_acrf_integrated(im, T, n, order, sch, d_out, s);
  if (e != cudaSuccess) return cuda_status(e, "ACRF with lag-time integration");
  return NX_OK;
}

int nx_srrf(const float* d_img, int T, int h, int w, int magnification, float ring_radius,
            int border, int positivity, int iw, int mpc, float* d_out, void* d_ws,
            size_t ws_bytes, void* stream) {
  if (T < 0 || h < 1 || w < 1) return invalid("bad image shape");
  if (magnification < 1) return invalid("magnification must be >= 1");
  const size_t need = std::max(nx_radiality_workspace_bytes(T, h, w) +
                                   align256((size_t)T * h * magnification * w * magnification * 4),
                               nx_macro_pixel_workspace_bytes(T, magnification));
  if (!d_ws || ws_bytes < need) {
    set_error("workspace too small: need %zu bytes", need);
    return NX_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const RingCoords rc = ring_coords(magnification, ring_radius);
  cudaError_t e = launch_srrf_fused(d_img, nullptr, T, h, w, magnification, rc, ring_radius,
                                    border, positivity ? 1 : 0, iw ? 1 : 0, d_out, s);
  if (e == cudaErrorNotSupported) {
    (void)cudaGetLastError();
    // general path: magnified intensity, gradients and the per-pixel kernel
    float* mag = (float*)((char*)d_ws + nx_radiality_workspace_bytes(T, h, w));
    float* zeros = (float*)d_ws;  // shift arrays (T zeros) at the start of the workspace
    e = cudaMemsetAsync(zeros, 0, (size_t)std::max(T, 1) * sizeof(float), s);
    if (e == cudaSuccess)
      e = launch_cr_shift_magnify(d_img, T, h, w, zeros, zeros, (float)magnification,
                                  (float)magnification, h * magnification, w * magnification,
                                  mag, s);
    float* gx = (float*)d_ws;
    float* gy = gx + (size_t)T * h * w;
    if (e == cudaSuccess) e = launch_gradient_radiality(d_img, T, h, w, gx, gy, s);
    if (e == cudaSuccess)
      e = launch_radiality(gx, gy, mag, T, h, w, magnification, rc, border, positivity ? 1 : 0,
                           iw ? 1 : 0, d_out, s);
  }
  if (e != cudaSuccess) return cuda_status(e, "SRRF");
  if (mpc) {
    e = launch_mpc(d_out, T, h * magnification, w * magnification, magnification, (float*)d_ws,
                   s);
    if (e != cudaSuccess) return cuda_status(e, "SRRF macro-pixel correction");
  }
  return NX_OK;
}

size_t nx_srrf_workspace_bytes(int T, int h, int w, int magnification) {
  return std::max(nx_radiality_workspace_bytes(T, h, w) +
                      align256((size_t)T * h * magnification * w * magnification * 4),
                  nx_macro_pixel_workspace_bytes(T, magnification));
}

size_t nx_macro_pixel_workspace_bytes(int S, int magnification) {
  return align256((size_t)std::max(S, 1) * magnification * magnification * kMpcChunks *
                  sizeof(float));
}

int nx_macro_pixel_correct(float* d_img, int S, int rowsM, int colsM, int magnification,
                           void* d_ws, size_t ws_bytes, void* stream) {
  if (S < 0 || rowsM < 0 || colsM < 0) return invalid("bad image shape");
  if (magnification < 1) return invalid("magnification must be >= 1");
  if (!d_ws || ws_bytes < nx_macro_pixel_workspace_bytes(S, magnification)) {
    set_error("workspace too small");
    return NX_ERR_WORKSPACE;
  }
  cudaError_t e = launch_mpc(d_img, S, rowsM, colsM, magnification, (float*)d_ws,
                             (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "macro-pixel correction");
  return NX_OK;
}

}  // extern "C"
