// Internal host-side launch interfaces shared by the C-ABI translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "esrrf_fused.cuh"

namespace nx {

// ---------------------------------------------------------------------------
// fused eSRRF instantiations: one table entry per (M, J)
// ---------------------------------------------------------------------------
using FusedLaunchFn = cudaError_t (*)(const UnitTable&, const TmapPack&, int, cudaStream_t);
using FusedOccupancyFn = int (*)(int ns_cap);
using FusedSmemFn = size_t (*)(int ns_cap);
struct FusedEntry {
  FusedLaunchFn launch[3];       // indexed by FusedMode
  FusedOccupancyFn occupancy[3]; // resident CTAs per SM (0: does not fit)
  FusedSmemFn smem[3];           // dynamic shared memory bytes
  FusedGeometry geo;
};
// variant 0: the default tiling; 1: one producer warp group fewer (m = 2, 4, 5)
constexpr int kTileVariants = 2;
const FusedEntry* fused_entry(int M, int J, int variant = 0);  // nullptr if not instantiated
const FusedEntry* fused_entry_m1(int J);
const FusedEntry* fused_entry_m2(int J);
const FusedEntry* fused_entry_m3(int J);
const FusedEntry* fused_entry_m4(int J);
const FusedEntry* fused_entry_m5(int J);
const FusedEntry* fused_entry_m6(int J);
const FusedEntry* fused_entry_m8(int J);
const FusedEntry* fused_entry_m2_alt(int J);
const FusedEntry* fused_entry_m4_alt(int J);
const FusedEntry* fused_entry_m5_alt(int J);

// ---------------------------------------------------------------------------
// standalone op launchers (ops.cu)
// ---------------------------------------------------------------------------
cudaError_t launch_cr_shift_magnify(const float* in, int T, int H, int W, const float* shift_r,
                                    const float* shift_c, float mag_r, float mag_c, int rowsM,
                                    int colsM, float* out, cudaStream_t s);
cudaError_t launch_roberts_cross(const float* in, int T, int H, int W, float* gc, float* gr,
                                 cudaStream_t s);

struct RgcScalars {
  float tSS, tSO;
  int start, end;  // window [start, end) on the half-pixel grid
  int margin;
  int sens_mode, sens_int;
  float sens;
};
RgcScalars rgc_scalars(int M, float radius, float sensitivity, int pad_edges);

cudaError_t launch_rgc(const float* gc, const float* gr, const float* img, int T, int rowsM,
                       int colsM, int M, const RgcScalars& sc, int iw, float* out,
                       cudaStream_t s);
cudaError_t launch_gradient_radiality(const float* in, int T, int h, int w, float* gx, float* gy,
                                      cudaStream_t s);
struct RingCoords {
  float x[12], y[12];
  float radius;
};
RingCoords ring_coords(int M, float ring_radius);
cudaError_t launch_radiality(const float* gx, const float* gy, const float* img_interp, int T,
                             int h, int w, int M, const RingCoords& rc, int border, int positivity,
                             int iw, float* out, cudaStream_t s);
// fused tile kernel (srrf_fused.cu); img_interp may be nullptr (intensity computed
// in the kernel); cudaErrorNotSupported when (M, ring radius) is not covered
cudaError_t launch_srrf_fused(const float* in, const float* img_interp, int T, int h, int w,
                              int M, const RingCoords& rc, float ring_radius, int border,
                              int positivity, int iw, float* out, cudaStream_t s);

// temporal records: fields mean, M2, C, A, B of Moments (planes of n_pixels)
cudaError_t launch_record_push_frame(const float* frame, long long n, float* rec, int it,
                                     cudaStream_t s);
cudaError_t launch_record_merge(float* acc, const float* blk, long long n, int n_acc, int n_blk,
                                cudaStream_t s);
// combine `nchunks` consecutive records (each F planes) of one timepoint with frame
// counts derived from nf, and write the correlations of corr_mask to out[ci*out_stride]
// one temporal finalisation of a batch: the chunk records of one timepoint
// (rec, F fields, nchunks chunks over nf frames, n pixels) -> the output
// planes at out (out_stride apart), VAR/TAC2/AVG per corr_mask, or the mean
// only (!full); block0 = the job's first block in the launch
struct FinalizeJob {
  const float* rec;
  float* out;
  long long n, out_stride;
  int F, nchunks, nf, corr_mask, full, block0;
};
// every job of a list in one launch (total_blocks = the last job's block0 +
// its blocks)
cudaError_t launch_finalize_jobs(const FinalizeJob* jobs, int njobs, int total_blocks,
                                 cudaStream_t s);
cudaError_t launch_finalize(const float* rec, int F, int nchunks, int nf, long long n,
                            int corr_mask, float* out, long long out_stride, bool full,
                            cudaStream_t s);
cudaError_t launch_temporal_stack(const float* stack, int T, long long n, int corr, float* out,
                                  cudaStream_t s);
cudaError_t launch_srrf_temporal(const float* stack, int T, long long n, int order, float* out,
                                 cudaStream_t s);
// ACRF with lag-time integration: per level, iterations over t, re-binned
// frames (a prefix of t) and the divisor (float32 of the reference's count)
constexpr int kMaxAcrfLevels = 48;
struct AcrfSchedule {
  int n_levels;
  int n_iter[kMaxAcrfLevels];
  int n_bin[kMaxAcrfLevels];
  float n_binned[kMaxAcrfLevels];
};
// im: a (T, n) working copy of the stack, re-binned in place
cudaError_t launch_srrf_acrf_integrated(float* im, int T, long long n, int order,
                                        const AcrfSchedule& sch, float* out, cudaStream_t s);
// macro-pixel correction of S images in place; the scratch it uses is
// mpc_scratch_bytes(S, rowsM, M) = max(S,1) * M^2 * min(kMpcChunks, max(1, rowsM/M))
// floats, never more than nx_macro_pixel_workspace_bytes(S, M)
constexpr int kMpcChunks = 64;
size_t mpc_scratch_bytes(int S, int rowsM, int M);
cudaError_t launch_mpc(float* img, int S, int rowsM, int colsM, int M, float* map,
                       cudaStream_t s);

}  // namespace nx
