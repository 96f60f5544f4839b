// Macro-pixel correction for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc -- nor any allocating
// routine, a framework's caching allocator included -- once they are running:
// a microscope acquisition loop that reserves all of its memory at start-up and
// then reconstructs frames under a fixed real-time budget, or a host
// application whose own allocator owns the GPU and hands this library nothing
// but finished image buffers.  nx_macro_pixel_correct() needs a scratch
// workspace from its caller; nx_macro_pixel_correct_static() below does the
// same correction with its scratch (the per-slice phase maps) in a fixed
// device array owned by the library, so the caller passes only the images.
//
// * The array holds kStaticScratchBytes = 256 KiB.  A call needs
//   max(S,1) * m^2 * min(64, max(1, rowsM / m)) floats of it (the per-slice,
//   per-phase partial sums of the map); one that needs more is rejected with
//   NX_ERR_INVALID_ARG and a message naming the limit, and nothing is launched.
//   For images of at least 64 macro-pixel rows that is S * m^2 <= 1024.
// * Host code cannot use the array's name as a device address.  The first call
//   on each device looks the address up with cudaGetSymbolAddress (with that
//   device current) and caches it.  With lazy module loading (the default of
//   CUDA 12.2 and later) that first call is also what loads this library's
//   kernels on the device and reserves the array there, so it can fail with
//   an out-of-memory error: make it once at start-up, before the phase that
//   must not allocate and before any stream capture.  Under eager loading the
//   array is reserved when the library's module loads.
// * The cached address belongs to the device's context: do not use this entry
//   point again after resetting that device (cudaDeviceReset) in the same
//   process.
// * All calls on a device share the array, which keeps the previous call's
//   contents.  The map kernel writes every entry the apply kernel then reads,
//   so nothing has to be cleared, but calls that overlap on the GPU (two
//   streams at once) race on the array and must be serialised by the caller.
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace {

constexpr size_t kStaticScratchBytes = 256 * 1024;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_mpc_static_scratch[kStaticScratchBytes];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

int static_scratch_address(void** out) {
  int dev = -1;
  NX_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    nx::set_error("device index %d out of range for the static scratch table", dev);
    return NX_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    NX_CUDA_TRY(cudaGetSymbolAddress(&p, g_mpc_static_scratch));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return NX_OK;
}

}  // namespace

extern "C" int nx_macro_pixel_correct_static(float* d_img, int S, int rowsM, int colsM,
                                             int magnification, void* stream) {
  if (!d_img && (long long)S * rowsM * colsM > 0) {
    nx::set_error("NULL image");
    return NX_ERR_INVALID_ARG;
  }
  if (S < 0 || rowsM < 0 || colsM < 0 || magnification < 1) {
    nx::set_error("bad image shape or magnification");
    return NX_ERR_INVALID_ARG;
  }
  const size_t need = nx::mpc_scratch_bytes(S, rowsM, magnification);
  if (need > kStaticScratchBytes) {
    nx::set_error(
        "macro-pixel correction of %d slices at magnification %d needs %zu bytes of scratch; "
        "the static scratch holds %zu bytes (use nx_macro_pixel_correct with a workspace)",
        S, magnification, need, kStaticScratchBytes);
    return NX_ERR_INVALID_ARG;
  }
  void* scratch = nullptr;
  int rc = static_scratch_address(&scratch);
  if (rc) return rc;
  cudaError_t e = nx::launch_mpc(d_img, S, rowsM, colsM, magnification,
                                 static_cast<float*>(scratch), (cudaStream_t)stream);
  if (e != cudaSuccess) return nx::cuda_status(e, "macro-pixel correction (static scratch)");
  return NX_OK;
}
