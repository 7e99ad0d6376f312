// noalloc.cu -- TV descent that allocates no device memory.
//
// mexct_tvmin3d_dev_noalloc computes the same thing as mexct_tvmin3d_dev, but
// its scratch (the second volume of the ping-pong pair, the FP64 per-CTA
// partial sums of ||g||^2, the reduction counter and the step scale) lives in
// one fixed array compiled into this library instead of a context workspace.
// It is meant for callers that must not allocate device memory while they
// run: a serving loop that reserved its whole HBM budget at start-up (a
// cudaMalloc/cudaFree on the request path can synchronise the device and
// stall every other stream), or a host application whose GPU memory is held by
// another allocator (MATLAB's gpuArray pool, for one) so that nothing is left
// for a second one.  The caller passes the input and output volumes.
//
// Limits and rules (also in include/mexct.h):
//   - at most kMaxVoxels = 2^21 voxels (e.g. 128^3) per call, and at most
//     kMaxPartials per-CTA partial sums; larger requests are rejected;
//   - the array is about 8.5 MiB and every GPU that loads the library keeps
//     it until the process exits;
//   - all calls share the array, so calls that overlap on the GPU (different
//     streams, or different host threads, without ordering) race;
//   - every call looks up the array's device address (cudaGetSymbolAddress)
//     with the caller's device current, so the address always belongs to the
//     current context (after cudaDeviceReset, or with another context current
//     on the device, a cached one would not); the first call on a device
//     also loads the library's device code there, so make that first call
//     before any stream capture.
#include <cstdint>

#include "../../include/mexct.h"
#include "api_internal.h"
#include "kernels.h"

namespace {

constexpr size_t kMaxVoxels = size_t(1) << 21;  // 2,097,152 voxels, e.g. 128^3
constexpr size_t kMaxPartials = 65536;          // FP64 partial sums (512 KiB)
constexpr size_t kOffPart = kMaxVoxels * sizeof(float);
constexpr size_t kOffCnt = kOffPart + kMaxPartials * sizeof(double);
constexpr size_t kOffScal = kOffCnt + 256;
constexpr size_t kScratchBytes = kOffScal + 256;

// The scratch itself.  In host code this name is only a host-side stand-in:
// the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_tv_noalloc_scratch[kScratchBytes];

}  // namespace

extern "C" mexct_status mexct_tvmin3d_dev_noalloc(const float* d_vol, int Nx,
                                                  int Ny, int Nz, float cval,
                                                  int n_steps, float* d_out,
                                                  void* stream) {
  using namespace mexct;
  if (!d_vol || !d_out) return set_err(MEXCT_ERR_ARG, "tvmin3d_noalloc: NULL pointer");
  if (Nx <= 0 || Ny <= 0 || Nz <= 0) return set_err(MEXCT_ERR_ARG, "tvmin3d_noalloc: bad dims");
  if (n_steps < 0) return set_err(MEXCT_ERR_ARG, "tvmin3d_noalloc: n_steps < 0");
  const size_t N = (size_t)Nx * Ny * Nz;
  if (N > kMaxVoxels)
    return set_err(MEXCT_ERR_UNSUPPORTED,
                   "tvmin3d_noalloc: %d x %d x %d = %zu voxels exceeds the fixed scratch "
                   "limit of %zu voxels; use mexct_tvmin3d_dev",
                   Nx, Ny, Nz, N, kMaxVoxels);
  if (!tv_shape_launchable(Nx, Ny, Nz))
    return set_err(MEXCT_ERR_UNSUPPORTED,
                   "tvmin3d_noalloc: %d x %d x %d exceeds the launch grid limits (at most "
                   "65535 tiles of %d rows in y and of %d slices in z)",
                   Nx, Ny, Nz, 15, 32);
  const size_t parts = tv_partials_needed(Nx, Ny, Nz);
  if (parts > kMaxPartials)
    return set_err(MEXCT_ERR_UNSUPPORTED,
                   "tvmin3d_noalloc: shape %d x %d x %d needs %zu reduction partials, "
                   "the fixed scratch holds %zu",
                   Nx, Ny, Nz, parts, kMaxPartials);
  void* addr = nullptr;
  MEXCT_TRY_CUDA(cudaGetSymbolAddress(&addr, g_tv_noalloc_scratch),
                 "tvmin3d_noalloc: scratch address");
  unsigned char* base = static_cast<unsigned char*>(addr);
  float* pong = reinterpret_cast<float*>(base);
  double* partials = reinterpret_cast<double*>(base + kOffPart);
  unsigned* counter = reinterpret_cast<unsigned*>(base + kOffCnt);
  float* scale = reinterpret_cast<float*>(base + kOffScal);
  double* norm = reinterpret_cast<double*>(base + kOffScal + 8);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t bytes = N * sizeof(float);
  if (n_steps == 0) {
    if (d_vol != d_out)
      MEXCT_TRY_CUDA(cudaMemcpyAsync(d_out, d_vol, bytes, cudaMemcpyDeviceToDevice, st),
                     "tvmin3d_noalloc: copy");
    return MEXCT_OK;
  }
  // The reduction counter must start at zero; an earlier call that failed
  // half-way could have left it set.
  MEXCT_TRY_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), st), "tvmin3d_noalloc: clear");
  const void* src = d_vol;
  if (d_vol == d_out && (n_steps % 2) == 1) {
    // In place with an odd step count: the first step would write its input.
    MEXCT_TRY_CUDA(cudaMemcpyAsync(pong, d_vol, bytes, cudaMemcpyDeviceToDevice, st),
                   "tvmin3d_noalloc: copy");
    src = pong;
  }
  for (int k = 0; k < n_steps; ++k) {
    void* dst = ((n_steps - 1 - k) % 2 == 0) ? static_cast<void*>(d_out) : static_cast<void*>(pong);
    MEXCT_TRY_CUDA(launch_tv_norm(src, kF32, Nx, Ny, Nz, cval, partials, counter, scale, norm, st),
                   "tvmin3d_noalloc: norm");
    MEXCT_TRY_CUDA(launch_tv_update(src, dst, kF32, Nx, Ny, Nz, scale, st),
                   "tvmin3d_noalloc: update");
    src = dst;
  }
  return MEXCT_OK;
}
