// api.cu -- host library behind include/mexct.h.
//
// Argument checking, the per-device context (stream, grow-only workspaces),
// per-view geometry tables, view chunking and the host<->device boundary of
// the MEX-equivalent entry points.  All compute runs in the kernels of
// k_proj.cu / k_iter.cu; there is no CPU fallback.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mexct.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;

namespace {
thread_local std::string g_err;
std::mutex g_default_mu;
mexct_ctx* g_default[64] = {nullptr};
}  // namespace

namespace mexct {

mexct_status set_err(mexct_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

mexct_status cuda_err(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation)
    return set_err(MEXCT_ERR_OOM, "%s: out of device memory", what);
  return set_err(MEXCT_ERR_CUDA, "%s: CUDA error %d (%s)", what, (int)e,
                 cudaGetErrorString(e));
}

void Buf::release() {
  if (p) {
    // Memory from cudaMallocAsync is freed in the order of its stream, after
    // the work queued there (cudaFree would not wait for it).
    if (is_async) cudaFreeAsync(p, ast);
    else cudaFree(p);
  }
  p = nullptr;
  n = 0;
  ast = nullptr;
  is_async = false;
}

void Buf::release_synced() {
  if (p && is_async) {
    cudaDeviceSynchronize();
    cudaFreeAsync(p, cudaStreamLegacy);
    cudaStreamSynchronize(cudaStreamLegacy);
    p = nullptr;
    n = 0;
    ast = nullptr;
    is_async = false;
    cudaGetLastError();
    return;
  }
  release();
}

cudaError_t Buf::ensure_async(size_t bytes, cudaStream_t st) {
  if (bytes <= n && p) return cudaSuccess;
  if (p && is_async && ast != st) {
    // The old block was allocated on another stream, which may be a caller's
    // stream that no longer exists.  Outside a stream capture it is freed
    // after the device has finished all its work; inside a capture (where the
    // device cannot be synchronised) the old stream is taken to be alive and
    // st waits for the work queued on it.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
      cudaGetLastError();
      cs = cudaStreamCaptureStatusNone;
    }
    if (cs == cudaStreamCaptureStatusNone) {
      release_synced();
    } else {
      cudaEvent_t ev = nullptr;
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess) {
        cudaEventRecord(ev, ast);
        cudaStreamWaitEvent(st, ev, 0);
        cudaEventDestroy(ev);
      }
      ast = st;
    }
  }
  release();
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(&p, bytes, st);
  if (e != cudaSuccess) {
    p = nullptr;
    n = 0;
    cudaGetLastError();
    return e;
  }
  n = bytes;
  ast = st;
  is_async = true;
  return cudaSuccess;
}

cudaError_t Buf::ensure(size_t bytes) {
  if (bytes <= n && p) return cudaSuccess;
  release();
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    p = nullptr;
    n = 0;
    cudaGetLastError();
    return e;
  }
  n = bytes;
  return cudaSuccess;
}

void trig_of(float beta, Trig* t) {
  // Correctly rounded binary32 sin/cos of the binary32 angle (the reference
  // calls host sincosf, CUDAmex_FP.cu:449).
  t->s = (float)std::sin((double)beta);
  t->c = (float)std::cos((double)beta);
}

mexct_ctx* resolve(mexct_ctx* ctx) {
  if (ctx) return ctx;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default[dev]) {
    mexct_ctx* c = nullptr;
    if (mexct_ctx_create(dev, &c) != MEXCT_OK) return nullptr;
    g_default[dev] = c;
  }
  return g_default[dev];
}

// Counter / partials / scalars for the FP64 reductions.
cudaError_t ensure_reduction(mexct_ctx* c, size_t nparts) {
  cudaError_t e = c->red.ensure(sizeof(double) * (nparts + 8));
  if (e != cudaSuccess) return e;
  if (!c->cnt.p) {
    e = c->cnt.ensure(64);
    if (e != cudaSuccess) return e;
    e = cudaMemset(c->cnt.p, 0, 64);
    if (e != cudaSuccess) return e;
  }
  return c->scal.ensure(64);
}

void fill_std_rays(RayArgs& a, int W, int H, float sad, int geom,
                   bool osc) {
  std::memset(&a, 0, sizeof a);
  a.det_w = W;
  a.det_h = H;
  a.S = W;
  a.Z = H;
  a.u0 = float(W - 1) / 2;          // CUDAmex_FP.cu:378-379
  a.v0 = float(H - 1) / 2;
  a.bx = -(float)W / 2.0f;          // :424-426
  a.by = -(float)W / 2.0f;
  a.bz = -(float)H / 2.0f;
  a.SR = sad;
  a.RD = sad;
  // Step: voxel/2 for par and fan, voxel/1 for cone (CUDAmex_FP.cu:133,231,
  // 328); voxel/2 for every geometry inside OSC (CUDAmex_oscIter.cu:244).
  a.step = (geom == 2 && !osc) ? 1.0f : 0.5f;
  a.P = (long long)W * H;
  a.vstride = 1;
  a.du = 1.0f;                      // the reference's detector: unit pitch,
  a.dv = 1.0f;                      // rays through the pixel centres
}

void fill_vox(VoxArgs& a, int W, int H, float sad) {
  std::memset(&a, 0, sizeof a);
  a.W = W;
  a.H = H;
  a.v0 = float(H - 1) / 2;          // CUDAmex_BP.cu:249
  a.SR = sad;
  a.hw = (uint32_t)W / 2u - 1u;     // :73
  a.P = (long long)W * H;
  a.det_w = W;                      // the volume's face, unit pitch
  a.det_h = H;
  a.hwd = (float)a.hw;
  a.v0d = a.v0;
  a.inv_du = 1.0f;
  a.inv_dv = 1.0f;
  a.zoff = 0;                       // the whole volume, every detector row
  a.nzs = H;
  a.row0 = 0;
  a.nrows = H;
}

}  // namespace mexct

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* mexct_last_error(void) { return g_err.c_str(); }
const char* mexct_version(void) { return "mexct-gb300 0.1 (sm_103a)"; }

mexct_status mexct_ctx_create(int device, mexct_ctx** out) {
  if (!out) return set_err(MEXCT_ERR_ARG, "ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return cuda_err(e, "ctx_create");
  if (device < 0 || device >= ndev)
    return set_err(MEXCT_ERR_ARG, "ctx_create: device %d of %d", device, ndev);
  int prev = 0;
  cudaGetDevice(&prev);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_err(e, "ctx_create: set device");
  mexct_ctx* c = new mexct_ctx();
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    delete c;
    return cuda_err(e, "ctx_create: stream");
  }
  *out = c;
  return MEXCT_OK;
}

mexct_status mexct_ctx_trim(mexct_ctx* c) {
  if (!c) return set_err(MEXCT_ERR_ARG, "ctx_trim: NULL context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaStreamSynchronize(c->stream);
  // Workspaces may have been allocated on caller streams that are gone by now.
  for (Buf* b : c->all_bufs()) b->release_synced();
  if (c->tex) {
    cudaDestroyTextureObject(c->tex);
    c->tex = 0;
  }
  if (c->tex_arr) {
    cudaFreeArray(c->tex_arr);
    c->tex_arr = nullptr;
  }
  return MEXCT_OK;
}

mexct_status mexct_ctx_set_wait_limit(mexct_ctx* ctx, int us) {
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "set_wait_limit: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  c->wait_us = us < 0 ? 0 : (us == 0 ? -1 : us);
  return MEXCT_OK;
}

mexct_status mexct_ctx_device_errors(mexct_ctx* ctx, unsigned* flags, int clear) {
  if (!flags) return set_err(MEXCT_ERR_ARG, "device_errors: flags is NULL");
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "device_errors: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  *flags = 0;
  if (!c->err.p) return MEXCT_OK;  // no slab launch yet
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  cudaError_t e = cudaMemcpy(flags, c->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && clear) e = cudaMemset(c->err.p, 0, sizeof(unsigned));
  cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_err(e, "device_errors");
  return MEXCT_OK;
}

mexct_status mexct_ctx_destroy(mexct_ctx* c) {
  if (!c) return MEXCT_OK;
  {
    std::lock_guard<std::mutex> lk(g_default_mu);
    for (auto& d : g_default)
      if (d == c) d = nullptr;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  mexct_ctx_trim(c);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    for (cudaEvent_t ev : c->chunk_ev)
      if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : c->feed_ev)
      if (ev) cudaEventDestroy(ev);
    cudaStreamDestroy(c->copy_stream);
  }
  cudaStreamDestroy(c->stream);
  cudaSetDevice(prev);
  delete c;
  return MEXCT_OK;
}

}  // extern "C"
