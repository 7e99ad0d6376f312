// api_internal.h -- context and helpers shared by the host translation units.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <initializer_list>
#include <functional>
#include <map>
#include <mutex>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/mexct.h"
#include "kernels.h"

namespace mexct {

// Grow-only device buffer.
struct Buf {
  void* p = nullptr;
  size_t n = 0;
  // Stream-ordered allocation: the stream it was allocated on (may be the
  // legacy default stream, handle 0) and whether it was.  Such memory must be
  // released with cudaFreeAsync: cudaFree does not wait for queued work.
  cudaStream_t ast = nullptr;
  bool is_async = false;
  cudaError_t ensure(size_t bytes);
  // Stream-ordered allocation (cudaMallocAsync): no device-wide
  // synchronisation on allocation or release, so work on other streams keeps
  // running.  The buffer is released with cudaFreeAsync on the same stream.
  cudaError_t ensure_async(size_t bytes, cudaStream_t st);
  // Free in the order of the stream the block was allocated on (that stream
  // must still exist: the owner's own stream).
  void release();
  // Free after all work on the device has finished, whatever stream the block
  // was allocated on: for context workspaces, whose allocation stream may be
  // a caller's stream that no longer exists.  Synchronises the device.
  void release_synced();
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// NVTX range over one library call ("mexct:fp", ...), visible in Nsight
// timelines; costs nothing when no tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// One entry of a context's launch-shape table.
struct TuneEntry {
  mexct_shape shape;
  double ms;   // time of the tuned shape on its tuning call (NaN if not tuned)
  int tuned;   // 1: chosen by timing, 0: set by the caller
};
// Shape class: operator, geometry, W, H, view count rounded up to a power of
// two, input and output storage types.
using TuneKey = std::array<int, 7>;

}  // namespace mexct

struct mexct_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;     // stream of the host entry points
  // Output copies of the host entry points, overlapped with the launches
  // still running on `stream` (created on first use), and one event per chunk.
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t chunk_ev[8] = {};
  cudaEvent_t feed_ev[4] = {};  // uploads of the host BP's view parts
  std::recursive_mutex mu;           // serialises calls on this context
  // Host entry points: staged inputs / outputs.
  mexct::Buf in, in2, in3, out;
  // Device entry points: transposed volume, subset residuals / TV ping-pong,
  // filter tables, FP64 reduction partials, counter and scalars.
  mexct::Buf volT, r1, r2, r3, tabs, red, cnt, scal;
  // Padded volumes of the slab FP (x-fastest and y-fastest) and the device
  // error word of bounded waits.
  mexct::Buf padx, pady, err;
  mexct::Buf spad;   // padded sinogram views for BP
  mexct::Buf bpart;  // BP view-block partial sums
  mexct::Buf subs;   // one sub-ray sinogram of a super-sampled FP
  // Launch shapes: MEXCT_TUNE_* mode and the per-class table.
  int tune_mode = MEXCT_TUNE_HEURISTIC;
  // Limit of one bounded wait in the slab FP (SlabEpi::wait_us encoding).
  int wait_us = 0;
  std::map<mexct::TuneKey, mexct::TuneEntry> tune;
  // Texture variant: cached 3D array + texture object.
  cudaArray_t tex_arr = nullptr;
  cudaTextureObject_t tex = 0;
  int tex_w = 0, tex_h = 0;
  // Pre-filter kernel cache.
  int filt_w = -1, filt_type = -1;
  float filt_cut = -1.f;
  std::vector<float> filt_kern;
  // The pre-filter tables in `tabs` (kernel, Parker weights, dbeta) and the
  // arguments they were built for: a call with the same scan geometry reuses
  // them (tab_buf: tabs.p when they were written; a trim or a reallocation
  // invalidates them).
  struct TabKey {
    int W = -1, H = -1, nP = -1, geom = -1, filter = -1;
    float sad = 0.f, cutoff = 0.f, q = 0.f;
    std::vector<float> angles;
    bool operator==(const TabKey& o) const {
      return W == o.W && H == o.H && nP == o.nP && geom == o.geom && filter == o.filter &&
             sad == o.sad && cutoff == o.cutoff && q == o.q && angles == o.angles;
    }
  } tab_key;
  const void* tab_buf = nullptr;

  std::vector<mexct::Buf*> all_bufs() {
    return {&in, &in2, &in3, &out, &volT, &r1, &r2, &r3, &tabs, &red, &cnt, &scal,
            &padx, &pady, &err, &spad, &bpart, &subs};
  }
};

namespace mexct {

mexct_status set_err(mexct_status code, const char* fmt, ...);
mexct_status cuda_err(cudaError_t e, const char* what);
void trig_of(float beta, Trig* t);
mexct_ctx* resolve(mexct_ctx* ctx);
cudaError_t ensure_reduction(mexct_ctx* c, size_t nparts);
void fill_std_rays(RayArgs& a, int W, int H, float sad, int geom, bool osc);
void fill_vox(VoxArgs& a, int W, int H, float sad);

// Scoped device switch to the context's device.
struct DevGuard {
  int prev = -1;
  explicit DevGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DevGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

inline size_t dsize(int t) { return t == kF32 ? 4 : 2; }

mexct_status prepare_slab_bufs(Buf& px, Buf& py, Buf& err, const void* d_vol, int vt, int W,
                               int H, bool border, int geom, CUtensorMap* mx, CUtensorMap* my,
                               int* Pf_out, cudaStream_t st);
mexct_status osc_tv_recon_typed(mexct_ctx* ctx, const float* pre, const float* post, int W, int H,
                                int nP, const float* angles, float sad, int geom, int n_iter,
                                float tv_const, int n_sub_init, int n_sub_final, float p_val,
                                const int32_t* first_picks, int mu_type, float* recon,
                                int data_type = 0);
mexct_status prepare_slab(mexct_ctx* c, const void* d_vol, int vt, int W, int H,
                          bool border, int geom, CUtensorMap* mx, CUtensorMap* my, int* Pf_out,
                          cudaStream_t st);

// Called after the launch of each chunk of an FP (views first .. first +
// count - 1) or BP (slices first .. first + count - 1) split into `chunks`
// launches; the results of each launch are bit-identical to the unsplit one.
struct ChunkHook {
  int chunks;
  std::function<mexct_status(int index, int first, int count)> fn;
};

// The context's copy stream and its events (created on first use): host <->
// device copies that overlap the launches on the context's stream.
cudaError_t copy_stream(mexct_ctx* c, cudaStream_t* out);

// FP with a concrete variant / BP with an explicit launch shape (arguments
// already checked; ops.cu).
mexct_status fp_run(mexct_ctx* c, const void* d_vol, int vt, int W, int H, float sad,
                    const float* angles, int nP, int geom, void* d_out, int ot, int variant,
                    cudaStream_t st, const ChunkHook* hook = nullptr);
// feed (BP, one view chunk and one view block): the views
// arrive in feed->chunks parts; feed->fn(i, first, count) is called before the
// work on views first .. first + count - 1 and makes `st` wait for them.  Each
// part's launch continues the stored sums, so the result is bit-identical to
// one launch; `hook` then splits the last part's launch by z.
mexct_status bp_run(mexct_ctx* c, const void* d_sino, int stype, int W, int H, int nP, float sad,
                    const float* angles, int geom, void* d_vol, int vt, const BpShape& shp,
                    cudaStream_t st, const ChunkHook* hook = nullptr,
                    const ChunkHook* feed = nullptr);
// Shape of a call's class from the context's table, its mode's default, or
// (MEXCT_TUNE_AUTO, outside stream capture) by timing the candidates on the
// call's own buffers (tune.cu).
mexct_status pick_fp_shape(mexct_ctx* c, const void* d_vol, int vt, int W, int H, float sad,
                           const float* angles, int nP, int geom, void* d_out, int ot,
                           cudaStream_t st, mexct_shape* out);
mexct_status pick_bp_shape(mexct_ctx* c, const void* d_sino, int stype, int W, int H, int nP,
                           float sad, const float* angles, int geom, void* d_vol, int vt,
                           cudaStream_t st, mexct_shape* out);
}  // namespace mexct

#define MEXCT_TRY_CUDA(expr, what)                         \
  do {                                                     \
    cudaError_t _e = (expr);                               \
    if (_e != cudaSuccess) return ::mexct::cuda_err(_e, what); \
  } while (0)
