// tune.cu -- launch-shape table and autotuner of the FP / BP entry points
// (include/mexct.h, "launch shapes and autotuning").
//
// A context maps each shape class (operator, geometry, W, H, view count
// rounded up to a power of two, storage types) to a launch shape.  Without a
// table entry the context's mode decides: the fixed shape, a heuristic that
// splits the views of small volumes into blocks so the grid fills the GPU, or
// (MEXCT_TUNE_AUTO) timing every candidate on the first call's own buffers.
// Candidates never change the arithmetic of a sample; view blocks only change
// the order of the FP32 sums (block partial sums added in block order).
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "../../include/mexct.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;

namespace {

constexpr int kTuneViewsBp = 256;  // views timed per BP candidate
constexpr int kTuneViewsFp = 64;   // views timed per FP candidate
constexpr size_t kMaxPartialBytes = size_t(2) << 30;

int pow2_ceil(int n) {
  int p = 1;
  while (p < n && p < (1 << 30)) p <<= 1;
  return p;
}

TuneKey key_of(int op, int geom, int W, int H, int nP, int it, int ot) {
  return TuneKey{op, geom, W, H, pow2_ceil(std::max(nP, 1)), it, ot};
}

int sm_count(int dev) {
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  return n > 0 ? n : 1;
}

mexct_shape fixed_shape() { return mexct_shape{MEXCT_FP_EXPLICIT, 16, 8, 1}; }

// View blocks until the grid covers every SM about 4 times (4 CTAs of 256
// threads stay resident per SM), keeping >= 16 views per block and the
// partial sums below 1 GiB; 4-row blocks for grids that need no view blocks.
mexct_shape heuristic_bp(int dev, int W, int H, int nP) {
  mexct_shape s = fixed_shape();
  const long long ctas = (long long)((W + 31) / 32) * ((W + 7) / 8) * ((H + 15) / 16);
  const long long want = 4ll * sm_count(dev);
  const size_t N = (size_t)W * W * H;
  int vb = 1;
  while (vb < 64 && ctas * vb < want && nP / (2 * vb) >= 16 &&
         N * 2 * vb * sizeof(float) <= (size_t(1) << 30))
    vb *= 2;
  s.vblocks = vb;
  // blocks of 32 x 4 columns once the grid is large enough: 3% faster than
  // 32 x 8 at 512^3 x 720 cone with the quad-layout views (66.3 vs 68.2 ms)
  if (vb == 1 && 2 * ctas >= 8ll * sm_count(dev)) s.rows = 4;
  return s;
}

mexct_shape default_shape(const mexct_ctx* c, int op, int W, int H, int nP) {
  if (op == MEXCT_OP_BP && c->tune_mode != MEXCT_TUNE_FIXED)
    return heuristic_bp(c->device, W, H, nP);
  return fixed_shape();
}

bool capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
    cudaGetLastError();
    return true;  // unknown: do not time
  }
  return cs != cudaStreamCaptureStatusNone;
}

// Best of the timed runs of fn() on st after one untimed run, in ms.  Short
// calls are repeated inside each timed run (about 2 ms of work per run) so
// launch jitter does not pick the shape.
template <typename F>
mexct_status time_on(cudaStream_t st, int reps, F&& fn, double* ms) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  MEXCT_TRY_CUDA(cudaEventCreate(&e0), "autotune: event");
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_err(ce, "autotune: event");
  }
  double best = std::numeric_limits<double>::infinity();
  int inner = 1;
  mexct_status s = MEXCT_OK;
  for (int r = -1; r < reps && s == MEXCT_OK; ++r) {  // r = -1: warm-up and sizing
    cudaEventRecord(e0, st);
    for (int i = 0; i < inner && s == MEXCT_OK; ++i) s = fn();
    cudaEventRecord(e1, st);
    ce = cudaEventSynchronize(e1);
    if (ce != cudaSuccess) {
      s = cuda_err(ce, "autotune: timing");
      break;
    }
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (r < 0) {
      inner = (int)std::min(20.0, std::max(1.0, std::ceil(2.0 / std::max((double)t, 1e-3))));
      continue;
    }
    best = std::min(best, (double)t / inner);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = best;
  return s;
}

std::vector<mexct_shape> bp_candidates(int W, int H, int nt) {
  std::vector<mexct_shape> out;
  const size_t N = (size_t)W * W * H;
  for (int zc : {16, 8})
    for (int rows : {8, 4})
      for (int vb = 1; vb <= 64; vb *= 2) {
        if (vb > 1 && (nt / vb < 8 || N * vb * sizeof(float) > kMaxPartialBytes)) break;
        out.push_back(mexct_shape{MEXCT_FP_EXPLICIT, zc, rows, vb});
      }
  return out;
}

// Time every BP candidate on the first min(nP, kTuneViewsBp) views.
mexct_status tune_bp(mexct_ctx* c, const void* d_sino, int stype, int W, int H, int nP,
                     float sad, const float* angles, int geom, void* d_vol, int vt,
                     cudaStream_t st, mexct_shape* best, double* best_ms) {
  const int nt = std::min(nP, kTuneViewsBp);
  *best = fixed_shape();
  *best_ms = std::numeric_limits<double>::infinity();
  for (const mexct_shape& cand : bp_candidates(W, H, nt)) {
    const BpShape b{cand.zc, cand.rows, cand.vblocks};
    double ms = 0;
    mexct_status s = time_on(st, 3, [&] {
      return bp_run(c, d_sino, stype, W, H, nt, sad, angles, geom, d_vol, vt, b, st);
    }, &ms);
    if (s == MEXCT_ERR_OOM) continue;  // workspace of a large view split: skip it
    if (s) return s;
    if (ms < *best_ms) {
      *best_ms = ms;
      *best = cand;
    }
  }
  return MEXCT_OK;
}

mexct_status tune_fp(mexct_ctx* c, const void* d_vol, int vt, int W, int H, float sad,
                     const float* angles, int nP, int geom, void* d_out, int ot,
                     cudaStream_t st, mexct_shape* best, double* best_ms) {
  const int nt = std::min(nP, kTuneViewsFp);
  *best = fixed_shape();
  *best_ms = std::numeric_limits<double>::infinity();
  for (int variant : {MEXCT_FP_EXPLICIT, MEXCT_FP_RAY}) {
    double ms = 0;
    mexct_status s = time_on(st, 3, [&] {
      return fp_run(c, d_vol, vt, W, H, sad, angles, nt, geom, d_out, ot, variant, st);
    }, &ms);
    if (s) return s;
    if (ms < *best_ms) {
      *best_ms = ms;
      *best = fixed_shape();
      best->variant = variant;
    }
  }
  return MEXCT_OK;
}

bool bad_op_args(int op, int geom, int W, int H, int nP, int it, int ot) {
  auto bad_t = [](int t) { return t != MEXCT_F32 && t != MEXCT_F16 && t != MEXCT_BF16; };
  return (op != MEXCT_OP_FP && op != MEXCT_OP_BP) || geom < 0 || geom > 2 || W <= 0 || H <= 0 ||
         nP < 0 || bad_t(it) || bad_t(ot);
}

}  // namespace

namespace mexct {

mexct_status pick_bp_shape(mexct_ctx* c, const void* d_sino, int stype, int W, int H, int nP,
                           float sad, const float* angles, int geom, void* d_vol, int vt,
                           cudaStream_t st, mexct_shape* out) {
  const TuneKey k = key_of(MEXCT_OP_BP, geom, W, H, nP, stype, vt);
  auto it = c->tune.find(k);
  if (it != c->tune.end()) {
    *out = it->second.shape;
    return MEXCT_OK;
  }
  if (c->tune_mode == MEXCT_TUNE_AUTO && !capturing(st)) {
    double ms = 0;
    mexct_status s = tune_bp(c, d_sino, stype, W, H, nP, sad, angles, geom, d_vol, vt, st, out,
                             &ms);
    if (s) return s;
    c->tune[k] = TuneEntry{*out, ms, 1};
    return MEXCT_OK;
  }
  *out = default_shape(c, MEXCT_OP_BP, W, H, nP);
  return MEXCT_OK;
}

mexct_status pick_fp_shape(mexct_ctx* c, const void* d_vol, int vt, int W, int H, float sad,
                           const float* angles, int nP, int geom, void* d_out, int ot,
                           cudaStream_t st, mexct_shape* out) {
  const TuneKey k = key_of(MEXCT_OP_FP, geom, W, H, nP, vt, ot);
  auto it = c->tune.find(k);
  if (it != c->tune.end()) {
    *out = it->second.shape;
    return MEXCT_OK;
  }
  if (c->tune_mode == MEXCT_TUNE_AUTO && !capturing(st)) {
    double ms = 0;
    mexct_status s = tune_fp(c, d_vol, vt, W, H, sad, angles, nP, geom, d_out, ot, st, out, &ms);
    if (s) return s;
    c->tune[k] = TuneEntry{*out, ms, 1};
    return MEXCT_OK;
  }
  *out = default_shape(c, MEXCT_OP_FP, W, H, nP);
  return MEXCT_OK;
}

}  // namespace mexct

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

mexct_status mexct_ctx_set_tune_mode(mexct_ctx* ctx, int mode) {
  if (mode != MEXCT_TUNE_FIXED && mode != MEXCT_TUNE_HEURISTIC && mode != MEXCT_TUNE_AUTO)
    return set_err(MEXCT_ERR_ARG, "set_tune_mode: unknown mode %d", mode);
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "set_tune_mode: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  c->tune_mode = mode;
  return MEXCT_OK;
}

mexct_status mexct_shape_set(mexct_ctx* ctx, int op, int geom, int W, int H, int nP,
                             int in_type, int out_type, const mexct_shape* shape) {
  if (!shape) return set_err(MEXCT_ERR_ARG, "shape_set: shape is NULL");
  if (bad_op_args(op, geom, W, H, nP, in_type, out_type))
    return set_err(MEXCT_ERR_ARG, "shape_set: bad shape class");
  if (op == MEXCT_OP_FP && shape->variant != MEXCT_FP_EXPLICIT && shape->variant != MEXCT_FP_RAY)
    return set_err(MEXCT_ERR_ARG, "shape_set: FP variant must be EXPLICIT or RAY");
  if (op == MEXCT_OP_BP && !bp_shape_valid(BpShape{shape->zc, shape->rows, shape->vblocks}))
    return set_err(MEXCT_ERR_ARG, "shape_set: BP needs zc 8/16, rows 4/8, vblocks 1..64");
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "shape_set: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  c->tune[key_of(op, geom, W, H, nP, in_type, out_type)] =
      TuneEntry{*shape, std::numeric_limits<double>::quiet_NaN(), 0};
  return MEXCT_OK;
}

mexct_status mexct_shape_get(mexct_ctx* ctx, int op, int geom, int W, int H, int nP,
                             int in_type, int out_type, mexct_shape* shape, double* ms,
                             int* tuned) {
  if (!shape) return set_err(MEXCT_ERR_ARG, "shape_get: shape is NULL");
  if (bad_op_args(op, geom, W, H, nP, in_type, out_type))
    return set_err(MEXCT_ERR_ARG, "shape_get: bad shape class");
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "shape_get: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  auto it = c->tune.find(key_of(op, geom, W, H, nP, in_type, out_type));
  if (it != c->tune.end()) {
    *shape = it->second.shape;
    if (ms) *ms = it->second.ms;
    if (tuned) *tuned = it->second.tuned;
  } else {
    *shape = default_shape(c, op, W, H, nP);
    if (ms) *ms = std::numeric_limits<double>::quiet_NaN();
    if (tuned) *tuned = -1;
  }
  return MEXCT_OK;
}

mexct_status mexct_shape_clear(mexct_ctx* ctx) {
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "shape_clear: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  c->tune.clear();
  return MEXCT_OK;
}

mexct_status mexct_autotune_bp(mexct_ctx* ctx, const void* d_sino, int stype, int W, int H,
                               int nP, float sad, const float* angles, int geom, void* d_vol,
                               int vt, void* stream, mexct_shape* best, double* best_ms) {
  if (!d_sino || !d_vol || !angles) return set_err(MEXCT_ERR_ARG, "autotune_bp: NULL pointer");
  if (bad_op_args(MEXCT_OP_BP, geom, W, H, nP, stype, vt) || nP == 0 || W > 16384 || H > 16384)
    return set_err(MEXCT_ERR_ARG, "autotune_bp: bad arguments");
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "autotune_bp: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  DevGuard dg(c->device);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  if (capturing(st)) return set_err(MEXCT_ERR_ARG, "autotune_bp: stream is capturing");
  mexct_shape b;
  double ms = 0;
  mexct_status s = tune_bp(c, d_sino, stype, W, H, nP, sad, angles, geom, d_vol, vt, st, &b, &ms);
  if (s) return s;
  c->tune[key_of(MEXCT_OP_BP, geom, W, H, nP, stype, vt)] = TuneEntry{b, ms, 1};
  s = bp_run(c, d_sino, stype, W, H, nP, sad, angles, geom, d_vol, vt,
             BpShape{b.zc, b.rows, b.vblocks}, st);
  if (s) return s;
  if (best) *best = b;
  if (best_ms) *best_ms = ms;
  return MEXCT_OK;
}

mexct_status mexct_autotune_fp(mexct_ctx* ctx, const void* d_vol, int vt, int W, int H,
                               float sad, const float* angles, int nP, int geom, void* d_out,
                               int ot, void* stream, mexct_shape* best, double* best_ms) {
  if (!d_vol || !d_out || !angles) return set_err(MEXCT_ERR_ARG, "autotune_fp: NULL pointer");
  if (bad_op_args(MEXCT_OP_FP, geom, W, H, nP, vt, ot) || nP == 0 || W > 16384 || H > 16384)
    return set_err(MEXCT_ERR_ARG, "autotune_fp: bad arguments");
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "autotune_fp: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  DevGuard dg(c->device);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  if (capturing(st)) return set_err(MEXCT_ERR_ARG, "autotune_fp: stream is capturing");
  mexct_shape b;
  double ms = 0;
  mexct_status s = tune_fp(c, d_vol, vt, W, H, sad, angles, nP, geom, d_out, ot, st, &b, &ms);
  if (s) return s;
  c->tune[key_of(MEXCT_OP_FP, geom, W, H, nP, vt, ot)] = TuneEntry{b, ms, 1};
  s = fp_run(c, d_vol, vt, W, H, sad, angles, nP, geom, d_out, ot, b.variant, st);
  if (s) return s;
  if (best) *best = b;
  if (best_ms) *best_ms = ms;
  return MEXCT_OK;
}

}  // extern "C"
