// Sub-volume (z-slab) FP / BP and the out-of-core FP / BP drivers.
//
// No counterpart in the reference, whose oscIter keeps three whole volumes on
// the device and lists sub-volume reconstruction of larger images as a TODO
// (iterative_reconstruction/CUDAmex_oscIter.cu:28-29).  A z-slab is slices
// z0 .. z0 + nz - 1 of a W x W x H volume.
//  - FP is linear in the volume: the FP of a slab is the FP of the volume with
//    every other slice zero (the clamp frame kept at the volume's own faces),
//    and the FPs of the slabs add up to the FP of the volume.
//  - BP is voxel-driven: a slab's voxels need only the detector rows their
//    columns project onto (mexct_sub_rows), and each voxel gets exactly the
//    operations of the whole-volume BP (one view block).
// The drivers stream a host volume (FP) or a host sinogram's row bands (BP)
// through the device within a byte budget.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "../../include/mexct.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;

namespace {

#define SUB_CTX(c, name)                                                    \
  NvtxRange _nvtx("mexct:" name);                                           \
  mexct_ctx* c = resolve(ctx);                                              \
  if (!c) return set_err(MEXCT_ERR_CUDA, name ": no CUDA device / context"); \
  std::lock_guard<std::recursive_mutex> _lk(c->mu);                         \
  DevGuard _dg(c->device)

bool bad_wh(int W, int H) { return W <= 0 || H <= 0 || W > 16384 || H > 16384; }

// Bytes per padded texel of the BP's quad layout (FP32 views).
constexpr size_t kLayBytes = sizeof(float4);

// Detector rows the BP of slab [z0, z0 + nz) reads, with one row of margin
// each side (cone): pz(z) = (z - v0) U + v0 + 0.5 with U = SR / (SR - s) and
// |s| <= R.  BP reaches only the columns inside the circle of radius
// hw = W/2 - 1 about texel (hw, hw) (CUDAmex_BP.cu:73-76), whose centres
// (ix - hw - 0.5, iy - hw - 0.5) lie within hw + 0.71 of the axis; R = W/2 + 1
// bounds them with margin.
void rows_of(int W, int H, float sad, int geom, int z0, int nz, int* row0, int* nrows) {
  if (geom < 2) {
    *row0 = z0;
    *nrows = nz;
    return;
  }
  const double R = W / 2.0 + 1.0;
  const double SR = sad;
  if (!(SR > R)) {  // the source is inside the volume's cylinder: every row
    *row0 = 0;
    *nrows = H;
    return;
  }
  const double v0 = (H - 1) / 2.0;
  const double Us[2] = {SR / (SR + R), SR / (SR - R)};
  const double zs[2] = {(double)z0, (double)(z0 + nz - 1)};
  double lo = 1e300, hi = -1e300;
  for (double U : Us)
    for (double z : zs) {
      const double pz = (z - v0) * U + v0 + 0.5;
      lo = std::min(lo, pz);
      hi = std::max(hi, pz);
    }
  // taps floor(pz - 0.5) and +1, one row of margin for FP32 rounding
  long long r0 = (long long)std::floor(lo - 0.5) - 1;
  long long r1 = (long long)std::floor(hi - 0.5) + 2;
  r0 = std::max(0LL, std::min(r0, (long long)H - 1));
  r1 = std::max(r0, std::min(r1, (long long)H - 1));
  *row0 = (int)r0;
  *nrows = (int)(r1 - r0 + 1);
}

mexct_status check_slab(const char* op, int W, int H, int z0, int nz, int nP, int geom) {
  if (bad_wh(W, H)) return set_err(MEXCT_ERR_ARG, "%s: bad volume dims %d x %d x %d", op, W, W, H);
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "%s: bad view count %d", op, nP);
  if (geom < 0 || geom > 2) return set_err(MEXCT_ERR_ARG, "%s: invalid geometry %d", op, geom);
  if (z0 < 0 || nz < 1 || z0 + (long long)nz > H)
    return set_err(MEXCT_ERR_ARG, "%s: slab z0 %d, nz %d outside 0..%d", op, z0, nz, H);
  return MEXCT_OK;
}

// FP of slab [z0, z0 + nz) (device slab W x W x nz) into the W x H x nP
// sinogram: stores, or adds to it with accumulate.
mexct_status fp_sub_impl(mexct_ctx* c, const float* d_slab, int W, int H, int z0, int nz,
                         float sad, const float* angles, int nP, int geom, float* d_sino,
                         bool accumulate, cudaStream_t st) {
  if (mexct_status s = check_slab("fp_sub", W, H, z0, nz, nP, geom)) return s;
  if (!d_slab || (nP > 0 && (!d_sino || !angles)))
    return set_err(MEXCT_ERR_ARG, "fp_sub: NULL pointer");
  if (!c || nP == 0) return MEXCT_OK;
  std::unique_ptr<RayArgs> a(new RayArgs);
  fill_std_rays(*a, W, H, sad, geom, false);
  // padded rows z0 .. z0 + nz + 1 of the whole volume's padded frame; the
  // rows that are not zero: the slab's slices, and a frame row at a face of
  // the volume (clamp copy)
  const int rlo = z0 + 1 - (z0 == 0 ? 1 : 0);
  const int rhi = z0 + nz + (z0 + nz == H ? 1 : 0);
  a->zoff = z0;
  a->zrows = nz + 2;
  a->zlo = (float)(rlo - 1);
  a->zhi = (float)(rhi + 1);
  a->accum = accumulate ? 1 : 0;
  const int Pf = slab_pitch(W);
  const size_t bytes = (size_t)Pf * (W + 2) * (nz + 2) * sizeof(float);
  MEXCT_TRY_CUDA(c->padx.ensure_async(bytes, st), "fp_sub: workspace");
  MEXCT_TRY_CUDA(c->pady.ensure_async(bytes, st), "fp_sub: workspace");
  if (!c->err.p) {
    MEXCT_TRY_CUDA(c->err.ensure(64), "fp_sub: workspace");
    MEXCT_TRY_CUDA(cudaMemset(c->err.p, 0, 64), "fp_sub: workspace");
  }
  MEXCT_TRY_CUDA(launch_pad_volume_sub(d_slab, W, nz, Pf, z0 > 0, z0 + nz < H,
                                       c->padx.as<float>(), c->pady.as<float>(), st),
                 "fp_sub: pad");
  CUtensorMap mx, my;
  MEXCT_TRY_CUDA(make_slab_tmap(&mx, c->padx.p, kF32, Pf, W + 2, nz + 2, geom), "fp_sub: tensor map");
  MEXCT_TRY_CUDA(make_slab_tmap(&my, c->pady.p, kF32, Pf, W + 2, nz + 2, geom), "fp_sub: tensor map");
  SlabEpi e{nullptr, nullptr, nullptr, nullptr, c->err.as<unsigned>(), c->wait_us};
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    a->nviews = std::min(kMaxViews, nP - v0);
    a->view0 = v0;
    for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
    MEXCT_TRY_CUDA(launch_fp_slab_sub(geom, *a, mx, my, c->padx.p, c->pady.p, Pf, d_sino, e, st),
                   "fp_sub: launch");
  }
  return MEXCT_OK;
}

// BP into slab [z0, z0 + nz) from detector rows [row0, row0 + nrows) of every
// view (device array W x nrows x nP), laying out and back-projecting at most
// pad_views views per launch (0: kMaxViews).  Each launch continues the
// stored sums, so the chunking leaves the result bit for bit unchanged.
mexct_status bp_sub_impl(mexct_ctx* c, const float* d_rows, int row0, int nrows, int W, int H,
                         int nP, float sad, const float* angles, int geom, int z0, int nz,
                         float* d_slab, bool accumulate, cudaStream_t st, int pad_views = 0) {
  if (mexct_status s = check_slab("bp_sub", W, H, z0, nz, nP, geom)) return s;
  if (!d_slab || (nP > 0 && (!d_rows || !angles)))
    return set_err(MEXCT_ERR_ARG, "bp_sub: NULL pointer");
  int need0, needn;
  rows_of(W, H, sad, geom, z0, nz, &need0, &needn);
  if (row0 < 0 || nrows < 1 || row0 + (long long)nrows > H || row0 > need0 ||
      row0 + nrows < need0 + needn)
    return set_err(MEXCT_ERR_ARG,
                   "bp_sub: rows %d..%d do not hold rows %d..%d that slab %d..%d reads", row0,
                   row0 + nrows - 1, need0, need0 + needn - 1, z0, z0 + nz - 1);
  if (!c) return MEXCT_OK;
  const long long Ns = (long long)W * W * nz;
  if (nP == 0) {
    if (!accumulate) MEXCT_TRY_CUDA(launch_fill(d_slab, kF32, Ns, 0.f, st), "bp_sub: zero");
    return MEXCT_OK;
  }
  std::unique_ptr<VoxArgs> a(new VoxArgs);
  fill_vox(*a, W, H, sad);
  a->zoff = z0;
  a->nzs = nz;
  a->row0 = row0;
  a->nrows = nrows;
  const int chunk = std::min(nP, pad_views > 0 ? std::min(pad_views, kMaxViews) : kMaxViews);
  MEXCT_TRY_CUDA(c->spad.ensure_async(sino_pad_elems(W, nrows, chunk) * kLayBytes, st),
                 "bp_sub: workspace");
  const size_t Pr = (size_t)W * nrows;
  for (int v0 = 0; v0 < nP; v0 += chunk) {
    a->nviews = std::min(chunk, nP - v0);
    a->view0 = 0;
    for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
    const float* rows = d_rows + (size_t)v0 * Pr;
    MEXCT_TRY_CUDA(launch_pad_sino_quad(rows, kF32, W, nrows, a->nviews, c->spad.p, st),
                   "bp_sub: pad");
    MEXCT_TRY_CUDA(launch_bp_sub(geom, *a, c->spad.p, d_slab, accumulate || v0 > 0, st),
                   "bp_sub: launch");
  }
  return MEXCT_OK;
}

// Device bytes of one FP slab of nz slices (slab + two padded layouts).
size_t fp_slab_bytes(int W, int nz) {
  return (size_t)W * W * nz * 4 + 2 * (size_t)slab_pitch(W) * (W + 2) * (nz + 2) * 4;
}

// Views laid out per BP launch of the out-of-core driver: the layout holds a
// few views while the raw rows hold them all.
constexpr int kOocPadViews = 32;

// Device bytes of a BP step: slab of nz slices, nv views of nr rows and the
// layout of up to kOocPadViews of them.
size_t bp_step_bytes(int W, int nz, int nr, int nv, int geom) {
  return (size_t)W * W * nz * 4 + (size_t)W * nr * nv * 4 +
         sino_pad_elems(W, nr, std::min(nv, kOocPadViews)) * kLayBytes;
}

// Widest row band over the slabs z0 = 0, nz, 2 nz, ... (the bands of the end
// slabs are cut by the detector's edges, so any slab can be the widest).
int bp_rows_max(int W, int H, float sad, int geom, int nz) {
  int m = 0;
  for (int z0 = 0; z0 < H; z0 += nz) {
    int r0, nr;
    rows_of(W, H, sad, geom, z0, std::min(nz, H - z0), &r0, &nr);
    m = std::max(m, nr);
  }
  return m;
}

}  // namespace

extern "C" {

mexct_status mexct_sub_rows(int W, int H, float sad, int geom, int z0, int nz, int* row0,
                            int* nrows) {
  if (mexct_status s = check_slab("sub_rows", W, H, z0, nz, 0, geom)) return s;
  if (!row0 || !nrows) return set_err(MEXCT_ERR_ARG, "sub_rows: NULL pointer");
  rows_of(W, H, sad, geom, z0, nz, row0, nrows);
  return MEXCT_OK;
}

mexct_status mexct_fp_sub_dev(mexct_ctx* ctx, const float* d_slab, int W, int H, int z0, int nz,
                              float sad, const float* angles, int nP, int geom, float* d_sino,
                              int accumulate, void* stream) {
  if (mexct_status s = fp_sub_impl(nullptr, d_slab, W, H, z0, nz, sad, angles, nP, geom, d_sino,
                                   accumulate != 0, nullptr))
    return s;
  SUB_CTX(c, "fp_sub");
  return fp_sub_impl(c, d_slab, W, H, z0, nz, sad, angles, nP, geom, d_sino, accumulate != 0,
                     static_cast<cudaStream_t>(stream));
}

mexct_status mexct_bp_sub_dev(mexct_ctx* ctx, const float* d_rows, int row0, int nrows, int W,
                              int H, int nP, float sad, const float* angles, int geom, int z0,
                              int nz, float* d_slab, int accumulate, void* stream) {
  if (mexct_status s = bp_sub_impl(nullptr, d_rows, row0, nrows, W, H, nP, sad, angles, geom,
                                   z0, nz, d_slab, accumulate != 0, nullptr))
    return s;
  SUB_CTX(c, "bp_sub");
  return bp_sub_impl(c, d_rows, row0, nrows, W, H, nP, sad, angles, geom, z0, nz, d_slab,
                     accumulate != 0, static_cast<cudaStream_t>(stream));
}

mexct_status mexct_fp_ooc(mexct_ctx* ctx, const float* vol, int W, int H, float sad,
                          const float* angles, int nP, int geom, size_t budget_bytes,
                          float* sino) {
  if (mexct_status s = check_slab("fp_ooc", W, H, 0, H, nP, geom)) return s;
  if (!vol || (nP > 0 && (!sino || !angles))) return set_err(MEXCT_ERR_ARG, "fp_ooc: NULL pointer");
  if (nP == 0) return MEXCT_OK;
  // views per pass: half the budget for the sinogram chunk; the rest for slabs
  const size_t view_bytes = (size_t)W * H * 4;
  int nv = (int)std::min<size_t>((size_t)nP, budget_bytes / 2 / view_bytes);
  if (nv < 1) nv = 1;
  const size_t left = budget_bytes > nv * view_bytes ? budget_bytes - nv * view_bytes : 0;
  // the thickest slab that fits with a second slab buffer for the next
  // upload (bytes grow linearly with nz)
  auto step_bytes = [&](int z) { return fp_slab_bytes(W, z) + (size_t)W * W * z * 4; };
  int nz = H;
  if (step_bytes(nz) > left) {
    const size_t b1 = step_bytes(1), per = step_bytes(2) - b1;
    nz = left >= b1 ? (int)std::min<size_t>((size_t)H, 1 + (left - b1) / per) : 1;
  }
  if (step_bytes(nz) > left)
    return set_err(MEXCT_ERR_BUDGET, "fp_ooc: %zu bytes hold no view and slab of %d x %d",
                   budget_bytes, W, W);
  SUB_CTX(c, "fp_ooc");
  cudaStream_t st = c->stream, cs;
  MEXCT_TRY_CUDA(copy_stream(c, &cs), "fp_ooc: copy stream");
  const size_t slab_bytes = (size_t)W * W * nz * 4;
  MEXCT_TRY_CUDA(c->in.ensure_async(2 * slab_bytes, st), "fp_ooc: workspace");
  MEXCT_TRY_CUDA(c->out.ensure_async((size_t)nv * view_bytes, st), "fp_ooc: workspace");
  // Two slab buffers: slab i uploads on the copy stream into buffer i & 1
  // once the FP that last read it has run, while the FP of slab i - 1 runs.
  cudaEvent_t landed[2] = {c->feed_ev[0], c->feed_ev[1]};
  cudaEvent_t freed[2] = {c->feed_ev[2], c->feed_ev[3]};
  for (cudaEvent_t e : freed) MEXCT_TRY_CUDA(cudaEventRecord(e, st), "fp_ooc: event");
  int slab = 0;
  for (int v0 = 0; v0 < nP; v0 += nv) {
    const int n = std::min(nv, nP - v0);
    for (int z0 = 0; z0 < H; z0 += nz, ++slab) {
      const int m = std::min(nz, H - z0), b = slab & 1;
      float* buf = c->in.as<float>() + (size_t)b * W * W * nz;
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(cs, freed[b], 0), "fp_ooc: event");
      MEXCT_TRY_CUDA(cudaMemcpyAsync(buf, vol + (size_t)z0 * W * W, (size_t)W * W * m * 4,
                                     cudaMemcpyHostToDevice, cs),
                     "fp_ooc: upload");
      MEXCT_TRY_CUDA(cudaEventRecord(landed[b], cs), "fp_ooc: event");
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(st, landed[b], 0), "fp_ooc: event");
      mexct_status s = fp_sub_impl(c, buf, W, H, z0, m, sad, angles + v0, n, geom,
                                   c->out.as<float>(), z0 > 0, st);
      if (s) return s;
      MEXCT_TRY_CUDA(cudaEventRecord(freed[b], st), "fp_ooc: event");
    }
    MEXCT_TRY_CUDA(cudaMemcpyAsync(sino + (size_t)v0 * W * H, c->out.p, (size_t)n * view_bytes,
                                   cudaMemcpyDeviceToHost, st),
                   "fp_ooc: download");
  }
  MEXCT_TRY_CUDA(cudaStreamSynchronize(st), "fp_ooc: sync");
  MEXCT_TRY_CUDA(cudaStreamSynchronize(cs), "fp_ooc: sync");
  return MEXCT_OK;
}

mexct_status mexct_bp_ooc(mexct_ctx* ctx, const float* sino, int W, int H, int nP, float sad,
                          const float* angles, int geom, size_t budget_bytes, float* vol) {
  if (mexct_status s = check_slab("bp_ooc", W, H, 0, H, nP, geom)) return s;
  if (!vol || (nP > 0 && (!sino || !angles))) return set_err(MEXCT_ERR_ARG, "bp_ooc: NULL pointer");
  // the largest slab, then the most views, that fit the budget
  int nv = std::max(1, std::min(nP, kMaxViews));
  int nz = H;
  for (;;) {
    // the thickest slab that fits: bisect (the bytes grow with nz)
    if (bp_step_bytes(W, nz, bp_rows_max(W, H, sad, geom, nz), nv, geom) > budget_bytes) {
      int lo = 1, hi = H;  // invariant: hi does not fit
      while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (bp_step_bytes(W, mid, bp_rows_max(W, H, sad, geom, mid), nv, geom) <= budget_bytes) lo = mid;
        else hi = mid;
      }
      nz = lo;
    }
    if (bp_step_bytes(W, nz, bp_rows_max(W, H, sad, geom, nz), nv, geom) <= budget_bytes) break;
    if (nv == 1)
      return set_err(MEXCT_ERR_BUDGET, "bp_ooc: %zu bytes hold no slab of %d x %d", budget_bytes,
                     W, W);
    nv = (nv + 1) / 2;
    nz = H;
  }
  SUB_CTX(c, "bp_ooc");
  cudaStream_t st = c->stream;
  const int nrmax = bp_rows_max(W, H, sad, geom, nz);
  MEXCT_TRY_CUDA(c->in.ensure_async((size_t)W * nrmax * std::max(nv, 1) * 4, st),
                 "bp_ooc: workspace");
  MEXCT_TRY_CUDA(c->out.ensure_async((size_t)W * W * nz * 4, st), "bp_ooc: workspace");
  for (int z0 = 0; z0 < H; z0 += nz) {
    const int m = std::min(nz, H - z0);
    int r0, nr;
    rows_of(W, H, sad, geom, z0, m, &r0, &nr);
    if (nP == 0) {
      MEXCT_TRY_CUDA(launch_fill(c->out.p, kF32, (long long)W * W * m, 0.f, st), "bp_ooc: zero");
    }
    for (int v0 = 0; v0 < nP; v0 += nv) {
      const int n = std::min(nv, nP - v0);
      // rows r0 .. r0 + nr - 1 of views v0 .. v0 + n - 1: one strided copy
      MEXCT_TRY_CUDA(cudaMemcpy2DAsync(c->in.p, (size_t)W * nr * 4,
                                       sino + ((size_t)v0 * H + r0) * W, (size_t)W * H * 4,
                                       (size_t)W * nr * 4, n, cudaMemcpyHostToDevice, st),
                     "bp_ooc: upload");
      mexct_status s = bp_sub_impl(c, c->in.as<float>(), r0, nr, W, H, n, sad, angles + v0, geom,
                                   z0, m, c->out.as<float>(), v0 > 0, st, kOocPadViews);
      if (s) return s;
    }
    MEXCT_TRY_CUDA(cudaMemcpyAsync(vol + (size_t)z0 * W * W, c->out.p, (size_t)W * W * m * 4,
                                   cudaMemcpyDeviceToHost, st),
                   "bp_ooc: download");
  }
  MEXCT_TRY_CUDA(cudaStreamSynchronize(st), "bp_ooc: sync");
  return MEXCT_OK;
}

}  // extern "C"
