// solver_ooc.cu -- OSC-TV over z-slabs with mu in host memory (out of core).
//
// The reference keeps mu, the subset's FP and both residual volumes on the
// device and lists reconstruction of images larger than the device as a TODO
// (iterative_reconstruction/CUDAmex_oscIter.cu:28-29).  Here mu lives in host
// memory (two pinned volumes used in turn) and streams through the device one
// z-slab at a time, within a device-memory budget.  An iteration of
// OSC_TV_recon.m:43-74 becomes a fixed sequence of slab sweeps; in each, slab
// i uploads on a copy stream while slab i - 1 computes and slab i - 2
// downloads on another:
//
//   sweep 0        FP of subset 0: every slab adds its part into the subset's
//                  line integrals (the FP is linear in the volume; with
//                  border addressing the other slabs' slices read as zeros);
//                  then the residual views of the subset
//   sweep s=1..n   dual BP + update of subset s-1 on the slab (voxel-driven:
//                  the slab and the residual views are all it reads), then
//                  the slab's part of the FP of subset s (s < n), or of
//                  ||mu_old - mu|| (s = n, k > 1)
//   k > 1:         one sweep for ||g(x_0)||, then 20 sweeps; sweep t writes
//                  x_{t+1} = x_t + scale_t g(x_t) (the gradient at slice z
//                  reads slices z-1 .. z+1: one halo slice each side) and sums
//                  ||g(x_{t+1})||^2 one slab behind, over slices whose
//                  neighbours are final (the last two slices of the previous
//                  slab's x_{t+1} are carried on the device); the last sweep
//                  also maps NaN/Inf to 0 (:69-70)
//
// Per voxel the dual BP + update and the TV step are the in-core kernels'
// operations.  What differs from the in-core solver is the order of two
// sums: a subset's line integrals are FP32 sums of the slabs' parts, and the
// FP64 norms are combined slab by slab.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/mexct.h"
#include "../../include/mexct_solver.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;

namespace {

constexpr int kTvSteps = 20;  // CUDAmex_TVmin_3D.cu:221
constexpr int kZc = 4;        // slices per dual-BP thread: slab starts are multiples of it
constexpr size_t kAlign = 256;

size_t al(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

// Device bytes of one slab buffer set for slabs of nz slices.
struct SetLayout {
  size_t x, work, old, total;
};
SetLayout set_layout(int W, int nz) {
  const size_t plane = (size_t)W * W * 4;
  SetLayout L;
  L.x = al((size_t)(nz + 2) * plane);  // the slab, one halo slice each side (TV)
  const size_t y = al((size_t)(nz + 3) * plane);  // x_{t+1}: two carried slices + slab + halo
  const size_t pad = 2 * al((size_t)slab_pitch(W) * (W + 2) * (nz + 2) * 4);  // FP layouts
  L.work = std::max(y, pad);
  L.old = al((size_t)nz * plane);  // mu_old of the slab (||mu_old - mu||)
  L.total = L.x + L.work + L.old;
  return L;
}

// Device bytes that do not depend on the slab thickness: the subset's line
// integrals, counts and residual views, the carried slices, reductions.
size_t fixed_bytes(int W, int H, int nvmax, int nslab_max) {
  const size_t views = (size_t)W * H * nvmax * 4;
  const size_t rq = sino_pad_elems(W, H, nvmax) * sizeof(float4);
  const size_t parts = std::max<size_t>(tv_partials_needed(W, W, H + 3), ssd_partials_needed()) + 8;
  return 3 * al(views) + 2 * al(rq) + al(2 * (size_t)W * W * 4) + al(parts * 8) +
         al((size_t)(nslab_max + 8) * 8) + 4 * kAlign;
}

struct DevBlock {
  void* p = nullptr;
  ~DevBlock() {
    if (p) cudaFree(p);
  }
};
struct HostBlock {
  void* p = nullptr;
  ~HostBlock() {
    if (p) cudaFreeHost(p);
  }
};
struct Streams {
  cudaStream_t st = nullptr, cin = nullptr, cout = nullptr;
  cudaEvent_t landed[2] = {}, done[2] = {}, freed[2] = {};
  cudaEvent_t sweep_end = nullptr, pp_landed = nullptr, resid_done = nullptr;
  ~Streams() {
    for (cudaStream_t s : {st, cin, cout})
      if (s) cudaStreamSynchronize(s);
    for (cudaEvent_t e : {landed[0], landed[1], done[0], done[1], freed[0], freed[1], sweep_end,
                          pp_landed, resid_done})
      if (e) cudaEventDestroy(e);
    for (cudaStream_t s : {st, cin, cout})
      if (s) cudaStreamDestroy(s);
  }
};

// The subset schedule (OSC_TV_recon.m:48-49), its largest subset and the
// thickest slab (the whole volume, or a multiple of 4 slices) whose buffer
// sets fit the budget beside the fixed part.  first_picks may be NULL (the
// schedule's subset counts do not depend on it).
struct OocPlan {
  int nz = 0, nvmax = 1;
  size_t bytes = 0;
  std::vector<int> nsubs;
  std::vector<std::vector<int32_t>> picks;
};
mexct_status ooc_plan(int W, int H, int nP, int geom, int n_iter, int n_sub_init, int n_sub_final,
                      float p_val, const int32_t* first_picks, size_t budget_bytes, OocPlan* pl) {
  if (W <= 0 || H <= 0 || nP <= 0 || W > 16384 || H > 16384 || n_iter < 1)
    return set_err(MEXCT_ERR_ARG, "osc_tv_ooc: bad dims %d x %d x %d / iterations %d", W, H, nP,
                   n_iter);
  if (geom < 0 || geom > 2) return set_err(MEXCT_ERR_ARG, "osc_tv_ooc: invalid geometry %d", geom);
  pl->nsubs.assign(n_iter, 0);
  pl->picks.assign(n_iter, {});
  pl->nvmax = 1;
  for (int k = 1; k <= n_iter; ++k) {
    const int ns = mexct_num_subsets(n_sub_init, n_sub_final, p_val, n_iter, k);
    if (ns <= 0) return set_err(MEXCT_ERR_ARG, "osc_tv_ooc: %d subsets at iteration %d", ns, k);
    if (first_picks) {
      const int first = ((first_picks[k - 1] % ns) + ns) % ns;
      pl->picks[k - 1].resize(ns);
      if (mexct_status e = mexct_subset_order(ns, first, pl->picks[k - 1].data())) return e;
    }
    pl->nsubs[k - 1] = ns;
    pl->nvmax = std::max(pl->nvmax, (nP + ns - 1) / ns);
  }
  if (pl->nvmax > kMaxViews)
    return set_err(MEXCT_ERR_UNSUPPORTED, "osc_tv_ooc: subsets of %d views (max %d)", pl->nvmax,
                   kMaxViews);
  auto need = [&](int nz) {
    const int nslab = (H + nz - 1) / nz;
    return fixed_bytes(W, H, pl->nvmax, nslab) + (nslab > 1 ? 2 : 1) * set_layout(W, nz).total;
  };
  int nz = H;
  if (need(nz) > budget_bytes) {
    nz = 0;
    for (int z = (H - 1) / kZc * kZc; z >= kZc; z -= kZc)
      if (need(z) <= budget_bytes) {
        nz = z;
        break;
      }
    if (nz == 0)
      return set_err(MEXCT_ERR_BUDGET,
                     "osc_tv_ooc: %zu bytes hold no slab of %d x %d x %d beside %d views",
                     budget_bytes, W, W, std::min(kZc, H), pl->nvmax);
  }
  pl->nz = nz;
  pl->bytes = need(nz);
  return MEXCT_OK;
}

}  // namespace

namespace mexct {

mexct_status osc_tv_recon_ooc(mexct_ctx* ctx, const float* pre, const float* post, int W, int H,
                              int nP, const float* angles, float sad, int geom, int n_iter,
                              float tv_const, int n_sub_init, int n_sub_final, float p_val,
                              const int32_t* first_picks, size_t budget_bytes, float* recon,
                              int* slab_planes) {
  if (!pre || !post || !angles || !recon || !first_picks)
    return set_err(MEXCT_ERR_ARG, "osc_tv_ooc: NULL pointer");
  OocPlan pl;
  // arguments first (no device needed), then the plan on the context's device
  // (its reduction buffers are sized by the device's SM count)
  if (mexct_status e = ooc_plan(W, H, nP, geom, n_iter, n_sub_init, n_sub_final, p_val,
                                first_picks, (size_t)-1, &pl))
    return e;
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "osc_tv_ooc: no CUDA device / context");
  NvtxRange nvtx("mexct:osc_tv_ooc");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  DevGuard dg(c->device);
  if (mexct_status e = ooc_plan(W, H, nP, geom, n_iter, n_sub_init, n_sub_final, p_val,
                                first_picks, budget_bytes, &pl))
    return e;
  const int nz = pl.nz, nvmax = pl.nvmax;
  const std::vector<int>& nsubs = pl.nsubs;
  const std::vector<std::vector<int32_t>>& picks = pl.picks;
  if (slab_planes) *slab_planes = nz;
  const int nslab = (H + nz - 1) / nz;
  const int nsets = nslab > 1 ? 2 : 1;

  const size_t plane = (size_t)W * W, N = plane * H, M = (size_t)W * H * nP;
  const size_t P = (size_t)W * H;
  // host: clamped counts (OSC_TV_recon.m:35-37) and two copies of mu
  HostBlock hb;
  MEXCT_TRY_CUDA(cudaHostAlloc(&hb.p, (2 * M + 2 * N) * sizeof(float), cudaHostAllocDefault),
                 "osc_tv_ooc: pinned host memory");
  float* hpre = static_cast<float*>(hb.p);
  float* hpost = hpre + M;
  float* hmu[2] = {hpost + M, hpost + M + N};
  for (size_t i = 0; i < M; ++i) {
    hpre[i] = pre[i] < 1e-6f ? 1e-6f : pre[i];
    hpost[i] = post[i] < 1e-6f ? 1e-6f : post[i];
  }
  for (size_t i = 0; i < N; ++i) hmu[0][i] = 1e-10f;  // OSC_TV_recon.m:33

  // device: one block, carved
  const SetLayout L = set_layout(W, nz);
  const size_t total = pl.bytes;
  DevBlock db;
  MEXCT_TRY_CUDA(cudaMalloc(&db.p, total), "osc_tv_ooc: device memory");
  unsigned char* q = static_cast<unsigned char*>(db.p);
  auto carve = [&](size_t b) {
    unsigned char* r = q;
    q += al(b);
    return r;
  };
  const size_t vb = (size_t)W * H * nvmax * 4;
  float* d_l = reinterpret_cast<float*>(carve(vb));
  float* d_pre = reinterpret_cast<float*>(carve(vb));
  float* d_post = reinterpret_cast<float*>(carve(vb));
  const size_t rqb = sino_pad_elems(W, H, nvmax) * sizeof(float4);
  float* d_rpre = reinterpret_cast<float*>(carve(rqb));
  float* d_rpost = reinterpret_cast<float*>(carve(rqb));
  float* d_carry = reinterpret_cast<float*>(carve(2 * plane * 4));
  const size_t nparts = std::max<size_t>(tv_partials_needed(W, W, H + 3), ssd_partials_needed()) + 8;
  double* d_parts = reinterpret_cast<double*>(carve(nparts * 8));
  double* d_slots = reinterpret_cast<double*>(carve((size_t)(nslab + 8) * 8));
  unsigned* d_cnt = reinterpret_cast<unsigned*>(carve(64));
  double* d_scal = reinterpret_cast<double*>(carve(64));  // [0] d_a, [1] ||g||, [2..3] floats
  float* d_scale = reinterpret_cast<float*>(d_scal + 2);
  float* d_dummy = reinterpret_cast<float*>(d_scal + 3);
  float* X[2];
  float* Wk[2];
  float* OLD[2];
  for (int b = 0; b < nsets; ++b) {
    X[b] = reinterpret_cast<float*>(carve(L.x));
    Wk[b] = reinterpret_cast<float*>(carve(L.work));
    OLD[b] = reinterpret_cast<float*>(carve(L.old));
  }
  if (nsets == 1) {
    X[1] = X[0];
    Wk[1] = Wk[0];
    OLD[1] = OLD[0];
  }
  if ((size_t)(q - static_cast<unsigned char*>(db.p)) > total)
    return set_err(MEXCT_ERR_CUDA, "osc_tv_ooc: internal layout error");
  const int Pf = slab_pitch(W);
  const size_t pad_half = al((size_t)Pf * (W + 2) * (nz + 2) * 4) / 4;  // floats

  Streams S;
  MEXCT_TRY_CUDA(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking), "osc_tv_ooc: stream");
  MEXCT_TRY_CUDA(cudaStreamCreateWithFlags(&S.cin, cudaStreamNonBlocking), "osc_tv_ooc: stream");
  MEXCT_TRY_CUDA(cudaStreamCreateWithFlags(&S.cout, cudaStreamNonBlocking), "osc_tv_ooc: stream");
  for (cudaEvent_t* e : {&S.landed[0], &S.landed[1], &S.done[0], &S.done[1], &S.freed[0],
                         &S.freed[1], &S.sweep_end, &S.pp_landed, &S.resid_done})
    MEXCT_TRY_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "osc_tv_ooc: event");
  cudaStream_t st = S.st;
  // the residual views' zero frame (border addressing) is written once
  MEXCT_TRY_CUDA(cudaMemsetAsync(d_rpre, 0, rqb, st), "osc_tv_ooc: residual");
  MEXCT_TRY_CUDA(cudaMemsetAsync(d_rpost, 0, rqb, st), "osc_tv_ooc: residual");
  MEXCT_TRY_CUDA(cudaMemsetAsync(d_cnt, 0, 64, st), "osc_tv_ooc: counter");
  MEXCT_TRY_CUDA(cudaMemsetAsync(d_scal, 0, 64, st), "osc_tv_ooc: scalars");
  if (!c->err.p) {
    MEXCT_TRY_CUDA(c->err.ensure(64), "osc_tv_ooc: error word");
    MEXCT_TRY_CUDA(cudaMemset(c->err.p, 0, 64), "osc_tv_ooc: error word");
  }
  for (int b = 0; b < 2; ++b) MEXCT_TRY_CUDA(cudaEventRecord(S.freed[b], st), "osc_tv_ooc: event");
  MEXCT_TRY_CUDA(cudaEventRecord(S.resid_done, st), "osc_tv_ooc: event");
  MEXCT_TRY_CUDA(cudaEventRecord(S.sweep_end, S.cout), "osc_tv_ooc: event");

  std::unique_ptr<RayArgs> ra(new RayArgs);
  std::unique_ptr<VoxArgs> va(new VoxArgs);
  std::vector<Trig> trig(nvmax);
  SlabEpi epi{nullptr, nullptr, nullptr, nullptr, c->err.as<unsigned>(), c->wait_us};
  long long gslab = 0;  // slabs processed: buffer set gslab & 1

  // Views of subset sel of ns: sel, sel + ns, ... (CUDAmex_oscIter.cu:181-185).
  auto subset_views = [&](int sel, int ns) { return sel >= nP ? 0 : (nP - 1 - sel) / ns + 1; };
  auto set_trig = [&](int sel, int ns, int nv) {
    for (int i = 0; i < nv; ++i) trig_of(angles[sel + (size_t)i * ns], &trig[i]);
  };
  // counts of the subset's views onto the device (copy stream), once the
  // residual kernel has read the previous subset's
  auto upload_counts = [&](int sel, int ns, int nv) -> mexct_status {
    if (nv == 0) return MEXCT_OK;
    MEXCT_TRY_CUDA(cudaStreamWaitEvent(S.cin, S.resid_done, 0), "osc_tv_ooc: event");
    for (int w = 0; w < 2; ++w) {
      const float* h = (w ? hpost : hpre) + (size_t)sel * P;
      MEXCT_TRY_CUDA(cudaMemcpy2DAsync(w ? d_post : d_pre, P * 4, h, (size_t)ns * P * 4, P * 4, nv,
                                       cudaMemcpyHostToDevice, S.cin),
                     "osc_tv_ooc: counts upload");
    }
    MEXCT_TRY_CUDA(cudaEventRecord(S.pp_landed, S.cin), "osc_tv_ooc: event");
    return MEXCT_OK;
  };
  auto residual = [&](int nv) -> mexct_status {
    if (nv > 0) {
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(st, S.pp_landed, 0), "osc_tv_ooc: event");
      MEXCT_TRY_CUDA(launch_osc_residual(d_l, d_pre, d_post, W, H, nv, d_rpre, d_rpost, st),
                     "osc_tv_ooc: residual");
    }
    MEXCT_TRY_CUDA(cudaEventRecord(S.resid_done, st), "osc_tv_ooc: event");
    return MEXCT_OK;
  };
  // The slab's part of the FP of nv views (trig) into d_l: stores for the
  // first slab, adds for the others.
  auto fp_part = [&](float* px, float* py, int z0, int m, int nv, bool accum) -> mexct_status {
    if (nv == 0) return MEXCT_OK;
    fill_std_rays(*ra, W, H, sad, geom, /*osc=*/true);
    ra->zoff = z0;  // border addressing: the nonzero padded rows are the slab's
    ra->zrows = m + 2;
    ra->zlo = (float)z0;
    ra->zhi = (float)(z0 + m + 1);
    ra->accum = accum ? 1 : 0;
    CUtensorMap mx, my;
    MEXCT_TRY_CUDA(make_slab_tmap(&mx, px, kF32, Pf, W + 2, m + 2, geom), "osc_tv_ooc: tensor map");
    MEXCT_TRY_CUDA(make_slab_tmap(&my, py, kF32, Pf, W + 2, m + 2, geom), "osc_tv_ooc: tensor map");
    for (int v0 = 0; v0 < nv; v0 += kMaxViews) {
      ra->nviews = std::min(kMaxViews, nv - v0);
      ra->view0 = v0;
      for (int i = 0; i < ra->nviews; ++i) ra->trig[i] = trig[v0 + i];
      MEXCT_TRY_CUDA(launch_fp_slab_sub(geom, *ra, mx, my, px, py, Pf, d_l, epi, st),
                     "osc_tv_ooc: fp");
    }
    return MEXCT_OK;
  };
  // Every sweep starts once the previous sweep's downloads have landed (the
  // host volume it reads is final).
  auto begin_sweep = [&]() -> mexct_status {
    MEXCT_TRY_CUDA(cudaEventRecord(S.sweep_end, S.cout), "osc_tv_ooc: event");
    MEXCT_TRY_CUDA(cudaStreamWaitEvent(S.cin, S.sweep_end, 0), "osc_tv_ooc: event");
    return MEXCT_OK;
  };
  // One slab of a sweep: upload (host slices [a, b) of src into X, and with
  // old_src the slab's slices of it into OLD), compute, download (slices
  // [z0, z1) from the returned pointer into dst, if dst).
  struct SlabIo {
    const float* src;
    int a, b;
    const float* old_src;
    float* dst;
  };
  auto run_slab = [&](const SlabIo& io, int z0, int z1, auto&& compute) -> mexct_status {
    const int bs = nsets == 1 ? 0 : (int)(gslab++ & 1);
    MEXCT_TRY_CUDA(cudaStreamWaitEvent(S.cin, S.freed[bs], 0), "osc_tv_ooc: event");
    MEXCT_TRY_CUDA(cudaMemcpyAsync(X[bs], io.src + (size_t)io.a * plane,
                                   (size_t)(io.b - io.a) * plane * 4, cudaMemcpyHostToDevice, S.cin),
                   "osc_tv_ooc: upload");
    if (io.old_src)
      MEXCT_TRY_CUDA(cudaMemcpyAsync(OLD[bs], io.old_src + (size_t)z0 * plane,
                                     (size_t)(z1 - z0) * plane * 4, cudaMemcpyHostToDevice, S.cin),
                     "osc_tv_ooc: upload");
    MEXCT_TRY_CUDA(cudaEventRecord(S.landed[bs], S.cin), "osc_tv_ooc: event");
    MEXCT_TRY_CUDA(cudaStreamWaitEvent(st, S.landed[bs], 0), "osc_tv_ooc: event");
    const float* out = nullptr;
    if (mexct_status e = compute(bs, &out)) return e;
    if (io.dst) {
      MEXCT_TRY_CUDA(cudaEventRecord(S.done[bs], st), "osc_tv_ooc: event");
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(S.cout, S.done[bs], 0), "osc_tv_ooc: event");
      MEXCT_TRY_CUDA(cudaMemcpyAsync(io.dst + (size_t)z0 * plane, out,
                                     (size_t)(z1 - z0) * plane * 4, cudaMemcpyDeviceToHost, S.cout),
                     "osc_tv_ooc: download");
      MEXCT_TRY_CUDA(cudaEventRecord(S.freed[bs], S.cout), "osc_tv_ooc: event");
    } else {
      MEXCT_TRY_CUDA(cudaEventRecord(S.freed[bs], st), "osc_tv_ooc: event");
    }
    return MEXCT_OK;
  };

  int cur = 0;  // hmu[cur]: mu at the start of the iteration
  for (int k = 1; k <= n_iter; ++k) {
    const int ns = nsubs[k - 1];
    const int32_t* pk = picks[k - 1].data();
    const int oth = 1 - cur;
    if (k == 2) {
      // OSC_TV_recon.m:41,62: from iteration 2 on, pre(1) = post(1) = 0
      MEXCT_TRY_CUDA(cudaStreamSynchronize(S.cin), "osc_tv_ooc: sync");
      hpre[0] = 0.f;
      hpost[0] = 0.f;
    }
    // sweep 0: FP of the first subset
    int nv = subset_views(pk[0], ns);
    set_trig(pk[0], ns, nv);
    if (mexct_status e = upload_counts(pk[0], ns, nv)) return e;
    if (mexct_status e = begin_sweep()) return e;
    for (int i = 0, z0 = 0; z0 < H; ++i, z0 += nz) {
      const int z1 = std::min(H, z0 + nz), m = z1 - z0;
      SlabIo io{hmu[cur], z0, z1, nullptr, nullptr};
      mexct_status e = run_slab(io, z0, z1, [&](int bs, const float**) -> mexct_status {
        float* px = Wk[bs];
        float* py = Wk[bs] + pad_half;
        MEXCT_TRY_CUDA(launch_pad_volume_sub(X[bs], W, m, Pf, false, false, px, py, st, true),
                       "osc_tv_ooc: pad");
        return fp_part(px, py, z0, m, nv, i > 0);
      });
      if (e) return e;
    }
    if (mexct_status e = residual(nv)) return e;
    // sweeps 1..ns: dual BP + update of subset s-1, FP of subset s
    for (int s = 1; s <= ns; ++s) {
      const int nvu = nv;  // views of the subset being applied
      std::vector<Trig> tu(trig.begin(), trig.begin() + nvu);
      const bool last = s == ns;
      int nvn = 0;
      if (!last) {
        nvn = subset_views(pk[s], ns);
        set_trig(pk[s], ns, nvn);
        if (mexct_status e = upload_counts(pk[s], ns, nvn)) return e;
      }
      if (mexct_status e = begin_sweep()) return e;
      const float* src = s == 1 ? hmu[cur] : hmu[oth];
      for (int i = 0, z0 = 0; z0 < H; ++i, z0 += nz) {
        const int z1 = std::min(H, z0 + nz), m = z1 - z0;
        SlabIo io{src, z0, z1, (last && k > 1) ? hmu[cur] : nullptr, hmu[oth]};
        mexct_status e = run_slab(io, z0, z1, [&](int bs, const float** out) -> mexct_status {
          float* px = Wk[bs];
          float* py = Wk[bs] + pad_half;
          MEXCT_TRY_CUDA(launch_pad_volume_sub(X[bs], W, m, Pf, false, false, px, py, st, true),
                         "osc_tv_ooc: pad");
          fill_vox(*va, W, H, sad);
          va->zoff = z0;
          va->nzs = m;
          va->nviews = nvu;
          for (int j = 0; j < nvu; ++j) va->trig[j] = tu[j];
          MEXCT_TRY_CUDA(launch_osc_bp_update(geom, *va, d_rpre, d_rpost, X[bs], kF32, px, py, Pf,
                                              st),
                         "osc_tv_ooc: bp/update");
          if (!last) {
            if (mexct_status e2 = fp_part(px, py, z0, m, nvn, i > 0)) return e2;
          } else if (k > 1) {
            // this slab's part of ||mu_old - mu|| (mu_old(1) = 0: OSC_TV_recon.m:45)
            MEXCT_TRY_CUDA(launch_ssd(OLD[bs], X[bs], kF32, (long long)m * plane, z0 == 0 ? 1 : 0,
                                      d_parts, d_cnt, d_slots + i, st),
                           "osc_tv_ooc: d_a");
          }
          *out = X[bs];
          return MEXCT_OK;
        });
        if (e) return e;
      }
      if (!last) {
        if (mexct_status e = residual(nvn)) return e;
      }
      nv = nvn;
    }
    if (k > 1) {
      MEXCT_TRY_CUDA(launch_combine_norms(d_slots, nslab, d_scal, 0.f, nullptr, nullptr, st),
                     "osc_tv_ooc: d_a");
      // ||g(x_0)||: one norm sweep (slab + halo slices; the halo slices are
      // faces of the sub-volume, where the kernel's gradient is 0)
      if (mexct_status e = begin_sweep()) return e;
      for (int i = 0, z0 = 0; z0 < H; ++i, z0 += nz) {
        const int z1 = std::min(H, z0 + nz);
        const int a = std::max(z0 - 1, 0), b = std::min(z1 + 1, H);
        SlabIo io{hmu[oth], a, b, nullptr, nullptr};
        mexct_status e = run_slab(io, z0, z1, [&](int bs, const float**) -> mexct_status {
          MEXCT_TRY_CUDA(launch_tv_norm(X[bs], kF32, W, W, b - a, 1.f, d_parts, d_cnt, d_dummy,
                                        d_slots + i, st),
                         "osc_tv_ooc: tv norm");
          return MEXCT_OK;
        });
        if (e) return e;
      }
      MEXCT_TRY_CUDA(launch_combine_norms(d_slots, nslab, d_scal + 1, tv_const, d_scal, d_scale, st),
                     "osc_tv_ooc: tv scale");
      // 20 steps between the two host volumes; an even count ends in hmu[oth]
      for (int t = 0; t < kTvSteps; ++t) {
        const float* tsrc = (t % 2 == 0) ? hmu[oth] : hmu[cur];
        float* tdst = (t % 2 == 0) ? hmu[cur] : hmu[oth];
        const bool final_step = t == kTvSteps - 1;
        if (mexct_status e = begin_sweep()) return e;
        for (int i = 0, z0 = 0; z0 < H; ++i, z0 += nz) {
          const int z1 = std::min(H, z0 + nz), m = z1 - z0;
          const int a = std::max(z0 - 1, 0), b = std::min(z1 + 1, H);
          const int ya = std::max(z0 - 2, 0);  // Y holds slices ya .. z1 (+1 halo)
          SlabIo io{tsrc, a, b, nullptr, tdst};
          mexct_status e = run_slab(io, z0, z1, [&](int bs, const float** out) -> mexct_status {
            float* Y = Wk[bs];
            MEXCT_TRY_CUDA(launch_tv_update(X[bs], Y + (size_t)(a - ya) * plane, kF32, W, W, b - a,
                                            d_scale, st),
                           "osc_tv_ooc: tv update");
            if (z0 > ya)  // x_{t+1} of the slices below the slab, from the previous slab
              MEXCT_TRY_CUDA(cudaMemcpyAsync(Y, d_carry + (size_t)(2 - (z0 - ya)) * plane,
                                             (size_t)(z0 - ya) * plane * 4,
                                             cudaMemcpyDeviceToDevice, st),
                             "osc_tv_ooc: carry");
            if (!final_step)  // ||g(x_{t+1})||^2 over slices ya+1 .. z1-2
              MEXCT_TRY_CUDA(launch_tv_norm(Y, kF32, W, W, z1 - ya, 1.f, d_parts, d_cnt, d_dummy,
                                            d_slots + i, st),
                             "osc_tv_ooc: tv norm");
            if (z1 < H)
              MEXCT_TRY_CUDA(cudaMemcpyAsync(d_carry, Y + (size_t)(z1 - 2 - ya) * plane,
                                             2 * plane * 4, cudaMemcpyDeviceToDevice, st),
                             "osc_tv_ooc: carry");
            float* own = Y + (size_t)(z0 - ya) * plane;
            if (final_step)
              MEXCT_TRY_CUDA(launch_finite(own, kF32, (long long)m * plane, st),
                             "osc_tv_ooc: finite");
            *out = own;
            return MEXCT_OK;
          });
          if (e) return e;
        }
        if (!final_step)
          MEXCT_TRY_CUDA(launch_combine_norms(d_slots, nslab, d_scal + 1, tv_const, d_scal,
                                              d_scale, st),
                         "osc_tv_ooc: tv scale");
      }
    }
    cur = oth;
  }
  for (cudaStream_t s : {S.st, S.cin, S.cout})
    MEXCT_TRY_CUDA(cudaStreamSynchronize(s), "osc_tv_ooc: sync");
  unsigned flags = 0;
  MEXCT_TRY_CUDA(cudaMemcpy(&flags, c->err.p, sizeof flags, cudaMemcpyDeviceToHost),
                 "osc_tv_ooc: error word");
  if (flags)
    return set_err(MEXCT_ERR_TIMEOUT, "osc_tv_ooc: a bounded wait of the slab FP gave up (0x%x)",
                   flags);
  std::memcpy(recon, hmu[cur], N * sizeof(float));
  return MEXCT_OK;
}

}  // namespace mexct

extern "C" mexct_status mexct_osc_tv_ooc_plan(int W, int H, int nP, int geom, int n_iter,
                                              int n_sub_init, int n_sub_final, float p_val,
                                              size_t budget_bytes, int* slab_planes,
                                              size_t* device_bytes) {
  OocPlan pl;
  if (mexct_status e = ooc_plan(W, H, nP, geom, n_iter, n_sub_init, n_sub_final, p_val, nullptr,
                                budget_bytes, &pl))
    return e;
  if (slab_planes) *slab_planes = pl.nz;
  if (device_bytes) *device_bytes = pl.bytes;
  return MEXCT_OK;
}

extern "C" mexct_status mexct_osc_tv_recon_ooc(mexct_ctx* ctx, const float* pre,
                                               const float* post, int W, int H, int nP,
                                               const float* angles, float sad, int geom,
                                               int n_iter, float tv_const, int n_sub_init,
                                               int n_sub_final, float p_val,
                                               const int32_t* first_picks, size_t budget_bytes,
                                               float* recon, int* slab_planes) {
  return mexct::osc_tv_recon_ooc(ctx, pre, post, W, H, nP, angles, sad, geom, n_iter, tv_const,
                                 n_sub_init, n_sub_final, p_val, first_picks, budget_bytes, recon,
                                 slab_planes);
}
