// solver.cu -- device-resident OSC-TV: OSC_TV_recon.m on the GPU.
//
// iterative_reconstruction/OSC_TV_recon.m:33-74 runs one MEX call per OSC
// iteration and one per TV call, re-uploading mu and pre/post every time; the
// reference's oscIter also resets the device (CUDAmex_oscIter.cu:582), so no
// state survives.  Here mu, mu_old, pre and post stay on the device for the
// whole reconstruction; an iteration is a fixed sequence of kernels:
//
//   mu_old <- mu                                     (:45)
//   per subset: pad(mu), slab FP + residual, dual BP + update         (:51-59)
//   k > 1: d_a = ||mu_old - mu|| in FP64 (mu_old(1) = 0, NaN dropped)  (:64-67)
//          20 TV steps with c = TV_constant * d_a read on the device    (:68)
//          NaN/Inf -> 0                                                 (:69-70)
//
// and is captured once as a CUDA graph per (subset count, subset order)
// and replayed, so a reconstruction issues a handful of graph launches
// instead of ~70 kernel launches per iteration.
#include <cmath>
#include <cstring>
#include <algorithm>
#include <map>
#include <memory>
#include <vector>

#include "../../include/mexct.h"
#include "../../include/mexct_solver.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;

struct mexct_osctv {
  mexct_ctx* ctx = nullptr;
  int device = 0;
  int W = 0, H = 0, nP = 0, geom = 0, mu_type = kF32;
  // Storage of the residual views: kF32, or kF16 holding the residuals times
  // 2^-data_exp (the OSC update num/den does not depend on a common scale of
  // the two residuals).
  int data_type = kF32, data_exp = 0;
  float sad = 0.f;
  std::vector<float> angles;
  Buf mu, mu_old, pre, post, padx, pady, err, r1, r2, tvbuf, red, cnt, scal, objp;
  int k_done = 0;
  bool pre_zeroed = false;
  bool obj_valid = false;  // the last iteration computed the objective
  struct Key {
    int k_gt1, nsub, use_obj;
    float tvc;
    std::vector<int> picks;
    bool operator<(const Key& o) const {
      if (k_gt1 != o.k_gt1) return k_gt1 < o.k_gt1;
      if (nsub != o.nsub) return nsub < o.nsub;
      if (tvc != o.tvc) return tvc < o.tvc;
      if (use_obj != o.use_obj) return use_obj < o.use_obj;
      return picks < o.picks;
    }
  };
  std::map<Key, cudaGraphExec_t> graphs;
  // Graphs are captured and launched on this stream (capture is not allowed
  // on the legacy default stream), joined to the caller's stream by events.
  cudaStream_t own = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  ~mexct_osctv() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    for (Buf* b : {&mu, &mu_old, &pre, &post, &padx, &pady, &err, &r1, &r2, &tvbuf, &red, &cnt, &scal,
                   &objp})
      b->release();  // stream-ordered on `own`, after all its work
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (own) cudaStreamDestroy(own);
  }
  size_t N() const { return (size_t)W * W * H; }
  size_t M() const { return (size_t)W * H * nP; }
  // Scalars on the device: [0] d_a (double), [1] TV scale (float, as double
  // slot), [2] ||g|| (double), [3] objective (double).
  double* d_a() { return scal.as<double>(); }
  double* objective() { return scal.as<double>() + 3; }
  // Detector tiles of one view in the slab FP (32 x 8 pixels each).
  int tiles() const { return ((W + 31) / 32) * ((H + 7) / 8); }
  float* tv_scale() { return reinterpret_cast<float*>(scal.as<double>() + 1); }
  double* tv_norm() { return scal.as<double>() + 2; }
};

namespace {

constexpr int kTvSteps = 20;  // CUDAmex_TVmin_3D.cu:221

int num_subsets(int s_init, int s_final, double p, int max_iters, int k) {
  if (max_iters <= 1) return s_final;
  const double v = (double)(s_init - s_final) / std::pow((double)(max_iters - 1), p) *
                       std::pow((double)(max_iters - k), p) +
                   (double)s_final;
  return (int)std::round(v);  // MATLAB round: half away from zero
}

bool subset_order(int n, int first, int32_t* picks) {
  if (n <= 0 || first < 0 || first >= n) return false;
  std::vector<int> rest;  // 1-based subset numbers still to pick
  for (int i = 1; i <= n; ++i)
    if (i != first + 1) rest.push_back(i);
  int cur = first + 1;
  picks[0] = first;
  for (int s = 1; s < n; ++s) {
    std::vector<int> lo, hi;
    for (int v : rest) (v < cur ? lo : hi).push_back(v);
    std::vector<int>& side = lo.size() > hi.size() ? lo : hi;
    if (side.empty()) return false;
    const size_t pos = (side.size() + 1) / 2 - 1;  // ceil(numel/2), 1-based
    cur = side[pos];
    side.erase(side.begin() + pos);
    rest.clear();
    rest.insert(rest.end(), lo.begin(), lo.end());
    rest.insert(rest.end(), hi.begin(), hi.end());
    picks[s] = cur - 1;
  }
  return true;
}

// The FP64 data-fidelity objective sum(pre*e^-l + post*l) over every view
// and pixel, with l the OSC forward pass (border, step 0.5) of the current mu
// (the Poisson negative log-likelihood up to a constant; the reference has no
// counterpart).  One FP of all views, its epilogue reducing per CTA; the
// partials are summed in a fixed order into the objective scalar.
mexct_status enqueue_objective(mexct_osctv* s, cudaStream_t st) {
  CUtensorMap mx, my;
  int Pf = 0;
  mexct_status ps = prepare_slab_bufs(s->padx, s->pady, s->err, s->mu.p, s->mu_type, s->W, s->H,
                                      /*border=*/true, s->geom, &mx, &my, &Pf, st);
  if (ps) return ps;
  std::unique_ptr<RayArgs> ra(new RayArgs);
  fill_std_rays(*ra, s->W, s->H, s->sad, s->geom, /*osc=*/true);
  const int tiles = s->tiles();
  // CTAs add their sums to their partial (a CTA covers up to two views)
  MEXCT_TRY_CUDA(cudaMemsetAsync(s->objp.p, 0, (size_t)s->nP * tiles * sizeof(double), st),
                 "osctv: objective partials");
  for (int v0 = 0; v0 < s->nP; v0 += kMaxViews) {
    const int nv = std::min(kMaxViews, s->nP - v0);
    ra->nviews = nv;
    ra->view0 = v0;
    ra->vstride = 1;
    for (int i = 0; i < nv; ++i) trig_of(s->angles[v0 + i], &ra->trig[i]);
    SlabEpi e{s->pre.as<float>(), s->post.as<float>(), nullptr, nullptr, s->err.as<unsigned>()};
    e.obj = s->objp.as<double>() + (size_t)v0 * tiles;
    MEXCT_TRY_CUDA(launch_fp_slab_objective(s->geom, *ra, mx, my, s->padx.p, s->pady.p, Pf,
                                            s->mu_type, e, st),
                   "osctv: objective fp");
  }
  MEXCT_TRY_CUDA(launch_sum_partials(s->objp.as<double>(), (long long)s->nP * tiles,
                                     s->objective(), st),
                 "osctv: objective sum");
  return MEXCT_OK;
}

mexct_status enqueue_iteration(mexct_osctv* s, bool k_gt1, int nsub,
                               const int32_t* picks, float tvc, bool objective,
                               cudaStream_t st) {
  const size_t N = s->N();
  const size_t P = (size_t)s->W * s->H;
  const size_t vb = N * dsize(s->mu_type);
  MEXCT_TRY_CUDA(cudaMemcpyAsync(s->mu_old.p, s->mu.p, vb, cudaMemcpyDeviceToDevice, st),
                 "osctv: mu_old");
  std::unique_ptr<RayArgs> ra(new RayArgs);
  std::unique_ptr<VoxArgs> va(new VoxArgs);
  fill_std_rays(*ra, s->W, s->H, s->sad, s->geom, /*osc=*/true);
  fill_vox(*va, s->W, s->H, s->sad);
  // mu is padded (zero frame) once per iteration; every subset update
  // rewrites the padded copies along with mu.
  CUtensorMap mx, my;
  int Pf = 0;
  mexct_status ps = prepare_slab_bufs(s->padx, s->pady, s->err, s->mu.p, s->mu_type, s->W, s->H,
                                      /*border=*/true, s->geom, &mx, &my, &Pf, st);
  if (ps) return ps;
  for (int si = 0; si < nsub; ++si) {
    const int sel = picks[si];
    const int nv = (sel < 0 || sel >= s->nP) ? 0 : (s->nP - 1 - sel) / nsub + 1;
    ra->nviews = nv;
    ra->view0 = sel;
    ra->vstride = nsub;
    va->nviews = nv;
    for (int i = 0; i < nv; ++i) {
      trig_of(s->angles[sel + i * nsub], &ra->trig[i]);
      va->trig[i] = ra->trig[i];
    }
    if (nv > 0) {
      SlabEpi e{s->pre.as<float>(), s->post.as<float>(), s->r1.p, s->r2.p,
                s->err.as<unsigned>()};
      e.rscale = std::ldexp(1.0f, -s->data_exp);
      MEXCT_TRY_CUDA(launch_fp_slab(s->geom, true, true, *ra, mx, my, s->padx.p, s->pady.p, Pf,
                                    s->mu_type, nullptr, s->data_type, e, st),
                     "osctv: fp");
    }
    MEXCT_TRY_CUDA(launch_osc_bp_update(s->geom, *va, s->r1.p, s->r2.p, s->mu.p, s->mu_type,
                                        s->padx.p, s->pady.p, Pf, st, s->data_type),
                   "osctv: bp/update");
  }
  (void)P;
  if (k_gt1) {
    MEXCT_TRY_CUDA(launch_ssd(s->mu_old.p, s->mu.p, s->mu_type, (long long)N, 1,
                              s->red.as<double>(), s->cnt.as<unsigned>(), s->d_a(), st),
                   "osctv: d_a");
    // 20 steps on the ping-pong pair (mu, tvbuf); an even count ends in mu.
    const void* src = s->mu.p;
    for (int k = 0; k < kTvSteps; ++k) {
      void* dst = ((kTvSteps - 1 - k) % 2 == 0) ? s->mu.p : s->tvbuf.p;
      MEXCT_TRY_CUDA(launch_tv_norm_scaled(src, s->mu_type, s->W, s->W, s->H, tvc, s->d_a(),
                                           s->red.as<double>(), s->cnt.as<unsigned>(),
                                           s->tv_scale(), s->tv_norm(), st),
                     "osctv: tv norm");
      MEXCT_TRY_CUDA(launch_tv_update(src, dst, s->mu_type, s->W, s->W, s->H, s->tv_scale(), st),
                     "osctv: tv update");
      src = dst;
    }
    MEXCT_TRY_CUDA(launch_finite(s->mu.p, s->mu_type, (long long)N, st), "osctv: finite");
  }
  if (objective) return enqueue_objective(s, st);
  return MEXCT_OK;
}

}  // namespace

extern "C" {

int mexct_num_subsets(int s_init, int s_final, float p_val, int max_iters, int k) {
  return num_subsets(s_init, s_final, (double)p_val, max_iters, k);
}

mexct_status mexct_subset_order(int n_sub, int first_pick, int32_t* picks) {
  if (!picks) return set_err(MEXCT_ERR_ARG, "subset_order: NULL pointer");
  if (!subset_order(n_sub, first_pick, picks))
    return set_err(MEXCT_ERR_ARG, "subset_order: bad n_sub %d / first pick %d", n_sub, first_pick);
  return MEXCT_OK;
}

mexct_status mexct_osctv_create(mexct_ctx* ctx, const float* d_pre, const float* d_post,
                                int W, int H, int nP, const float* angles, float sad, int geom,
                                int mu_type, void* stream, mexct_osctv** out) {
  return mexct_osctv_create_ex(ctx, d_pre, d_post, W, H, nP, angles, sad, geom, mu_type,
                               MEXCT_F32, stream, out);
}

mexct_status mexct_osctv_create_ex(mexct_ctx* ctx, const float* d_pre, const float* d_post,
                                   int W, int H, int nP, const float* angles, float sad,
                                   int geom, int mu_type, int data_type, void* stream,
                                   mexct_osctv** out) {
  if (!out) return set_err(MEXCT_ERR_ARG, "osctv_create: out is NULL");
  *out = nullptr;
  if (!d_pre || !d_post || !angles) return set_err(MEXCT_ERR_ARG, "osctv_create: NULL pointer");
  if (W <= 0 || H <= 0 || nP <= 0 || W > 16384 || H > 16384)
    return set_err(MEXCT_ERR_ARG, "osctv_create: bad dims %d x %d x %d", W, H, nP);
  if (geom < 0 || geom > 2) return set_err(MEXCT_ERR_ARG, "osctv_create: invalid geometry %d", geom);
  if (mu_type != kF32 && mu_type != kF16 && mu_type != kBF16)
    return set_err(MEXCT_ERR_ARG, "osctv_create: bad storage type %d", mu_type);
  if (data_type != kF32 && data_type != kF16)
    return set_err(MEXCT_ERR_ARG, "osctv_create: bad data storage type %d", data_type);
  if (data_type == kF16 && mu_type != kF32)
    return set_err(MEXCT_ERR_UNSUPPORTED, "osctv_create: FP16 residual views need FP32 mu");
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "osctv_create: no CUDA device / context");
  DevGuard dg(c->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::unique_ptr<mexct_osctv> s(new mexct_osctv);
  s->ctx = c;
  s->device = c->device;
  s->W = W;
  s->H = H;
  s->nP = nP;
  s->geom = geom;
  s->sad = sad;
  s->mu_type = mu_type;
  s->data_type = data_type;
  s->angles.assign(angles, angles + nP);
  MEXCT_TRY_CUDA(cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking), "osctv_create: stream");
  MEXCT_TRY_CUDA(cudaEventCreateWithFlags(&s->ev_in, cudaEventDisableTiming), "osctv_create: event");
  MEXCT_TRY_CUDA(cudaEventCreateWithFlags(&s->ev_out, cudaEventDisableTiming), "osctv_create: event");
  const size_t N = s->N(), M = s->M(), vb = N * dsize(mu_type);
  const size_t P = (size_t)W * H;

  // Buffers are allocated stream-ordered on the solver's stream, so creating
  // and destroying solvers never synchronises the device (other streams keep
  // running); the caller's stream waits for the allocations.
  cudaStream_t a = s->own;
  const size_t pb = (size_t)slab_pitch(W) * (W + 2) * (H + 2) * dsize(mu_type);
  const size_t parts = std::max<size_t>(tv_partials_needed(W, W, H), ssd_partials_needed()) + 8;
  MEXCT_TRY_CUDA(s->mu.ensure_async(vb, a), "osctv_create: mu");
  MEXCT_TRY_CUDA(s->mu_old.ensure_async(vb, a), "osctv_create: mu_old");
  MEXCT_TRY_CUDA(s->tvbuf.ensure_async(vb, a), "osctv_create: tv");
  MEXCT_TRY_CUDA(s->padx.ensure_async(pb, a), "osctv_create: padded mu");
  MEXCT_TRY_CUDA(s->pady.ensure_async(pb, a), "osctv_create: padded mu");
  MEXCT_TRY_CUDA(s->pre.ensure_async(M * 4, a), "osctv_create: pre");
  MEXCT_TRY_CUDA(s->post.ensure_async(M * 4, a), "osctv_create: post");
  // the residual views are sized by mexct_osctv_run for its largest subset
  (void)P;
  MEXCT_TRY_CUDA(s->red.ensure_async(parts * sizeof(double), a), "osctv_create: reduction");
  MEXCT_TRY_CUDA(s->err.ensure_async(64, a), "osctv_create: error word");
  MEXCT_TRY_CUDA(s->cnt.ensure_async(64, a), "osctv_create: counter");
  MEXCT_TRY_CUDA(s->scal.ensure_async(64, a), "osctv_create: scalars");
  MEXCT_TRY_CUDA(s->objp.ensure_async((size_t)nP * s->tiles() * sizeof(double), a),
                 "osctv_create: objective partials");
  MEXCT_TRY_CUDA(cudaMemsetAsync(s->err.p, 0, 64, a), "osctv_create: error word");
  MEXCT_TRY_CUDA(cudaMemsetAsync(s->cnt.p, 0, 64, a), "osctv_create: counter");
  MEXCT_TRY_CUDA(cudaMemsetAsync(s->scal.p, 0, 64, a), "osctv_create: scalars");
  MEXCT_TRY_CUDA(cudaEventRecord(s->ev_in, a), "osctv_create: join");
  MEXCT_TRY_CUDA(cudaStreamWaitEvent(st, s->ev_in, 0), "osctv_create: join");
  // OSC_TV_recon.m:33 mu = 1e-10; :35-37 pre/post clamped to >= 1e-6.
  MEXCT_TRY_CUDA(launch_fill(s->mu.p, mu_type, (long long)N, 1e-10f, st), "osctv_create: mu");
  if (data_type == kF16) {
    // one power-of-two scale for both residuals (|pre e^-l - post| and
    // pre e^-l l are below max(pre, post)): the largest count to (2^14, 2^15],
    // so counts of any magnitude (photon counts or intensities below 1) keep
    // FP16's 11-bit precision away from its subnormal range
    unsigned* d_max = reinterpret_cast<unsigned*>(s->scal.as<double>() + 4);
    MEXCT_TRY_CUDA(cudaMemsetAsync(d_max, 0, sizeof(unsigned), st), "osctv_create: scale");
    MEXCT_TRY_CUDA(launch_max_nonneg(d_pre, (long long)M, d_max, st), "osctv_create: scale");
    MEXCT_TRY_CUDA(launch_max_nonneg(d_post, (long long)M, d_max, st), "osctv_create: scale");
    unsigned bits = 0;
    MEXCT_TRY_CUDA(cudaMemcpyAsync(&bits, d_max, sizeof bits, cudaMemcpyDeviceToHost, st),
                   "osctv_create: scale");
    MEXCT_TRY_CUDA(cudaStreamSynchronize(st), "osctv_create: scale");
    float mx;
    std::memcpy(&mx, &bits, sizeof mx);
    const double top = std::max((double)mx, 1e-6);  // the clamped counts' largest
    int e = 0;
    while (e < 100 && std::ldexp(top, -e) > 32768.0) ++e;
    while (e > -100 && std::ldexp(top, -(e - 1)) <= 32768.0) --e;
    s->data_exp = e;
  }
  MEXCT_TRY_CUDA(launch_clamp_copy(d_pre, s->pre.as<float>(), (long long)M, 1e-6f, st),
                 "osctv_create: pre");
  MEXCT_TRY_CUDA(launch_clamp_copy(d_post, s->post.as<float>(), (long long)M, 1e-6f, st),
                 "osctv_create: post");
  // Run one eager iteration-free launch setup so kernel attributes are set
  // outside any later stream capture.
  {
    CUtensorMap mx, my;
    int Pf = 0;
    mexct_status ps = prepare_slab_bufs(s->padx, s->pady, s->err, s->mu.p, mu_type, W, H, true,
                                        geom, &mx, &my, &Pf, st);
    if (ps) return ps;
    std::unique_ptr<RayArgs> ra(new RayArgs);
    fill_std_rays(*ra, W, H, sad, geom, true);
    ra->nviews = 0;  // no work: sets attributes only
    SlabEpi e{s->pre.as<float>(), s->post.as<float>(), s->r1.p, s->r2.p, s->err.as<unsigned>()};
    MEXCT_TRY_CUDA(launch_fp_slab(geom, true, true, *ra, mx, my, s->padx.p, s->pady.p, Pf,
                                  mu_type, nullptr, data_type, e, st),
                   "osctv_create: kernel setup");
    e.obj = s->objp.as<double>();
    MEXCT_TRY_CUDA(launch_fp_slab_objective(geom, *ra, mx, my, s->padx.p, s->pady.p, Pf, mu_type,
                                            e, st),
                   "osctv_create: kernel setup");
  }
  *out = s.release();
  return MEXCT_OK;
}

mexct_status mexct_osctv_run(mexct_osctv* s, const mexct_osctv_params* p,
                             const int32_t* first_picks, int n, void* stream) {
  if (!s || !p || (!first_picks && n > 0)) return set_err(MEXCT_ERR_ARG, "osctv_run: NULL pointer");
  if (n < 0 || p->n_iter < 1) return set_err(MEXCT_ERR_ARG, "osctv_run: bad iteration count");
  DevGuard dg(s->device);
  NvtxRange nvtx("mexct:osctv_run");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  {
    // Residual views for the largest subset of this call's iterations, in the
    // padded quad layout; their zero frame (border addressing) is written when
    // they are allocated and never touched again.
    int nvmax = 1;
    for (int i = 0; i < n; ++i) {
      const int ns = num_subsets(p->n_sub_init, p->n_sub_final, p->p_val, p->n_iter,
                                 s->k_done + 1 + i);
      if (ns > 0) nvmax = std::max(nvmax, (s->nP + ns - 1) / ns);
    }
    if (nvmax > kMaxViews)
      return set_err(MEXCT_ERR_UNSUPPORTED, "osctv_run: subset of %d views (max %d)", nvmax,
                     kMaxViews);
    const size_t rb = sino_pad_elems(s->W, s->H, nvmax) * 4 * dsize(s->data_type);
    if (!s->r1.p || rb > s->r1.n) {
      // work queued on the caller's stream may still read the old views
      MEXCT_TRY_CUDA(cudaEventRecord(s->ev_in, st), "osctv_run: join");
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(s->own, s->ev_in, 0), "osctv_run: join");
      MEXCT_TRY_CUDA(s->r1.ensure_async(rb, s->own), "osctv_run: residual");
      MEXCT_TRY_CUDA(s->r2.ensure_async(rb, s->own), "osctv_run: residual");
      MEXCT_TRY_CUDA(cudaMemsetAsync(s->r1.p, 0, s->r1.n, s->own), "osctv_run: residual");
      MEXCT_TRY_CUDA(cudaMemsetAsync(s->r2.p, 0, s->r2.n, s->own), "osctv_run: residual");
      MEXCT_TRY_CUDA(cudaEventRecord(s->ev_out, s->own), "osctv_run: join");
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(st, s->ev_out, 0), "osctv_run: join");
      // captured iterations hold the old buffers (an executing graph is freed
      // when it completes)
      for (auto& g : s->graphs) cudaGraphExecDestroy(g.second);
      s->graphs.clear();
    }
  }
  for (int i = 0; i < n; ++i) {
    const int k = s->k_done + 1;  // 1-based iteration number
    const int nsub = num_subsets(p->n_sub_init, p->n_sub_final, p->p_val, p->n_iter, k);
    if (nsub <= 0) return set_err(MEXCT_ERR_ARG, "osctv_run: %d subsets at iteration %d", nsub, k);
    if ((size_t)((s->nP + nsub - 1) / nsub) > (size_t)kMaxViews)
      return set_err(MEXCT_ERR_UNSUPPORTED, "osctv_run: subset too large");
    int fp = first_picks[i];
    fp = ((fp % nsub) + nsub) % nsub;
    std::vector<int32_t> picks(nsub);
    if (!subset_order(nsub, fp, picks.data()))
      return set_err(MEXCT_ERR_ARG, "osctv_run: subset order");
    if (k >= 2 && !s->pre_zeroed) {
      // OSC_TV_recon.m:41,62: from iteration 2 on, pre(1) = post(1) = 0.
      MEXCT_TRY_CUDA(cudaMemsetAsync(s->pre.p, 0, sizeof(float), st), "osctv_run: pre(1)");
      MEXCT_TRY_CUDA(cudaMemsetAsync(s->post.p, 0, sizeof(float), st), "osctv_run: post(1)");
      s->pre_zeroed = true;
    }
    const bool kg1 = k > 1;
    if (p->use_graph) {
      mexct_osctv::Key key{kg1 ? 1 : 0, nsub, p->objective ? 1 : 0, p->tv_const,
                           std::vector<int>(picks.begin(), picks.end())};
      auto it = s->graphs.find(key);
      if (it == s->graphs.end()) {
        cudaGraph_t g = nullptr;
        MEXCT_TRY_CUDA(cudaStreamBeginCapture(s->own, cudaStreamCaptureModeThreadLocal),
                       "osctv_run: begin capture");
        mexct_status e = enqueue_iteration(s, kg1, nsub, picks.data(), p->tv_const,
                                           p->objective != 0, s->own);
        cudaError_t ce = cudaStreamEndCapture(s->own, &g);
        if (e != MEXCT_OK) {
          if (g) cudaGraphDestroy(g);
          return e;
        }
        MEXCT_TRY_CUDA(ce, "osctv_run: end capture");
        cudaGraphExec_t ex = nullptr;
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        MEXCT_TRY_CUDA(ce, "osctv_run: instantiate");
        it = s->graphs.emplace(key, ex).first;
      }
      MEXCT_TRY_CUDA(cudaEventRecord(s->ev_in, st), "osctv_run: join");
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(s->own, s->ev_in, 0), "osctv_run: join");
      MEXCT_TRY_CUDA(cudaGraphLaunch(it->second, s->own), "osctv_run: graph launch");
      MEXCT_TRY_CUDA(cudaEventRecord(s->ev_out, s->own), "osctv_run: join");
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(st, s->ev_out, 0), "osctv_run: join");
    } else {
      mexct_status e = enqueue_iteration(s, kg1, nsub, picks.data(), p->tv_const,
                                         p->objective != 0, st);
      if (e != MEXCT_OK) return e;
    }
    s->k_done = k;
    s->obj_valid = p->objective != 0;
  }
  return MEXCT_OK;
}

mexct_status mexct_osctv_mu(mexct_osctv* s, float* d_out, void* stream) {
  if (!s || !d_out) return set_err(MEXCT_ERR_ARG, "osctv_mu: NULL pointer");
  DevGuard dg(s->device);
  MEXCT_TRY_CUDA(launch_convert(s->mu.p, s->mu_type, d_out, kF32, (long long)s->N(),
                                static_cast<cudaStream_t>(stream)),
                 "osctv_mu: convert");
  return MEXCT_OK;
}

mexct_status mexct_osctv_stats(mexct_osctv* s, int* iters, double* d_a, double* obj) {
  if (!s) return set_err(MEXCT_ERR_ARG, "osctv_stats: NULL solver");
  DevGuard dg(s->device);
  double h[4] = {0, 0, 0, 0};
  MEXCT_TRY_CUDA(cudaMemcpy(h, s->scal.p, sizeof h, cudaMemcpyDeviceToHost), "osctv_stats");
  if (iters) *iters = s->k_done;
  if (d_a) *d_a = h[0];
  if (obj) *obj = s->obj_valid ? h[3] : std::nan("");
  return MEXCT_OK;
}

size_t mexct_osctv_state_bytes(const mexct_osctv* s) {
  if (!s) return 0;
  return 64 + 2 * s->N() * dsize(s->mu_type);
}

mexct_status mexct_osctv_snapshot(mexct_osctv* s, void* host, void* stream) {
  if (!s || !host) return set_err(MEXCT_ERR_ARG, "osctv_snapshot: NULL pointer");
  DevGuard dg(s->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t hdr[8] = {0x4d455843, s->W, s->H, s->nP, s->mu_type, s->k_done, s->pre_zeroed, 0};
  std::memcpy(host, hdr, sizeof hdr);
  const size_t vb = s->N() * dsize(s->mu_type);
  unsigned char* h = static_cast<unsigned char*>(host) + 64;
  MEXCT_TRY_CUDA(cudaMemcpyAsync(h, s->mu.p, vb, cudaMemcpyDeviceToHost, st), "osctv_snapshot");
  MEXCT_TRY_CUDA(cudaMemcpyAsync(h + vb, s->mu_old.p, vb, cudaMemcpyDeviceToHost, st),
                 "osctv_snapshot");
  MEXCT_TRY_CUDA(cudaStreamSynchronize(st), "osctv_snapshot");
  return MEXCT_OK;
}

mexct_status mexct_osctv_restore(mexct_osctv* s, const void* host, void* stream) {
  if (!s || !host) return set_err(MEXCT_ERR_ARG, "osctv_restore: NULL pointer");
  int64_t hdr[8];
  std::memcpy(hdr, host, sizeof hdr);
  if (hdr[0] != 0x4d455843 || hdr[1] != s->W || hdr[2] != s->H || hdr[3] != s->nP ||
      hdr[4] != s->mu_type)
    return set_err(MEXCT_ERR_ARG, "osctv_restore: snapshot does not match this solver");
  DevGuard dg(s->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t vb = s->N() * dsize(s->mu_type);
  const unsigned char* h = static_cast<const unsigned char*>(host) + 64;
  MEXCT_TRY_CUDA(cudaMemcpyAsync(s->mu.p, h, vb, cudaMemcpyHostToDevice, st), "osctv_restore");
  MEXCT_TRY_CUDA(cudaMemcpyAsync(s->mu_old.p, h + vb, vb, cudaMemcpyHostToDevice, st),
                 "osctv_restore");
  if (hdr[6] && !s->pre_zeroed) {
    MEXCT_TRY_CUDA(cudaMemsetAsync(s->pre.p, 0, sizeof(float), st), "osctv_restore");
    MEXCT_TRY_CUDA(cudaMemsetAsync(s->post.p, 0, sizeof(float), st), "osctv_restore");
    s->pre_zeroed = true;
  }
  MEXCT_TRY_CUDA(cudaStreamSynchronize(st), "osctv_restore");
  s->k_done = (int)hdr[5];
  return MEXCT_OK;
}

mexct_status mexct_osctv_destroy(mexct_osctv* s) {
  if (!s) return MEXCT_OK;
  DevGuard dg(s->device);
  delete s;
  return MEXCT_OK;
}

mexct_status mexct_osc_tv_recon(mexct_ctx* ctx, const float* pre, const float* post, int W,
                                int H, int nP, const float* angles, float sad, int geom,
                                int n_iter, float tv_const, int n_sub_init, int n_sub_final,
                                float p_val, const int32_t* first_picks, float* recon) {
  return mexct::osc_tv_recon_typed(ctx, pre, post, W, H, nP, angles, sad, geom, n_iter, tv_const,
                                   n_sub_init, n_sub_final, p_val, first_picks, kF32, recon);
}

}  // extern "C"

namespace mexct {

// OSC_TV_recon with host arrays on a context's stream, mu stored as mu_type.
mexct_status osc_tv_recon_typed(mexct_ctx* ctx, const float* pre, const float* post, int W, int H,
                                int nP, const float* angles, float sad, int geom, int n_iter,
                                float tv_const, int n_sub_init, int n_sub_final, float p_val,
                                const int32_t* first_picks, int mu_type, float* recon,
                                int data_type) {
  if (!pre || !post || !angles || !recon || !first_picks)
    return set_err(MEXCT_ERR_ARG, "osc_tv_recon: NULL pointer");
  if (W <= 0 || H <= 0 || nP <= 0 || n_iter < 1)
    return set_err(MEXCT_ERR_ARG, "osc_tv_recon: bad dims / iterations");
  if (geom < 0 || geom > 2) return set_err(MEXCT_ERR_ARG, "osc_tv_recon: invalid geometry %d", geom);
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "osc_tv_recon: no CUDA device / context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  DevGuard dg(c->device);
  const size_t M = (size_t)W * H * nP, N = (size_t)W * W * H;
  MEXCT_TRY_CUDA(c->in.ensure_async(M * 4, c->stream), "osc_tv_recon: upload");
  MEXCT_TRY_CUDA(c->in2.ensure_async(M * 4, c->stream), "osc_tv_recon: upload");
  MEXCT_TRY_CUDA(c->out.ensure_async(N * 4, c->stream), "osc_tv_recon: workspace");
  MEXCT_TRY_CUDA(cudaMemcpyAsync(c->in.p, pre, M * 4, cudaMemcpyHostToDevice, c->stream),
                 "osc_tv_recon: upload");
  MEXCT_TRY_CUDA(cudaMemcpyAsync(c->in2.p, post, M * 4, cudaMemcpyHostToDevice, c->stream),
                 "osc_tv_recon: upload");
  mexct_osctv* s = nullptr;
  mexct_status r = mexct_osctv_create_ex(c, c->in.as<float>(), c->in2.as<float>(), W, H, nP,
                                         angles, sad, geom, mu_type,
                                         data_type == 0 ? (int)kF32 : data_type, c->stream, &s);
  if (r) return r;
  mexct_osctv_params p{n_iter, tv_const, n_sub_init, n_sub_final, p_val, 1, 0};
  r = mexct_osctv_run(s, &p, first_picks, n_iter, c->stream);
  if (!r) r = mexct_osctv_mu(s, c->out.as<float>(), c->stream);
  if (!r) {
    cudaError_t e = cudaMemcpyAsync(recon, c->out.p, N * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) r = cuda_err(e, "osc_tv_recon: download");
  }
  mexct_osctv_destroy(s);
  return r;
}

}  // namespace mexct
