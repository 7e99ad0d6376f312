// batch.cu -- batched FP / BP over many independent problems of different
// sizes and geometries (include/mexct_batch.h).
//
// A batch is planned once (padded-volume buffers, per-problem device
// descriptors with TMA maps and trig tables); each operator then runs as a
// fixed, capturable sequence: one batched padding launch plus one persistent
// FP launch, or one sinogram-padding launch per problem plus one persistent BP
// launch.  Persistent CTAs take work items
// (problem, view, tile) / (problem, brick) from a global counter, so uneven
// problems load-balance inside one launch.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/mexct.h"
#include "../../include/mexct_batch.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;

struct mexct_batch {
  int device = 0;
  int n = 0;
  std::vector<Buf> pads;   // 2 per problem: padded volume, both layouts
  std::vector<Buf> spads;  // 1 per problem: the BP views in the quad layout
  std::vector<mexct_problem> probs;
  // BP launch arguments per problem and view chunk (at most kMaxViews views)
  std::vector<std::vector<std::unique_ptr<VoxArgs>>> vox;
  Buf fp_desc, trig, counters, err;
  long long fp_items = 0, pad_items = 0;
  int sms = 1;  // set from cudaDevAttrMultiProcessorCount at creation
  // BP: the problems' launches fan out over kAux streams (fork / join events
  // on the caller's stream, so a capture records them as graph branches)
  static constexpr int kAux = 8;
  cudaStream_t aux[kAux] = {};
  cudaEvent_t fork = nullptr, join[kAux] = {};
  ~mexct_batch() {
    for (Buf& b : pads) b.release();
    for (Buf& b : spads) b.release();
    for (Buf* b : {&fp_desc, &trig, &counters, &err}) b->release();
    for (int k = 0; k < kAux; ++k) {
      if (aux[k]) cudaStreamDestroy(aux[k]);
      if (join[k]) cudaEventDestroy(join[k]);
    }
    if (fork) cudaEventDestroy(fork);
  }
};

extern "C" {

mexct_status mexct_batch_create(mexct_ctx* ctx, const mexct_problem* probs, int n,
                                mexct_batch** out) {
  if (!out) return set_err(MEXCT_ERR_ARG, "batch_create: out is NULL");
  *out = nullptr;
  if (!probs || n <= 0) return set_err(MEXCT_ERR_ARG, "batch_create: no problems");
  for (int i = 0; i < n; ++i) {
    const mexct_problem& p = probs[i];
    if (p.W <= 0 || p.H <= 0 || p.nP <= 0 || p.W > 16384 || p.H > 16384 || p.nP > 1 << 20)
      return set_err(MEXCT_ERR_ARG, "batch_create: problem %d has bad dims", i);
    if (p.geom < 0 || p.geom > 2)
      return set_err(MEXCT_ERR_ARG, "batch_create: problem %d: invalid geometry %d", i, p.geom);
    if (!p.angles || !p.d_vol || !p.d_sino || !p.d_rec)
      return set_err(MEXCT_ERR_ARG, "batch_create: problem %d: NULL pointer", i);
  }
  mexct_ctx* c = resolve(ctx);
  if (!c) return set_err(MEXCT_ERR_CUDA, "batch_create: no CUDA device / context");
  DevGuard dg(c->device);
  std::unique_ptr<mexct_batch> b(new mexct_batch);
  b->device = c->device;
  b->n = n;
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, c->device);
  size_t ntrig = 0;
  for (int i = 0; i < n; ++i) ntrig += probs[i].nP;
  std::vector<Trig> trig(ntrig);
  std::vector<BatchFp> fd(n);
  b->pads.resize(2 * n);
  b->spads.resize(n);
  b->vox.resize(n);
  for (int k = 0; k < mexct_batch::kAux; ++k) {
    MEXCT_TRY_CUDA(cudaStreamCreateWithFlags(&b->aux[k], cudaStreamNonBlocking),
                   "batch_create: streams");
    MEXCT_TRY_CUDA(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming),
                   "batch_create: events");
  }
  MEXCT_TRY_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming),
                 "batch_create: events");
  b->probs.assign(probs, probs + n);
  size_t toff = 0;
  MEXCT_TRY_CUDA(b->trig.ensure(ntrig * sizeof(Trig)), "batch_create: trig");
  const Trig* dtrig = b->trig.as<Trig>();
  for (int i = 0; i < n; ++i) {
    const mexct_problem& p = probs[i];
    const int W = p.W, H = p.H;
    const int Pf = slab_pitch(W);
    const size_t pb = (size_t)Pf * (W + 2) * (H + 2) * sizeof(float);
    MEXCT_TRY_CUDA(b->pads[2 * i].ensure(pb), "batch_create: padded volume");
    MEXCT_TRY_CUDA(b->pads[2 * i + 1].ensure(pb), "batch_create: padded volume");
    for (int v = 0; v < p.nP; ++v) trig_of(p.angles[v], &trig[toff + v]);
    BatchFp& f = fd[i];
    std::memset(&f, 0, sizeof f);
    MEXCT_TRY_CUDA(make_slab_tmap(&f.tmx, b->pads[2 * i].p, kF32, Pf, W + 2, H + 2, p.geom),
                   "batch_create: tensor map");
    MEXCT_TRY_CUDA(make_slab_tmap(&f.tmy, b->pads[2 * i + 1].p, kF32, Pf, W + 2, H + 2, p.geom),
                   "batch_create: tensor map");
    f.W = W;
    f.H = H;
    f.geom = p.geom;
    f.nviews = p.nP;
    f.Pf = Pf;
    f.tiles_u = (W + 31) / 32;
    f.u0 = float(W - 1) / 2;  // CUDAmex_FP.cu:378-379
    f.v0 = float(H - 1) / 2;
    f.bx = -(float)W / 2.0f;  // :424-426
    f.by = -(float)W / 2.0f;
    f.bz = -(float)H / 2.0f;
    f.sad = p.sad;
    f.step = p.geom == 2 ? 1.0f : 0.5f;
    f.item0 = b->fp_items;
    b->fp_items += (long long)p.nP * f.tiles_u * ((H + 7) / 8);
    f.px = b->pads[2 * i].p;
    f.py = b->pads[2 * i + 1].p;
    f.out = p.d_sino;
    f.trig = dtrig + toff;
    f.vol = p.d_vol;
    f.pad_item0 = b->pad_items;
    const long long nt = (Pf + 31) / 32;
    b->pad_items += nt * nt * (H + 2);
    // BP: views in the quad layout, one launch per kMaxViews views
    // (mexct_bp_dev's shapes without view blocks)
    MEXCT_TRY_CUDA(b->spads[i].ensure(sino_pad_elems(W, H, p.nP) * sizeof(float4)),
                   "batch_create: padded sinogram");
    for (int v0 = 0; v0 < p.nP; v0 += kMaxViews) {
      std::unique_ptr<VoxArgs> va(new VoxArgs);
      fill_vox(*va, W, H, p.sad);
      va->nviews = std::min(kMaxViews, p.nP - v0);
      va->view0 = 0;
      for (int v = 0; v < va->nviews; ++v) trig_of(p.angles[v0 + v], &va->trig[v]);
      b->vox[i].push_back(std::move(va));
    }
    toff += p.nP;
  }
  MEXCT_TRY_CUDA(b->fp_desc.ensure(n * sizeof(BatchFp)), "batch_create: descriptors");
  MEXCT_TRY_CUDA(b->counters.ensure(64), "batch_create: counters");
  MEXCT_TRY_CUDA(b->err.ensure(64), "batch_create: error word");
  MEXCT_TRY_CUDA(cudaMemcpy(b->trig.p, trig.data(), ntrig * sizeof(Trig), cudaMemcpyHostToDevice),
                 "batch_create: upload");
  MEXCT_TRY_CUDA(cudaMemcpy(b->fp_desc.p, fd.data(), n * sizeof(BatchFp), cudaMemcpyHostToDevice),
                 "batch_create: upload");
  MEXCT_TRY_CUDA(cudaMemset(b->err.p, 0, 64), "batch_create: error word");
  *out = b.release();
  return MEXCT_OK;
}

mexct_status mexct_batch_fp(mexct_batch* b, void* stream) {
  if (!b) return set_err(MEXCT_ERR_ARG, "batch_fp: NULL batch");
  DevGuard dg(b->device);
  NvtxRange nvtx("mexct:batch_fp");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MEXCT_TRY_CUDA(launch_pad_batch(b->fp_desc.as<BatchFp>(), b->n, b->pad_items, st),
                 "batch_fp: padding");
  MEXCT_TRY_CUDA(cudaMemsetAsync(b->counters.p, 0, sizeof(unsigned long long), st),
                 "batch_fp: counter");
  MEXCT_TRY_CUDA(launch_fp_batch(b->fp_desc.as<BatchFp>(), b->n, b->fp_items,
                                 b->counters.as<unsigned long long>(), b->err.as<unsigned>(),
                                 b->sms * slab_ctas_per_sm(), st),
                 "batch_fp: launch");
  return MEXCT_OK;
}

mexct_status mexct_batch_bp(mexct_batch* b, void* stream) {
  if (!b) return set_err(MEXCT_ERR_ARG, "batch_bp: NULL batch");
  DevGuard dg(b->device);
  NvtxRange nvtx("mexct:batch_bp");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MEXCT_TRY_CUDA(cudaEventRecord(b->fork, st), "batch_bp: fork");
  for (int k = 0; k < mexct_batch::kAux; ++k)
    MEXCT_TRY_CUDA(cudaStreamWaitEvent(b->aux[k], b->fork, 0), "batch_bp: fork");
  for (int i = 0; i < b->n; ++i) {
    const mexct_problem& p = b->probs[i];
    cudaStream_t s = b->aux[i % mexct_batch::kAux];
    MEXCT_TRY_CUDA(launch_pad_sino_quad(p.d_sino, kF32, p.W, p.H, p.nP, b->spads[i].p, s),
                   "batch_bp: padding");
    const size_t vstride = sino_pad_elems(p.W, p.H, 1) * sizeof(float4);
    const BpShape shp{16, 8, 1};
    int v0 = 0;
    for (const auto& va : b->vox[i]) {
      const char* src = static_cast<const char*>(b->spads[i].p) + (size_t)v0 * vstride;
      MEXCT_TRY_CUDA(launch_bp_quad(p.geom, *va, src, kF32, p.d_rec, kF32, v0 > 0, shp, nullptr,
                                    s),
                     "batch_bp: launch");
      v0 += va->nviews;
    }
  }
  for (int k = 0; k < mexct_batch::kAux; ++k) {
    MEXCT_TRY_CUDA(cudaEventRecord(b->join[k], b->aux[k]), "batch_bp: join");
    MEXCT_TRY_CUDA(cudaStreamWaitEvent(st, b->join[k], 0), "batch_bp: join");
  }
  return MEXCT_OK;
}

mexct_status mexct_batch_destroy(mexct_batch* b) {
  if (!b) return MEXCT_OK;
  DevGuard dg(b->device);
  delete b;
  return MEXCT_OK;
}

}  // extern "C"
