// ops.cu -- operator entry points of the C ABI (include/mexct.h).
//
// Device twins (*_dev) run stream-ordered on caller memory; host entry points
// stage the MATLAB arrays through the context's workspaces on the context's
// stream and synchronise before returning (the MEX gateway contract).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/mexct.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;

namespace {

bool bad_geom(int g) { return g < 0 || g > 2; }
bool bad_type(int t) { return t != kF32 && t != kF16 && t != kBF16; }

// Shape limits: every index below fits the int/size_t arithmetic used by the
// kernels and a detector tile grid fits gridDim.y.
bool bad_dims(long long W, long long H) {
  return W <= 0 || H <= 0 || W > 16384 || H > 16384;
}

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

mexct_status upload(Buf& b, const void* src, size_t bytes, cudaStream_t st,
                    const char* what) {
  MEXCT_TRY_CUDA(b.ensure_async(bytes, st), what);
  if (bytes) MEXCT_TRY_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, st), what);
  return MEXCT_OK;
}

mexct_status finish(mexct_ctx* c, void* dst, const Buf& b, size_t bytes,
                    const char* what) {
  if (bytes)
    MEXCT_TRY_CUDA(cudaMemcpyAsync(dst, b.p, bytes, cudaMemcpyDeviceToHost, c->stream), what);
  MEXCT_TRY_CUDA(cudaStreamSynchronize(c->stream), what);
  return MEXCT_OK;
}

// ---------------------------------------------------------------------------
// FP
// ---------------------------------------------------------------------------
mexct_status fp_tex(mexct_ctx* c, const float* d_vol, int W, int H, int geom,
                    RayArgs& a, const float* angles, int nP, float* d_out,
                    cudaStream_t st) {
  if (!c->tex_arr || c->tex_w != W || c->tex_h != H) {
    if (c->tex) cudaDestroyTextureObject(c->tex);
    if (c->tex_arr) cudaFreeArray(c->tex_arr);
    c->tex = 0;
    c->tex_arr = nullptr;
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float>();
    MEXCT_TRY_CUDA(cudaMalloc3DArray(&c->tex_arr, &ch, make_cudaExtent(W, W, H), 0),
                   "fp(texture): 3D array");
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof rd);
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = c->tex_arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof td);
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    MEXCT_TRY_CUDA(cudaCreateTextureObject(&c->tex, &rd, &td, nullptr),
                   "fp(texture): texture object");
    c->tex_w = W;
    c->tex_h = H;
  }
  cudaMemcpy3DParms p;
  std::memset(&p, 0, sizeof p);
  p.srcPtr = make_cudaPitchedPtr((void*)d_vol, (size_t)W * sizeof(float), W, W);
  p.dstArray = c->tex_arr;
  p.extent = make_cudaExtent(W, W, H);
  p.kind = cudaMemcpyDeviceToDevice;
  MEXCT_TRY_CUDA(cudaMemcpy3DAsync(&p, st), "fp(texture): copy to array");
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    a.nviews = std::min(kMaxViews, nP - v0);
    a.view0 = v0;
    for (int i = 0; i < a.nviews; ++i) trig_of(angles[v0 + i], &a.trig[i]);
    MEXCT_TRY_CUDA(launch_fp_tex(geom, a, c->tex, d_out, st), "fp(texture): launch");
  }
  return MEXCT_OK;
}

}  // namespace

namespace mexct {
// Padded copies of a W x W x H volume in both layouts (clamp: replicated edge;
// border: zeros) in the given buffers, and TMA maps over them.
mexct_status prepare_slab_bufs(Buf& px, Buf& py, Buf& err, const void* d_vol, int vt, int W,
                               int H, bool border, int geom, CUtensorMap* mx, CUtensorMap* my,
                               int* Pf_out, cudaStream_t st) {
  const int Pf = slab_pitch(W);
  const size_t bytes = (size_t)Pf * (W + 2) * (H + 2) * dsize(vt);
  MEXCT_TRY_CUDA(px.ensure(bytes), "fp: workspace");
  MEXCT_TRY_CUDA(py.ensure(bytes), "fp: workspace");
  if (!err.p) {
    MEXCT_TRY_CUDA(err.ensure(64), "fp: workspace");
    MEXCT_TRY_CUDA(cudaMemset(err.p, 0, 64), "fp: workspace");
  }
  MEXCT_TRY_CUDA(launch_pad_volume(d_vol, vt, W, H, Pf, border, px.p, py.p, st),
                 "fp: pad volume");
  MEXCT_TRY_CUDA(make_slab_tmap(mx, px.p, vt, Pf, W + 2, H + 2, geom), "fp: tensor map");
  MEXCT_TRY_CUDA(make_slab_tmap(my, py.p, vt, Pf, W + 2, H + 2, geom), "fp: tensor map");
  *Pf_out = Pf;
  return MEXCT_OK;
}

mexct_status prepare_slab(mexct_ctx* c, const void* d_vol, int vt, int W, int H,
                          bool border, int geom, CUtensorMap* mx, CUtensorMap* my, int* Pf_out,
                          cudaStream_t st) {
  return prepare_slab_bufs(c->padx, c->pady, c->err, d_vol, vt, W, H, border, geom, mx, my,
                           Pf_out, st);
}

// The context's copy stream (created on first use).
cudaError_t copy_stream(mexct_ctx* c, cudaStream_t* out) {
  if (!c->copy_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    for (cudaEvent_t& ev : c->chunk_ev) {
      e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e != cudaSuccess) return e;
    }
    for (cudaEvent_t& ev : c->feed_ev) {
      e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e != cudaSuccess) return e;
    }
  }
  *out = c->copy_stream;
  return cudaSuccess;
}
}  // namespace mexct

namespace {

}  // namespace

namespace mexct {

// FP with a concrete variant (EXPLICIT, RAY or TEXTURE); arguments checked.
mexct_status fp_run(mexct_ctx* c, const void* d_vol, int vt, int W, int H, float sad,
                    const float* angles, int nP, int geom, void* d_out, int ot, int variant,
                    cudaStream_t st, const ChunkHook* hook) {
  if (nP == 0) return MEXCT_OK;
  std::unique_ptr<RayArgs> a(new RayArgs);
  fill_std_rays(*a, W, H, sad, geom, false);
  if (variant == MEXCT_FP_TEXTURE) {
    if (vt != kF32 || ot != kF32)
      return set_err(MEXCT_ERR_UNSUPPORTED, "fp(texture): FP32 storage only");
    return fp_tex(c, (const float*)d_vol, W, H, geom, *a, angles, nP, (float*)d_out, st);
  }
  if (variant == MEXCT_FP_EXPLICIT) {
    CUtensorMap mx, my;
    int Pf = 0;
    mexct_status s = prepare_slab(c, d_vol, vt, W, H, false, geom, &mx, &my, &Pf, st);
    if (s) return s;
    SlabEpi e{nullptr, nullptr, nullptr, nullptr, c->err.as<unsigned>(), c->wait_us};
    // launches of at most kMaxViews views, or hook->chunks launches
    const int step = hook ? std::min(kMaxViews, (nP + hook->chunks - 1) / hook->chunks)
                          : kMaxViews;
    for (int v0 = 0, ci = 0; v0 < nP; v0 += step, ++ci) {
      a->nviews = std::min(step, nP - v0);
      a->view0 = v0;
      for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
      MEXCT_TRY_CUDA(launch_fp_slab(geom, false, false, *a, mx, my, c->padx.p, c->pady.p, Pf, vt,
                                    d_out, ot, e, st),
                     "fp: launch");
      if (hook)
        if (mexct_status s2 = hook->fn(ci, v0, a->nviews)) return s2;
    }
    return MEXCT_OK;
  }
  const size_t N = (size_t)W * W * H;
  MEXCT_TRY_CUDA(c->volT.ensure(N * dsize(vt)), "fp: workspace");
  MEXCT_TRY_CUDA(launch_transpose_xy(d_vol, c->volT.p, W, H, vt, st), "fp: transpose");
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    a->nviews = std::min(kMaxViews, nP - v0);
    a->view0 = v0;
    for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
    MEXCT_TRY_CUDA(launch_fp(geom, false, *a, d_vol, c->volT.p, vt, nullptr, d_out, ot, st),
                   "fp: launch");
  }
  return MEXCT_OK;
}

// BP with an explicit launch shape; arguments checked.  Views go through a
// padded copy (clamp frame) in chunks of kMaxViews.
mexct_status bp_run(mexct_ctx* c, const void* d_sino, int stype, int W, int H, int nP, float sad,
                    const float* angles, int geom, void* d_vol, int vt, const BpShape& shp,
                    cudaStream_t st, const ChunkHook* hook, const ChunkHook* feed) {
  std::unique_ptr<VoxArgs> a(new VoxArgs);
  fill_vox(*a, W, H, sad);
  if (nP == 0) {
    MEXCT_TRY_CUDA(launch_fill(d_vol, vt, (long long)W * W * H, 0.f, st), "bp: zero");
    return MEXCT_OK;
  }
  if (!bp_shape_valid(shp)) return set_err(MEXCT_ERR_ARG, "bp: invalid launch shape");
  const int chunk = std::min(nP, kMaxViews);
  // every view in the quad layout: one 16-byte load per voxel and view (cone)
  // or per z pair of voxels (par / fan) for FP32 views, 8 bytes for FP16 / BF16
  const size_t es = 4 * dsize(stype);
  MEXCT_TRY_CUDA(c->spad.ensure_async(sino_pad_elems(W, H, chunk) * es, st), "bp: workspace");
  const size_t N = (size_t)W * W * H;
  if (shp.vblocks > 1)
    MEXCT_TRY_CUDA(c->bpart.ensure_async(N * shp.vblocks * sizeof(float), st), "bp: workspace");
  const size_t P = (size_t)W * H;
  const size_t vpad = sino_pad_elems(W, H, 1) * es;  // bytes of one laid-out view
  // one view chunk and one view block: the z split (hook) and the view parts
  // (feed) keep each voxel's operations those of one launch
  const bool single = nP <= kMaxViews && shp.vblocks == 1;
  const bool zsplit = hook && single;
  const int nparts = feed && single ? std::min(4, std::max(1, feed->chunks)) : 1;
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    const int nv = std::min(kMaxViews, nP - v0);
    for (int part = 0; part < nparts; ++part) {
      // parts of 1/16, 3/16, 1/4 and 1/2 of the views: the first, whose
      // upload nothing hides, is small
      static const int kEnd[4] = {1, 4, 8, 16};
      const int s0 = part == 0 ? 0 : (int)((long long)nv * kEnd[part - 1] / 16);
      const int s1 = nparts == 1 || part == nparts - 1 ? nv : (int)((long long)nv * kEnd[part] / 16);
      if (s1 <= s0) continue;
      if (nparts > 1)
        if (mexct_status s2 = feed->fn(part, v0 + s0, s1 - s0)) return s2;
      a->nviews = s1 - s0;
      a->view0 = 0;
      for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + s0 + i], &a->trig[i]);
      const char* src = static_cast<const char*>(d_sino) + (size_t)(v0 + s0) * P * dsize(stype);
      void* lay = static_cast<char*>(c->spad.p) + (size_t)s0 * vpad;
      MEXCT_TRY_CUDA(launch_pad_sino_quad(src, stype, W, H, a->nviews, lay, st), "bp: pad");
      // z ranges of the volume in hook->chunks launches for the last part
      const bool zs = zsplit && part == nparts - 1;
      const int nzb = (H + shp.zc - 1) / shp.zc;
      const int zstep = zs ? (nzb + hook->chunks - 1) / hook->chunks : nzb;
      const bool accum = v0 > 0 || s0 > 0;
      for (int zb = 0, ci = 0; zb < nzb; zb += zstep, ++ci) {
        BpShape sh = shp;
        sh.zb0 = zb;
        sh.nzb = zs ? zstep : 0;
        MEXCT_TRY_CUDA(launch_bp_quad(geom, *a, lay, stype, d_vol, vt, accum, sh,
                                      c->bpart.as<float>(), st),
                       "bp: launch");
        if (zs) {
          const int z0 = zb * shp.zc;
          if (mexct_status s2 = hook->fn(ci, z0, std::min(H, z0 + zstep * shp.zc) - z0))
            return s2;
        }
      }
    }
  }
  return MEXCT_OK;
}

}  // namespace mexct

namespace {

mexct_status fp_dev_impl(mexct_ctx* c, const void* d_vol, int vt, int W,
                         int H, float sad, const float* angles, int nP,
                         int geom, void* d_out, int ot, int variant,
                         cudaStream_t st) {
  // With nP == 0 there is no output and no angle to read (an empty MATLAB array
  // may come with a NULL data pointer).
  if (!d_vol || (nP > 0 && (!d_out || !angles))) return set_err(MEXCT_ERR_ARG, "fp: NULL pointer");
  if (bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "fp: bad volume dims %d x %d x %d", W, W, H);
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "fp: nProj must be >= 0 (got %d)", nP);
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "fp: invalid geometry %d", geom);
  if (bad_type(vt) || bad_type(ot)) return set_err(MEXCT_ERR_ARG, "fp: bad storage type");
  if (variant != MEXCT_FP_EXPLICIT && variant != MEXCT_FP_TEXTURE && variant != MEXCT_FP_RAY &&
      variant != MEXCT_FP_AUTO)
    return set_err(MEXCT_ERR_ARG, "fp: unknown variant %d", variant);
  if (!c || nP == 0) return MEXCT_OK;  // c == NULL: validate only
  if (variant == MEXCT_FP_AUTO) {
    mexct_shape shp;
    mexct_status s = pick_fp_shape(c, d_vol, vt, W, H, sad, angles, nP, geom, d_out, ot, st,
                                   &shp);
    if (s) return s;
    variant = shp.variant;
  }
  return fp_run(c, d_vol, vt, W, H, sad, angles, nP, geom, d_out, ot, variant, st);
}

// ---------------------------------------------------------------------------
// BP
// ---------------------------------------------------------------------------
mexct_status bp_dev_impl(mexct_ctx* c, const void* d_sino, int stype, int W,
                         int H, int nP, float sad, const float* angles,
                         int geom, void* d_vol, int vt, cudaStream_t st) {
  if (!d_vol || (nP > 0 && (!d_sino || !angles))) return set_err(MEXCT_ERR_ARG, "bp: NULL pointer");
  if (bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "bp: bad sinogram dims %d x %d", W, H);
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "bp: bad view count %d", nP);
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "bp: invalid geometry %d", geom);
  if (bad_type(stype) || bad_type(vt)) return set_err(MEXCT_ERR_ARG, "bp: bad storage type");
  if (!c) return MEXCT_OK;  // validate only
  mexct_shape shp{MEXCT_FP_EXPLICIT, 16, 8, 1};
  if (nP > 0) {
    mexct_status s = pick_bp_shape(c, d_sino, stype, W, H, nP, sad, angles, geom, d_vol, vt, st,
                                   &shp);
    if (s) return s;
  }
  return bp_run(c, d_sino, stype, W, H, nP, sad, angles, geom, d_vol, vt,
                BpShape{shp.zc, shp.rows, shp.vblocks}, st);
}

// ---------------------------------------------------------------------------
// Decoupled detector
// ---------------------------------------------------------------------------
mexct_status bad_detector(const mexct_detector* d, const char* op) {
  if (!d) return set_err(MEXCT_ERR_ARG, "%s: NULL detector", op);
  if (d->det_w < 1 || d->det_h < 1 || d->det_w > 32768 || d->det_h > 32768)
    return set_err(MEXCT_ERR_ARG, "%s: bad detector size %d x %d", op, d->det_w, d->det_h);
  if (!(d->du > 0.f) || !(d->dv > 0.f) || !std::isfinite(d->du) || !std::isfinite(d->dv))
    return set_err(MEXCT_ERR_ARG, "%s: detector pitch must be finite and > 0", op);
  if (d->ss < 1 || d->ss > 8)
    return set_err(MEXCT_ERR_ARG, "%s: rays per pixel side must be 1..8 (got %d)", op, d->ss);
  return MEXCT_OK;
}

// FP onto a det_w x det_h detector of pitch du x dv: the slab kernel with the
// rays through the pixel centres, or (ss > 1) once per sub-ray offset into a
// scratch sinogram whose views are averaged into the output.
mexct_status fp_det_impl(mexct_ctx* c, const float* d_vol, int W, int H, float sad,
                         const float* angles, int nP, int geom, const mexct_detector* det,
                         float* d_out, cudaStream_t st) {
  if (!d_vol || (nP > 0 && (!d_out || !angles))) return set_err(MEXCT_ERR_ARG, "fp: NULL pointer");
  if (bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "fp: bad volume dims %d x %d x %d", W, W, H);
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "fp: nProj must be >= 0 (got %d)", nP);
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "fp: invalid geometry %d", geom);
  if (mexct_status s = bad_detector(det, "fp")) return s;
  if (!c || nP == 0) return MEXCT_OK;
  std::unique_ptr<RayArgs> a(new RayArgs);
  fill_std_rays(*a, W, H, sad, geom, false);
  a->det_w = det->det_w;
  a->det_h = det->det_h;
  a->u0 = float(det->det_w - 1) / 2;
  a->v0 = float(det->det_h - 1) / 2;
  a->P = (long long)det->det_w * det->det_h;
  a->du = det->du;
  a->dv = det->dv;
  CUtensorMap mx, my;
  int Pf = 0;
  mexct_status s = prepare_slab(c, d_vol, kF32, W, H, false, geom, &mx, &my, &Pf, st);
  if (s) return s;
  const int ss = det->ss;
  const long long M = a->P * nP;
  float* dst = d_out;
  if (ss > 1) {
    MEXCT_TRY_CUDA(c->subs.ensure_async((size_t)M * sizeof(float), st), "fp: workspace");
    dst = c->subs.as<float>();
  }
  SlabEpi e{nullptr, nullptr, nullptr, nullptr, c->err.as<unsigned>(), c->wait_us};
  const float wsub = 1.0f / (float)(ss * ss);
  for (int sa = 0; sa < ss; ++sa) {
    for (int sb = 0; sb < ss; ++sb) {
      a->ou = ss == 1 ? 0.0f : ((float)sb + 0.5f) / (float)ss - 0.5f;
      a->ov = ss == 1 ? 0.0f : ((float)sa + 0.5f) / (float)ss - 0.5f;
      for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
        a->nviews = std::min(kMaxViews, nP - v0);
        a->view0 = v0;
        for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
        MEXCT_TRY_CUDA(launch_fp_slab_det(geom, *a, mx, my, c->padx.p, c->pady.p, Pf, dst, e, st),
                       "fp: launch");
      }
      if (ss > 1)
        MEXCT_TRY_CUDA(launch_add_scaled(dst, d_out, M, wsub, sa == 0 && sb == 0, st),
                       "fp: sub-ray mean");
    }
  }
  return MEXCT_OK;
}

// BP from a det_w x det_h detector of pitch du x dv.
mexct_status bp_det_impl(mexct_ctx* c, const float* d_sino, const mexct_detector* det, int nP,
                         float sad, const float* angles, int geom, int W, int H, float* d_vol,
                         cudaStream_t st) {
  if (!d_vol || (nP > 0 && (!d_sino || !angles))) return set_err(MEXCT_ERR_ARG, "bp: NULL pointer");
  if (bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "bp: bad volume dims %d x %d x %d", W, W, H);
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "bp: bad view count %d", nP);
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "bp: invalid geometry %d", geom);
  if (mexct_status s = bad_detector(det, "bp")) return s;
  if (!c) return MEXCT_OK;
  std::unique_ptr<VoxArgs> a(new VoxArgs);
  fill_vox(*a, W, H, sad);
  if (nP == 0) {
    MEXCT_TRY_CUDA(launch_fill(d_vol, kF32, (long long)W * W * H, 0.f, st), "bp: zero");
    return MEXCT_OK;
  }
  const int Wd = det->det_w, Hd = det->det_h;
  a->det_w = Wd;
  a->det_h = Hd;
  a->hwd = (float)(Wd / 2) - 1.0f;
  a->v0d = float(Hd - 1) / 2;
  a->inv_du = 1.0f / det->du;
  a->inv_dv = 1.0f / det->dv;
  a->P = (long long)Wd * Hd;
  const int chunk = std::min(nP, kMaxViews);
  MEXCT_TRY_CUDA(c->spad.ensure_async(sino_pad_elems(Wd, Hd, chunk) * sizeof(float4), st),
                 "bp: workspace");
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    a->nviews = std::min(kMaxViews, nP - v0);
    a->view0 = 0;
    for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
    MEXCT_TRY_CUDA(launch_pad_sino_quad(d_sino + (size_t)v0 * a->P, kF32, Wd, Hd, a->nviews,
                                        c->spad.p, st),
                   "bp: pad");
    MEXCT_TRY_CUDA(launch_bp_det(geom, *a, c->spad.p, d_vol, v0 > 0, st),
                   "bp: launch");
  }
  return MEXCT_OK;
}

// ---------------------------------------------------------------------------
// general3D
// ---------------------------------------------------------------------------
void fill_g3d(RayArgs& a, int S, int Z, int W, int H, int per_view) {
  std::memset(&a, 0, sizeof a);
  a.det_w = W;
  a.det_h = H;
  a.S = S;
  a.Z = Z;
  a.bx = -(float)S / 2.0f;  // CUDAmex_general3D_FP.cu:175-177
  a.by = a.bx;
  a.bz = -(float)Z / 2.0f;
  a.step = 0.5f;            // :132
  a.P = (long long)W * H;
  a.pts_per_view = per_view;
  a.vstride = 1;
  a.du = 1.0f;
  a.dv = 1.0f;
}

mexct_status g3d_fp_dev_impl(mexct_ctx* c, const float* d_vol, int S, int Z,
                             const float* angles, const float* d_pts, int W,
                             int H, int nP, int per_view, float* d_out,
                             cudaStream_t st) {
  if (!d_vol || !d_pts || !d_out || (!angles && nP > 0))
    return set_err(MEXCT_ERR_ARG, "g3d_fp: NULL pointer");
  if (bad_dims(S, Z) || bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "g3d_fp: bad dims");
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "g3d_fp: bad view count %d", nP);
  if (!c || nP == 0) return MEXCT_OK;  // c == NULL: validate only
  // the slab kernel over the zero-framed padded volume (border addressing)
  std::unique_ptr<RayArgs> a(new RayArgs);
  fill_g3d(*a, S, Z, W, H, per_view ? 1 : 0);
  a->pts = d_pts;
  CUtensorMap mx, my;
  int Pf = 0;
  mexct_status s = prepare_slab(c, d_vol, kF32, S, Z, /*border=*/true, /*geom=*/3, &mx, &my,
                                &Pf, st);
  if (s) return s;
  SlabEpi e{nullptr, nullptr, nullptr, nullptr, c->err.as<unsigned>(), c->wait_us};
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    a->nviews = std::min(kMaxViews, nP - v0);
    a->view0 = v0;
    for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
    MEXCT_TRY_CUDA(launch_fp_slab_g3d(*a, mx, my, c->padx.p, c->pady.p, Pf, d_out, e, st),
                   "g3d_fp: launch");
  }
  return MEXCT_OK;
}

mexct_status g3d_bp_dev_impl(mexct_ctx* c, const float* d_sino, int W, int H,
                             int nP, const float* angles, const float* d_pts,
                             int per_view, int S, int Z, float* d_vol,
                             cudaStream_t st) {
  if (!d_sino || !d_pts || !d_vol || (!angles && nP > 0))
    return set_err(MEXCT_ERR_ARG, "g3d_bp: NULL pointer");
  if (bad_dims(S, Z) || bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "g3d_bp: bad dims");
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "g3d_bp: bad view count %d", nP);
  if (!c) return MEXCT_OK;  // validate only
  MEXCT_TRY_CUDA(cudaMemsetAsync(d_vol, 0, (size_t)S * S * Z * sizeof(float), st), "g3d_bp: zero");
  std::unique_ptr<RayArgs> a(new RayArgs);
  fill_g3d(*a, S, Z, W, H, per_view ? 1 : 0);
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    a->nviews = std::min(kMaxViews, nP - v0);
    a->view0 = v0;
    for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
    MEXCT_TRY_CUDA(launch_g3d_bp(*a, d_sino, d_pts, d_vol, st), "g3d_bp: launch");
  }
  return MEXCT_OK;
}

// OSC iteration onto a decoupled detector (no counterpart in the reference,
// whose detector is the volume's face): pre/post are det_w x det_h x nP; the
// forward pass casts one ray per pixel centre (ss must be 1) and the dual BP
// interpolates the residuals bilinearly in u and v.  FP32 mu.
mexct_status osc_det_impl(mexct_ctx* c, float* d_mu, const float* d_pre, const float* d_post,
                          const mexct_detector* det, int W, int H, int nP, int nSub,
                          const int32_t* picks, const float* angles, float sad, int geom,
                          cudaStream_t st) {
  if (!d_mu || !d_pre || !d_post || !picks || (!angles && nP > 0))
    return set_err(MEXCT_ERR_ARG, "osc_iter_det: NULL pointer");
  if (bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "osc_iter_det: bad dims");
  if (nP < 0 || nSub <= 0)
    return set_err(MEXCT_ERR_ARG, "osc_iter_det: bad nProj %d / nSub %d", nP, nSub);
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "osc_iter_det: invalid geometry %d", geom);
  if (mexct_status s = bad_detector(det, "osc_iter_det")) return s;
  if (det->ss != 1)
    return set_err(MEXCT_ERR_UNSUPPORTED, "osc_iter_det: ss = %d (one ray per pixel only)", det->ss);
  int maxv = 0;
  for (int si = 0; si < nSub; ++si) {
    const int sel = picks[si];
    const int nv = (sel < 0 || sel >= nP) ? 0 : (nP - 1 - sel) / nSub + 1;
    maxv = std::max(maxv, nv);
  }
  if (maxv > kMaxViews)
    return set_err(MEXCT_ERR_UNSUPPORTED, "osc_iter_det: %d views in one subset (max %d)", maxv,
                   kMaxViews);
  if (!c) return MEXCT_OK;
  const int Wd = det->det_w, Hd = det->det_h;
  const size_t rbytes = sino_pad_elems(Wd, Hd, std::max(maxv, 1)) * sizeof(float4);
  MEXCT_TRY_CUDA(c->r1.ensure(rbytes), "osc_iter_det: workspace");
  MEXCT_TRY_CUDA(c->r2.ensure(rbytes), "osc_iter_det: workspace");
  MEXCT_TRY_CUDA(cudaMemsetAsync(c->r1.p, 0, rbytes, st), "osc_iter_det: workspace");
  MEXCT_TRY_CUDA(cudaMemsetAsync(c->r2.p, 0, rbytes, st), "osc_iter_det: workspace");
  CUtensorMap mx, my;
  int Pf = 0;
  mexct_status ps = prepare_slab(c, d_mu, kF32, W, H, /*border=*/true, geom, &mx, &my, &Pf, st);
  if (ps) return ps;
  std::unique_ptr<RayArgs> ra(new RayArgs);
  std::unique_ptr<VoxArgs> va(new VoxArgs);
  fill_std_rays(*ra, W, H, sad, geom, /*osc=*/true);
  ra->det_w = Wd;
  ra->det_h = Hd;
  ra->u0 = float(Wd - 1) / 2;
  ra->v0 = float(Hd - 1) / 2;
  ra->P = (long long)Wd * Hd;
  ra->du = det->du;
  ra->dv = det->dv;
  fill_vox(*va, W, H, sad);
  va->det_w = Wd;
  va->det_h = Hd;
  va->hwd = (float)(Wd / 2) - 1.0f;
  va->v0d = float(Hd - 1) / 2;
  va->inv_du = 1.0f / det->du;
  va->inv_dv = 1.0f / det->dv;
  va->P = (long long)Wd * Hd;
  for (int si = 0; si < nSub; ++si) {
    const int sel = picks[si];
    const int nv = (sel < 0 || sel >= nP) ? 0 : (nP - 1 - sel) / nSub + 1;
    ra->nviews = nv;
    ra->view0 = sel;
    ra->vstride = nSub;
    va->nviews = nv;
    for (int i = 0; i < nv; ++i) {
      trig_of(angles[sel + i * nSub], &ra->trig[i]);
      va->trig[i] = ra->trig[i];
    }
    if (nv > 0) {
      SlabEpi e{d_pre, d_post, c->r1.as<float>(), c->r2.as<float>(), c->err.as<unsigned>(),
                c->wait_us};
      MEXCT_TRY_CUDA(launch_fp_slab_osc_det(geom, *ra, mx, my, c->padx.p, c->pady.p, Pf, e, st),
                     "osc_iter_det: fp");
    }
    MEXCT_TRY_CUDA(launch_osc_bp_update_det(geom, *va, c->r1.as<float>(), c->r2.as<float>(), d_mu,
                                            kF32, c->padx.p, c->pady.p, Pf, st),
                   "osc_iter_det: bp/update");
  }
  return MEXCT_OK;
}

// Matched-adjoint general3D BP: the transpose of g3d_fp_dev_impl.
mexct_status g3d_bp_matched_impl(mexct_ctx* c, const float* d_sino, int W, int H, int nP,
                                 const float* angles, const float* d_pts, int per_view, int S,
                                 int Z, float* d_vol, cudaStream_t st) {
  if (!d_sino || !d_pts || !d_vol || (!angles && nP > 0))
    return set_err(MEXCT_ERR_ARG, "g3d_bp_matched: NULL pointer");
  if (bad_dims(S, Z) || bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "g3d_bp_matched: bad dims");
  if (nP < 0) return set_err(MEXCT_ERR_ARG, "g3d_bp_matched: bad view count %d", nP);
  if (!c) return MEXCT_OK;  // validate only
  MEXCT_TRY_CUDA(cudaMemsetAsync(d_vol, 0, (size_t)S * S * Z * sizeof(float), st),
                 "g3d_bp_matched: zero");
  std::unique_ptr<RayArgs> a(new RayArgs);
  fill_g3d(*a, S, Z, W, H, per_view ? 1 : 0);
  for (int v0 = 0; v0 < nP; v0 += kMaxViews) {
    a->nviews = std::min(kMaxViews, nP - v0);
    a->view0 = v0;
    for (int i = 0; i < a->nviews; ++i) trig_of(angles[v0 + i], &a->trig[i]);
    MEXCT_TRY_CUDA(launch_g3d_bp_adjoint(*a, d_sino, d_pts, d_vol, st), "g3d_bp_matched: launch");
  }
  return MEXCT_OK;
}

// ---------------------------------------------------------------------------
// OSC iteration (CUDAmex_oscIter.cu:504-557): per subset, the fused FP +
// residual over the subset's views, then the fused dual BP + update.
// ---------------------------------------------------------------------------
mexct_status osc_dev_impl(mexct_ctx* c, float* d_mu, int mu_type,
                          const float* d_pre, const float* d_post, int W,
                          int H, int nP, int nSub, const int32_t* picks,
                          const float* angles, float sad, int geom,
                          cudaStream_t st) {
  if (!d_mu || !d_pre || !d_post || !picks || (!angles && nP > 0))
    return set_err(MEXCT_ERR_ARG, "osc_iter: NULL pointer");
  if (bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "osc_iter: bad dims");
  if (nP < 0 || nSub <= 0) return set_err(MEXCT_ERR_ARG, "osc_iter: bad nProj %d / nSub %d", nP, nSub);
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "osc_iter: invalid geometry %d", geom);
  if (bad_type(mu_type)) return set_err(MEXCT_ERR_ARG, "osc_iter: bad storage type");
  const size_t N = (size_t)W * W * H;
  const size_t P = (size_t)W * H;
  int maxv = 0;
  for (int si = 0; si < nSub; ++si) {
    const int sel = picks[si];
    const int nv = (sel < 0 || sel >= nP) ? 0 : (nP - 1 - sel) / nSub + 1;
    maxv = std::max(maxv, nv);
  }
  if (maxv > kMaxViews)
    return set_err(MEXCT_ERR_UNSUPPORTED, "osc_iter: %d views in one subset (max %d)", maxv, kMaxViews);
  if (!c) return MEXCT_OK;  // validate only
  (void)N;
  (void)P;
  // Residual views in the padded quad layout (4 floats per texel) with a zero
  // frame (border addressing).
  const size_t rbytes = sino_pad_elems(W, H, std::max(maxv, 1)) * sizeof(float4);
  MEXCT_TRY_CUDA(c->r1.ensure(rbytes), "osc_iter: workspace");
  MEXCT_TRY_CUDA(c->r2.ensure(rbytes), "osc_iter: workspace");
  MEXCT_TRY_CUDA(cudaMemsetAsync(c->r1.p, 0, rbytes, st), "osc_iter: workspace");
  MEXCT_TRY_CUDA(cudaMemsetAsync(c->r2.p, 0, rbytes, st), "osc_iter: workspace");
  // mu is padded (zero frame) once; every subset update rewrites the padded
  // copies along with mu.
  CUtensorMap mx, my;
  int Pf = 0;
  mexct_status ps = prepare_slab(c, d_mu, mu_type, W, H, /*border=*/true, geom, &mx, &my, &Pf, st);
  if (ps) return ps;
  std::unique_ptr<RayArgs> ra(new RayArgs);
  std::unique_ptr<VoxArgs> va(new VoxArgs);
  fill_std_rays(*ra, W, H, sad, geom, /*osc=*/true);
  fill_vox(*va, W, H, sad);
  for (int si = 0; si < nSub; ++si) {
    const int sel = picks[si];
    const int nv = (sel < 0 || sel >= nP) ? 0 : (nP - 1 - sel) / nSub + 1;
    ra->nviews = nv;
    ra->view0 = sel;
    ra->vstride = nSub;
    va->nviews = nv;
    for (int i = 0; i < nv; ++i) {
      trig_of(angles[sel + i * nSub], &ra->trig[i]);
      va->trig[i] = ra->trig[i];
    }
    if (nv > 0) {
      SlabEpi e{d_pre, d_post, c->r1.as<float>(), c->r2.as<float>(), c->err.as<unsigned>(),
                c->wait_us};
      MEXCT_TRY_CUDA(launch_fp_slab(geom, true, true, *ra, mx, my, c->padx.p, c->pady.p, Pf,
                                    mu_type, nullptr, kF32, e, st),
                     "osc_iter: fp");
    }
    // An empty subset still runs the update: num = den = 0 gives
    // max(mu + mu*0/0, 0) = 0 inside the circle, as in the reference.
    MEXCT_TRY_CUDA(launch_osc_bp_update(geom, *va, c->r1.as<float>(), c->r2.as<float>(),
                                        d_mu, mu_type, c->padx.p, c->pady.p, Pf, st),
                   "osc_iter: bp/update");
  }
  return MEXCT_OK;
}

// ---------------------------------------------------------------------------
// TV descent: n_steps of (norm, update) on a ping-pong pair whose last write
// lands in d_out.
// ---------------------------------------------------------------------------
mexct_status tv_dev_impl(mexct_ctx* c, const void* d_in, int t, int Nx,
                         int Ny, int Nz, float cval, int n_steps,
                         void* d_out, cudaStream_t st) {
  if (!d_in || !d_out) return set_err(MEXCT_ERR_ARG, "tvmin3d: NULL pointer");
  if (Nx <= 0 || Ny <= 0 || Nz <= 0) return set_err(MEXCT_ERR_ARG, "tvmin3d: bad dims");
  if (n_steps < 0) return set_err(MEXCT_ERR_ARG, "tvmin3d: n_steps < 0");
  if (bad_type(t)) return set_err(MEXCT_ERR_ARG, "tvmin3d: bad storage type");
  if (!tv_shape_launchable(Nx, Ny, Nz))
    return set_err(MEXCT_ERR_UNSUPPORTED, "tvmin3d: %d x %d x %d exceeds the launch grid limits",
                   Nx, Ny, Nz);
  if (!c) return MEXCT_OK;  // validate only
  const size_t N = (size_t)Nx * Ny * Nz;
  const size_t bytes = N * dsize(t);
  if (n_steps == 0) {
    if (d_in != d_out)
      MEXCT_TRY_CUDA(cudaMemcpyAsync(d_out, d_in, bytes, cudaMemcpyDeviceToDevice, st), "tvmin3d: copy");
    return MEXCT_OK;
  }
  MEXCT_TRY_CUDA(ensure_reduction(c, tv_partials_needed(Nx, Ny, Nz)), "tvmin3d: workspace");
  MEXCT_TRY_CUDA(c->r1.ensure(bytes), "tvmin3d: workspace");
  const void* src = d_in;
  if (d_in == d_out && (n_steps % 2) == 1) {
    // The first write would land on the input: read it from a copy.
    MEXCT_TRY_CUDA(c->r2.ensure(bytes), "tvmin3d: workspace");
    MEXCT_TRY_CUDA(cudaMemcpyAsync(c->r2.p, d_in, bytes, cudaMemcpyDeviceToDevice, st), "tvmin3d: copy");
    src = c->r2.p;
  }
  float* scale = c->scal.as<float>();
  double* norm = reinterpret_cast<double*>(c->scal.as<char>() + 8);
  for (int k = 0; k < n_steps; ++k) {
    void* dst = ((n_steps - 1 - k) % 2 == 0) ? d_out : c->r1.p;
    MEXCT_TRY_CUDA(launch_tv_norm(src, t, Nx, Ny, Nz, cval, c->red.as<double>(),
                                  c->cnt.as<unsigned>(), scale, norm, st),
                   "tvmin3d: norm");
    MEXCT_TRY_CUDA(launch_tv_update(src, dst, t, Nx, Ny, Nz, scale, st), "tvmin3d: update");
    src = dst;
  }
  return MEXCT_OK;
}

// ---------------------------------------------------------------------------
// Pre-filter tables: designFilter (preFilterSinogram.m:95-152) -> spatial
// kernel real(ifft(H)); Parker window (parker_weight.m:181-240); dbeta/2.
// ---------------------------------------------------------------------------
int filter_order(int W) {
  int order = 64;
  while (order < 2 * W) order *= 2;  // max(64, 2^nextpow2(2*len))
  return order;
}

void filter_kernel(int W, int filter, double d, std::vector<float>& out) {
  const double pi = 3.14159265358979323846;
  const int order = filter_order(W), half = order / 2;
  std::vector<double> ct(order);
  for (int i = 0; i < order; ++i) ct[i] = std::cos(2.0 * pi * i / order);
  std::vector<double> H(order, 1.0);
  if (filter != 0) {
    std::vector<double> h(order, 0.0);
    h[0] = 0.25;  // DC term
    for (int n = 1; n <= half; n += 2) {
      const double v = -1.0 / ((pi * n) * (pi * n));
      h[n] = v;
      if (n < half) h[order - n] = v;
    }
    std::vector<double> filt(half + 1);
    for (int m = 0; m <= half; ++m) {
      double acc = 0.0;
      for (int n = 0; n < order; ++n) acc += h[n] * ct[((long long)m * n) % order];
      filt[m] = 2.0 * acc;
    }
    for (int m = 1; m <= half; ++m) {
      const double w = 2.0 * pi * m / order;
      if (filter == 2) filt[m] *= std::sin(w / (2 * d)) / (w / (2 * d));
      else if (filter == 3) filt[m] *= std::cos(w / (2 * d));
      else if (filter == 4) filt[m] *= (.54 + .46 * std::cos(w / d));
      else if (filter == 5) filt[m] *= (1 + std::cos(w / d)) / 2;
    }
    for (int m = 0; m <= half; ++m)
      if (2.0 * pi * m / order > pi * d) filt[m] = 0.0;
    for (int m = 0; m <= half; ++m) H[m] = filt[m];
    for (int m = 1; m < half; ++m) H[half + m] = filt[half - m];
  }
  out.assign(order, 0.f);
  for (int n = 0; n < order; ++n) {
    double acc = 0.0;
    for (int m = 0; m < order; ++m) acc += H[m] * ct[((long long)m * n) % order];
    out[n] = (float)(acc / order);
  }
}

double s_window(double b) {
  if (std::fabs(b) < 0.5) return 0.5 * (1 + std::sin(3.14159265358979323846 * b));
  if (b >= 0.5) return 1.0;
  return 0.0;
}

mexct_status prefilter_tables(mexct_ctx* c, int W, int H, int nP, const float* angles, int geom,
                              float sad, int filter, float cutoff, float q, int order,
                              cudaStream_t st);

// The (modified) Parker window of parker_weight.m:29-72 per view i and row
// element u of a W x W detector, in FP64, stored as single as the reference
// does (:72): fan / cone angle alpha_u = atan((u - W/2 + 1/2) / SAD) (0 for
// parallel rays, :29-32), negated when the angles increase (:36-39); delta
// half the fan angle, epsilon the overscan beyond pi + 2 delta (:42-59); the
// window is the Wesarg et al. sum of four S terms of b = q (2 delta - 2 alpha
// + epsilon) (:64-70, :81-99).
void parker_table(int W, int nP, const float* angles, int geom, double sad, double q,
                  float* out) {
  const double pi = 3.14159265358979323846;
  std::vector<double> alpha(W, 0.0);
  if (geom != 0)
    for (int j = 0; j < W; ++j) alpha[j] = std::atan((-W / 2.0 + 0.5 + j) / sad);
  bool incr = true;
  for (int i = 1; i < nP; ++i)
    if (!(angles[i] - angles[i - 1] >= 0)) incr = false;
  if (incr)
    for (double& a : alpha) a = -a;
  const double delta = std::fabs(alpha[W - 1] - alpha[0]) / 2;
  const double extent = nP > 0 ? std::fabs((double)(angles[nP - 1] - angles[0])) : 0.0;
  const double eps = std::max(extent - (pi + 2 * delta), 0.0);
  auto b2 = [&](double a) { return q * (2 * delta - 2 * a + eps); };
  for (int i = 0; i < nP; ++i) {
    const double beta = std::fabs((double)(angles[i] - angles[0]));
    for (int j = 0; j < W; ++j) {
      const double a = alpha[j];
      out[(size_t)i * W + j] = (float)(
          0.5 * (s_window(beta / b2(a) - 0.5) +
                 s_window((beta - 2 * delta + 2 * a - eps) / b2(a) + 0.5) -
                 s_window((beta - pi + 2 * a) / b2(-a) - 0.5) -
                 s_window((beta - pi - 2 * delta - eps) / b2(-a) + 0.5)));
    }
  }
}

mexct_status prefilter_dev_impl(mexct_ctx* c, const float* d_sino,
                                const float* d_pre, int W, int H, int nP,
                                const float* angles, int geom, float sad,
                                int filter, float cutoff, float q,
                                float* d_out, cudaStream_t st) {
  if (!d_sino || !d_out || !angles) return set_err(MEXCT_ERR_ARG, "prefilter: NULL pointer");
  if (bad_dims(W, H)) return set_err(MEXCT_ERR_ARG, "prefilter: bad dims");
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "prefilter: invalid geometry %d", geom);
  if (filter < 0 || filter > 5) return set_err(MEXCT_ERR_ARG, "prefilter: unknown filter %d", filter);
  if (nP < 2) return set_err(MEXCT_ERR_ARG, "prefilter: needs at least 2 views (dbeta)");
  if (W != H)
    return set_err(MEXCT_ERR_UNSUPPORTED,
                   "prefilter: W (%d) != H (%d); the Parker weighting of the reference "
                   "(parker_weight.m:225) needs a square detector", W, H);
  if (!c) return MEXCT_OK;  // validate only
  const int order = filter_order(W);
  mexct_ctx::TabKey key;
  key.W = W;
  key.H = H;
  key.nP = nP;
  key.geom = geom;
  key.filter = filter;
  key.sad = sad;
  key.cutoff = cutoff;
  key.q = q;
  key.angles.assign(angles, angles + nP);
  if (!(c->tab_buf && c->tab_buf == c->tabs.p && c->tab_key == key)) {
    mexct_status s = prefilter_tables(c, W, H, nP, angles, geom, sad, filter, cutoff, q, order,
                                      st);
    if (s) return s;
    c->tab_key = std::move(key);
    c->tab_buf = c->tabs.p;
  }
  FiltArgs fa;
  fa.W = W;
  fa.H = H;
  fa.nP = nP;
  fa.order = order;
  fa.geom = geom;
  fa.log_input = d_pre ? 1 : 0;
  fa.sad = sad;
  const float* dt = c->tabs.as<float>();
  MEXCT_TRY_CUDA(launch_prefilter(fa, d_sino, d_pre, dt + order, dt + order + (size_t)nP * W, dt,
                                  d_out, st),
                 "prefilter: launch");
  return MEXCT_OK;
}

// Filter kernel, Parker window per (view, row element) and dbeta/2 per view,
// computed on the host in FP64 and copied to the context's tables.
mexct_status prefilter_tables(mexct_ctx* c, int W, int H, int nP, const float* angles, int geom,
                              float sad, int filter, float cutoff, float q, int order,
                              cudaStream_t st) {
  const double pi = 3.14159265358979323846;
  if (c->filt_w != W || c->filt_type != filter || c->filt_cut != cutoff) {
    filter_kernel(W, filter, cutoff, c->filt_kern);
    c->filt_w = W;
    c->filt_type = filter;
    c->filt_cut = cutoff;
  }
  // Parker window per (view, row element) and dbeta/2 per view.
  (void)pi;
  std::vector<float> tab((size_t)order + (size_t)nP * W + nP);
  std::memcpy(tab.data(), c->filt_kern.data(), sizeof(float) * order);
  float* parker = tab.data() + order;
  float* dbeta = parker + (size_t)nP * W;
  parker_table(W, nP, angles, geom, sad, q, parker);
  for (int i = 0; i < nP; ++i)
    dbeta[i] = (i > 0) ? (angles[i] - angles[i - 1]) / 2 : (angles[1] - angles[0]) / 2;
  MEXCT_TRY_CUDA(c->tabs.ensure(tab.size() * sizeof(float)), "prefilter: workspace");
  // from a pageable host vector: cudaMemcpyAsync returns once the bytes are
  // staged, so the vector may go out of scope
  MEXCT_TRY_CUDA(cudaMemcpyAsync(c->tabs.p, tab.data(), tab.size() * sizeof(float),
                                 cudaMemcpyHostToDevice, st),
                 "prefilter: tables");
  return MEXCT_OK;
}


// Downloads of the chunks recorded by a ChunkHook: chunk i waits for its
// event and copies `bytes` from d + off to h + off on the copy stream.  All
// launches are enqueued before the first copy (a pageable destination makes
// the copy call wait), then both streams are drained.
struct ChunkCopies {
  struct Item { size_t off, bytes; };
  std::vector<Item> items;
  mexct_status run(mexct_ctx* c, cudaStream_t cs, void* h, const void* d, const char* what) {
    for (size_t i = 0; i < items.size(); ++i) {
      MEXCT_TRY_CUDA(cudaStreamWaitEvent(cs, c->chunk_ev[i], 0), what);
      MEXCT_TRY_CUDA(cudaMemcpyAsync(static_cast<char*>(h) + items[i].off,
                                     static_cast<const char*>(d) + items[i].off, items[i].bytes,
                                     cudaMemcpyDeviceToHost, cs),
                     what);
    }
    MEXCT_TRY_CUDA(cudaStreamSynchronize(cs), what);
    MEXCT_TRY_CUDA(cudaStreamSynchronize(c->stream), what);
    return MEXCT_OK;
  }
};

// z ranges of the host BP's downloads
constexpr int kHostChunks = 8;
// view chunks of the host FP: each launch boundary costs part of a wave (one
// 512^3 x 720-view cone FP on a GB300: 178.5 ms in one launch, 181.3 in 4,
// 185.1 in 8), the last chunk's download is exposed; 4 balances the two
constexpr int kFpHostChunks = 4;

mexct_status fp_host_overlapped(mexct_ctx* c, int W, int H, float sad, const float* angles,
                                int nP, int geom, float* out) {
  cudaStream_t cs;
  MEXCT_TRY_CUDA(copy_stream(c, &cs), "fp: copy stream");
  const size_t P = (size_t)W * H;
  ChunkCopies cc;
  ChunkHook hook{kFpHostChunks, [&](int i, int v0, int n) -> mexct_status {
                   if (i >= kFpHostChunks) return set_err(MEXCT_ERR_ARG, "fp: too many chunks");
                   MEXCT_TRY_CUDA(cudaEventRecord(c->chunk_ev[i], c->stream), "fp: event");
                   cc.items.push_back({(size_t)v0 * P * 4, (size_t)n * P * 4});
                   return MEXCT_OK;
                 }};
  mexct_status s = fp_run(c, c->in.p, kF32, W, H, sad, angles, nP, geom, c->out.p, kF32,
                          MEXCT_FP_EXPLICIT, c->stream, &hook);
  if (s) return s;
  return cc.run(c, cs, out, c->out.p, "fp: download");
}

// Host BP with the views uploaded in four parts on the copy stream, each
// part's BP starting once its views have landed (the later uploads overlap
// the earlier parts' launches), and the volume's z ranges downloaded as the
// last part's launches finish.  Bit-identical to one launch.
mexct_status bp_host_overlapped(mexct_ctx* c, const float* sino, int W, int H, int nP, float sad,
                                const float* angles, int geom, const BpShape& shp, float* vol) {
  cudaStream_t cs;
  MEXCT_TRY_CUDA(copy_stream(c, &cs), "bp: copy stream");
  const size_t slice = (size_t)W * W * 4, P = (size_t)W * H;
  // the copy stream writes c->in only after the launch stream's earlier work
  MEXCT_TRY_CUDA(cudaEventRecord(c->feed_ev[0], c->stream), "bp: event");
  MEXCT_TRY_CUDA(cudaStreamWaitEvent(cs, c->feed_ev[0], 0), "bp: event");
  int fed = 0;
  ChunkHook feed{4, [&](int i, int first, int count) -> mexct_status {
                   if (i >= 4) return set_err(MEXCT_ERR_ARG, "bp: too many view parts");
                   MEXCT_TRY_CUDA(cudaMemcpyAsync(c->in.as<float>() + (size_t)first * P,
                                                  sino + (size_t)first * P,
                                                  (size_t)count * P * 4, cudaMemcpyHostToDevice,
                                                  cs),
                                  "bp: upload");
                   MEXCT_TRY_CUDA(cudaEventRecord(c->feed_ev[i], cs), "bp: event");
                   MEXCT_TRY_CUDA(cudaStreamWaitEvent(c->stream, c->feed_ev[i], 0), "bp: event");
                   fed += count;
                   return MEXCT_OK;
                 }};
  ChunkCopies cc;
  ChunkHook hook{kHostChunks, [&](int i, int z0, int nz) -> mexct_status {
                   if (i >= kHostChunks) return set_err(MEXCT_ERR_ARG, "bp: too many chunks");
                   MEXCT_TRY_CUDA(cudaEventRecord(c->chunk_ev[i], c->stream), "bp: event");
                   cc.items.push_back({(size_t)z0 * slice, (size_t)nz * slice});
                   return MEXCT_OK;
                 }};
  mexct_status s = bp_run(c, c->in.p, kF32, W, H, nP, sad, angles, geom, c->out.p, kF32, shp,
                          c->stream, &hook, &feed);
  if (s) return s;
  if (fed != nP) return set_err(MEXCT_ERR_ARG, "bp: %d of %d views uploaded", fed, nP);
  if (cc.items.empty()) {  // the shape ran as one launch: plain download
    MEXCT_TRY_CUDA(cudaMemcpyAsync(vol, c->out.p, slice * H, cudaMemcpyDeviceToHost, c->stream),
                   "bp: download");
    MEXCT_TRY_CUDA(cudaStreamSynchronize(c->stream), "bp: download");
    MEXCT_TRY_CUDA(cudaStreamSynchronize(cs), "bp: upload");
    return MEXCT_OK;
  }
  return cc.run(c, cs, vol, c->out.p, "bp: download");
}

}  // namespace

// ===========================================================================
// Every entry point validates its arguments first (the impl functions with a
// NULL context only validate), then resolves the device context.
extern "C" {

#define VALIDATE(call)              \
  do {                              \
    mexct_status _v = (call);       \
    if (_v != MEXCT_OK) return _v;  \
  } while (0)

#define CTX_OR_FAIL(c, name)                                                \
  NvtxRange _nvtx("mexct:" name);                                           \
  mexct_ctx* c = resolve(ctx);                                              \
  if (!c) return set_err(MEXCT_ERR_CUDA, name ": no CUDA device / context"); \
  std::lock_guard<std::recursive_mutex> _lk(c->mu);                         \
  DevGuard _dg(c->device)

mexct_status mexct_fp_dev(mexct_ctx* ctx, const float* d_vol, int W, int H,
                          float sad, const float* angles, int nP, int geom,
                          float* d_out, void* stream) {
  VALIDATE(fp_dev_impl(nullptr, d_vol, kF32, W, H, sad, angles, nP, geom, d_out, kF32,
                       MEXCT_FP_AUTO, nullptr));
  CTX_OR_FAIL(c, "fp");
  return fp_dev_impl(c, d_vol, kF32, W, H, sad, angles, nP, geom, d_out, kF32,
                     MEXCT_FP_AUTO, as_stream(stream));
}

mexct_status mexct_fp_dev_ex(mexct_ctx* ctx, const void* d_vol, int vt, int W,
                             int H, float sad, const float* angles, int nP,
                             int geom, void* d_out, int ot, int variant,
                             void* stream) {
  VALIDATE(fp_dev_impl(nullptr, d_vol, vt, W, H, sad, angles, nP, geom, d_out, ot, variant,
                       nullptr));
  CTX_OR_FAIL(c, "fp");
  return fp_dev_impl(c, d_vol, vt, W, H, sad, angles, nP, geom, d_out, ot, variant,
                     as_stream(stream));
}

mexct_status mexct_fp(mexct_ctx* ctx, const float* vol, int W, int H,
                      float sad, const float* angles, int nP, int geom,
                      float* out) {
  VALIDATE(fp_dev_impl(nullptr, vol, kF32, W, H, sad, angles, nP, geom, out, kF32,
                       MEXCT_FP_AUTO, nullptr));
  CTX_OR_FAIL(c, "fp");
  const size_t N = (size_t)W * W * H, M = (size_t)W * H * nP;
  mexct_status s = upload(c->in, vol, N * 4, c->stream, "fp: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->out.ensure_async(M * 4, c->stream), "fp: workspace");
  if (nP >= 16 && nP <= kFpHostChunks * kMaxViews && M * 4 >= ((size_t)64 << 20)) {
    // the slab FP in view chunks, each chunk's download overlapping the
    // launches after it (same result as one launch: rays are independent)
    mexct_shape shp;
    s = pick_fp_shape(c, c->in.p, kF32, W, H, sad, angles, nP, geom, c->out.p, kF32, c->stream,
                      &shp);
    if (s) return s;
    if (shp.variant == MEXCT_FP_EXPLICIT) return fp_host_overlapped(c, W, H, sad, angles, nP,
                                                                    geom, out);
  }
  s = fp_dev_impl(c, c->in.p, kF32, W, H, sad, angles, nP, geom, c->out.p, kF32,
                  MEXCT_FP_AUTO, c->stream);
  if (s) return s;
  return finish(c, out, c->out, M * 4, "fp: download");
}

mexct_status mexct_bp_dev(mexct_ctx* ctx, const float* d_sino, int W, int H,
                          int nP, float sad, const float* angles, int geom,
                          float* d_vol, void* stream) {
  VALIDATE(bp_dev_impl(nullptr, d_sino, kF32, W, H, nP, sad, angles, geom, d_vol, kF32,
                       nullptr));
  CTX_OR_FAIL(c, "bp");
  return bp_dev_impl(c, d_sino, kF32, W, H, nP, sad, angles, geom, d_vol, kF32,
                     as_stream(stream));
}

mexct_status mexct_bp_dev_ex(mexct_ctx* ctx, const void* d_sino, int stype,
                             int W, int H, int nP, float sad,
                             const float* angles, int geom, void* d_vol,
                             int vt, void* stream) {
  VALIDATE(bp_dev_impl(nullptr, d_sino, stype, W, H, nP, sad, angles, geom, d_vol, vt,
                       nullptr));
  CTX_OR_FAIL(c, "bp");
  return bp_dev_impl(c, d_sino, stype, W, H, nP, sad, angles, geom, d_vol, vt,
                     as_stream(stream));
}

mexct_status mexct_fp_slab_occupancy(int* ctas_per_sm) {
  if (!ctas_per_sm) return set_err(MEXCT_ERR_ARG, "fp_slab_occupancy: NULL pointer");
  mexct_ctx* c = resolve(nullptr);
  if (!c) return set_err(MEXCT_ERR_CUDA, "fp_slab_occupancy: no CUDA device / context");
  DevGuard dg(c->device);
  const int n = slab_resident_ctas();
  if (n < 0) return set_err(MEXCT_ERR_CUDA, "fp_slab_occupancy: occupancy query failed");
  *ctas_per_sm = n;
  return MEXCT_OK;
}

mexct_status mexct_fp_det_dev(mexct_ctx* ctx, const float* d_vol, int W, int H,
                              float sad, const float* angles, int nP, int geom,
                              const mexct_detector* det, float* d_out, void* stream) {
  VALIDATE(fp_det_impl(nullptr, d_vol, W, H, sad, angles, nP, geom, det, d_out, nullptr));
  CTX_OR_FAIL(c, "fp_det");
  return fp_det_impl(c, d_vol, W, H, sad, angles, nP, geom, det, d_out, as_stream(stream));
}

mexct_status mexct_bp_det_dev(mexct_ctx* ctx, const float* d_sino, const mexct_detector* det,
                              int nP, float sad, const float* angles, int geom, int W, int H,
                              float* d_vol, void* stream) {
  VALIDATE(bp_det_impl(nullptr, d_sino, det, nP, sad, angles, geom, W, H, d_vol, nullptr));
  CTX_OR_FAIL(c, "bp_det");
  return bp_det_impl(c, d_sino, det, nP, sad, angles, geom, W, H, d_vol, as_stream(stream));
}

mexct_status mexct_fp_det(mexct_ctx* ctx, const float* vol, int W, int H, float sad,
                          const float* angles, int nP, int geom, const mexct_detector* det,
                          float* out) {
  VALIDATE(fp_det_impl(nullptr, vol, W, H, sad, angles, nP, geom, det, out, nullptr));
  CTX_OR_FAIL(c, "fp_det");
  const size_t N = (size_t)W * W * H;
  const size_t M = (size_t)det->det_w * (size_t)det->det_h * (size_t)nP;
  mexct_status s = upload(c->in, vol, N * 4, c->stream, "fp_det: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->out.ensure_async(M * 4, c->stream), "fp_det: workspace");
  s = fp_det_impl(c, c->in.as<float>(), W, H, sad, angles, nP, geom, det, c->out.as<float>(),
                  c->stream);
  if (s) return s;
  return finish(c, out, c->out, M * 4, "fp_det: download");
}

mexct_status mexct_parker_weight(const float* sino, int W, int H, int nP, const float* angles,
                                 int geom, double sad, double q, float* out) {
  if (nP > 0 && (!sino || !angles || !out))
    return set_err(MEXCT_ERR_ARG, "parker_weight: NULL pointer");
  if (bad_dims(W, H) || nP < 0) return set_err(MEXCT_ERR_ARG, "parker_weight: bad dims");
  if (bad_geom(geom)) return set_err(MEXCT_ERR_ARG, "parker_weight: invalid geometry %d", geom);
  if (W != H)
    return set_err(MEXCT_ERR_UNSUPPORTED,
                   "parker_weight: W (%d) != H (%d); the reference's weighting "
                   "(parker_weight.m:73) needs a square detector", W, H);
  if (geom != 0 && !(sad > 0.0)) return set_err(MEXCT_ERR_ARG, "parker_weight: SAD must be > 0");
  std::vector<float> win((size_t)nP * W);
  parker_table(W, nP, angles, geom, sad, q, win.data());
  const size_t P = (size_t)W * H;
  for (int i = 0; i < nP; ++i) {
    const float* w = win.data() + (size_t)i * W;
    for (int v = 0; v < H; ++v) {
      const size_t r = (size_t)i * P + (size_t)v * W;
      for (int u = 0; u < W; ++u) out[r + u] = sino[r + u] * w[u];  // :73, in single
    }
  }
  return MEXCT_OK;
}

mexct_status mexct_bp_det(mexct_ctx* ctx, const float* sino, const mexct_detector* det, int nP,
                          float sad, const float* angles, int geom, int W, int H, float* vol) {
  VALIDATE(bp_det_impl(nullptr, sino, det, nP, sad, angles, geom, W, H, vol, nullptr));
  CTX_OR_FAIL(c, "bp_det");
  const size_t N = (size_t)W * W * H;
  const size_t M = (size_t)det->det_w * (size_t)det->det_h * (size_t)nP;
  mexct_status s = upload(c->in, sino, M * 4, c->stream, "bp_det: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->out.ensure_async(N * 4, c->stream), "bp_det: workspace");
  s = bp_det_impl(c, c->in.as<float>(), det, nP, sad, angles, geom, W, H, c->out.as<float>(),
                  c->stream);
  if (s) return s;
  return finish(c, vol, c->out, N * 4, "bp_det: download");
}

mexct_status mexct_bp(mexct_ctx* ctx, const float* sino, int W, int H, int nP,
                      float sad, const float* angles, int geom, float* vol) {
  VALIDATE(bp_dev_impl(nullptr, sino, kF32, W, H, nP, sad, angles, geom, vol, kF32, nullptr));
  CTX_OR_FAIL(c, "bp");
  const size_t N = (size_t)W * W * H, M = (size_t)W * H * nP;
  MEXCT_TRY_CUDA(c->in.ensure_async(M * 4, c->stream), "bp: workspace");
  MEXCT_TRY_CUDA(c->out.ensure_async(N * 4, c->stream), "bp: workspace");
  mexct_status s = MEXCT_OK;
  if (nP > 0 && nP <= kMaxViews && N * 4 >= ((size_t)64 << 20)) {
    // views uploaded in parts under the launches, z ranges downloaded under
    // the launches after them (same per-voxel operations as one launch), when
    // one view block is used.  A tuning run (MEXCT_TUNE_AUTO) times its
    // candidates before the views are uploaded: only its timings are used.
    mexct_shape shp{MEXCT_FP_EXPLICIT, 16, 8, 1};
    s = pick_bp_shape(c, c->in.p, kF32, W, H, nP, sad, angles, geom, c->out.p, kF32, c->stream,
                      &shp);
    if (s) return s;
    if (shp.vblocks == 1)
      return bp_host_overlapped(c, sino, W, H, nP, sad, angles, geom,
                                BpShape{shp.zc, shp.rows, 1}, vol);
  }
  s = upload(c->in, sino, M * 4, c->stream, "bp: upload");
  if (s) return s;
  s = bp_dev_impl(c, c->in.p, kF32, W, H, nP, sad, angles, geom, c->out.p, kF32, c->stream);
  if (s) return s;
  return finish(c, vol, c->out, N * 4, "bp: download");
}

mexct_status mexct_g3d_fp_dev(mexct_ctx* ctx, const float* d_vol, int S,
                              int Z, const float* angles, const float* d_pts,
                              int W, int H, int nP, int per_view,
                              float* d_out, void* stream) {
  VALIDATE(g3d_fp_dev_impl(nullptr, d_vol, S, Z, angles, d_pts, W, H, nP, per_view, d_out,
                           nullptr));
  CTX_OR_FAIL(c, "g3d_fp");
  return g3d_fp_dev_impl(c, d_vol, S, Z, angles, d_pts, W, H, nP, per_view, d_out,
                         as_stream(stream));
}

mexct_status mexct_g3d_fp(mexct_ctx* ctx, const float* vol, int S, int Z,
                          const float* angles, const float* pts, int W, int H,
                          int nP, int per_view, float* out) {
  VALIDATE(g3d_fp_dev_impl(nullptr, vol, S, Z, angles, pts, W, H, nP, per_view, out, nullptr));
  CTX_OR_FAIL(c, "g3d_fp");
  const size_t N = (size_t)S * S * Z, M = (size_t)W * H * nP;
  const size_t npts = (size_t)W * H * 6 * (per_view ? nP : 1);
  mexct_status s = upload(c->in, vol, N * 4, c->stream, "g3d_fp: upload");
  if (s) return s;
  s = upload(c->in2, pts, npts * 4, c->stream, "g3d_fp: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->out.ensure_async(M * 4, c->stream), "g3d_fp: workspace");
  s = g3d_fp_dev_impl(c, c->in.as<float>(), S, Z, angles, c->in2.as<float>(), W, H, nP,
                      per_view, c->out.as<float>(), c->stream);
  if (s) return s;
  return finish(c, out, c->out, M * 4, "g3d_fp: download");
}

mexct_status mexct_g3d_bp_dev(mexct_ctx* ctx, const float* d_sino, int W,
                              int H, int nP, const float* angles,
                              const float* d_pts, int per_view, int S, int Z,
                              float* d_vol, void* stream) {
  VALIDATE(g3d_bp_dev_impl(nullptr, d_sino, W, H, nP, angles, d_pts, per_view, S, Z, d_vol,
                           nullptr));
  CTX_OR_FAIL(c, "g3d_bp");
  return g3d_bp_dev_impl(c, d_sino, W, H, nP, angles, d_pts, per_view, S, Z, d_vol,
                         as_stream(stream));
}

mexct_status mexct_osc_iter_det_dev(mexct_ctx* ctx, float* d_mu, const float* d_pre,
                                    const float* d_post, const mexct_detector* det, int W, int H,
                                    int nP, int nSub, const int32_t* picks, const float* angles,
                                    float sad, int geom, void* stream) {
  VALIDATE(osc_det_impl(nullptr, d_mu, d_pre, d_post, det, W, H, nP, nSub, picks, angles, sad,
                        geom, nullptr));
  CTX_OR_FAIL(c, "osc_iter_det");
  return osc_det_impl(c, d_mu, d_pre, d_post, det, W, H, nP, nSub, picks, angles, sad, geom,
                      as_stream(stream));
}

mexct_status mexct_g3d_bp_matched_dev(mexct_ctx* ctx, const float* d_sino, int W, int H,
                                      int nP, const float* angles, const float* d_pts,
                                      int per_view, int S, int Z, float* d_vol, void* stream) {
  VALIDATE(g3d_bp_matched_impl(nullptr, d_sino, W, H, nP, angles, d_pts, per_view, S, Z, d_vol,
                               nullptr));
  CTX_OR_FAIL(c, "g3d_bp_matched");
  return g3d_bp_matched_impl(c, d_sino, W, H, nP, angles, d_pts, per_view, S, Z, d_vol,
                             as_stream(stream));
}

mexct_status mexct_g3d_bp_matched(mexct_ctx* ctx, const float* sino, int W, int H, int nP,
                                  const float* angles, const float* pts, int per_view, int S,
                                  int Z, float* vol) {
  VALIDATE(g3d_bp_matched_impl(nullptr, sino, W, H, nP, angles, pts, per_view, S, Z, vol,
                               nullptr));
  CTX_OR_FAIL(c, "g3d_bp_matched");
  const size_t N = (size_t)S * S * Z, M = (size_t)W * H * nP;
  const size_t npts = (size_t)W * H * 6 * (per_view ? nP : 1);
  mexct_status s = upload(c->in, sino, M * 4, c->stream, "g3d_bp_matched: upload");
  if (s) return s;
  s = upload(c->in2, pts, npts * 4, c->stream, "g3d_bp_matched: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->out.ensure_async(N * 4, c->stream), "g3d_bp_matched: workspace");
  s = g3d_bp_matched_impl(c, c->in.as<float>(), W, H, nP, angles, c->in2.as<float>(), per_view,
                          S, Z, c->out.as<float>(), c->stream);
  if (s) return s;
  return finish(c, vol, c->out, N * 4, "g3d_bp_matched: download");
}

mexct_status mexct_g3d_bp(mexct_ctx* ctx, const float* sino, int W, int H,
                          int nP, const float* angles, const float* pts,
                          int per_view, int S, int Z, float* vol) {
  VALIDATE(g3d_bp_dev_impl(nullptr, sino, W, H, nP, angles, pts, per_view, S, Z, vol, nullptr));
  CTX_OR_FAIL(c, "g3d_bp");
  const size_t N = (size_t)S * S * Z, M = (size_t)W * H * nP;
  const size_t npts = (size_t)W * H * 6 * (per_view ? nP : 1);
  mexct_status s = upload(c->in, sino, M * 4, c->stream, "g3d_bp: upload");
  if (s) return s;
  s = upload(c->in2, pts, npts * 4, c->stream, "g3d_bp: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->out.ensure_async(N * 4, c->stream), "g3d_bp: workspace");
  s = g3d_bp_dev_impl(c, c->in.as<float>(), W, H, nP, angles, c->in2.as<float>(), per_view,
                      S, Z, c->out.as<float>(), c->stream);
  if (s) return s;
  return finish(c, vol, c->out, N * 4, "g3d_bp: download");
}

mexct_status mexct_osc_iter_dev(mexct_ctx* ctx, float* d_mu,
                                const float* d_pre, const float* d_post,
                                int W, int H, int nP, int nSub,
                                const int32_t* picks, const float* angles,
                                float sad, int geom, void* stream) {
  VALIDATE(osc_dev_impl(nullptr, d_mu, kF32, d_pre, d_post, W, H, nP, nSub, picks, angles, sad,
                        geom, nullptr));
  CTX_OR_FAIL(c, "osc_iter");
  return osc_dev_impl(c, d_mu, kF32, d_pre, d_post, W, H, nP, nSub, picks, angles, sad,
                      geom, as_stream(stream));
}

mexct_status mexct_osc_iter(mexct_ctx* ctx, float* mu, const float* pre,
                            const float* post, int W, int H, int nP,
                            int nSub, const int32_t* picks,
                            const float* angles, float sad, int geom) {
  VALIDATE(osc_dev_impl(nullptr, mu, kF32, pre, post, W, H, nP, nSub, picks, angles, sad, geom,
                        nullptr));
  CTX_OR_FAIL(c, "osc_iter");
  const size_t N = (size_t)W * W * H, M = (size_t)W * H * nP;
  mexct_status s = upload(c->out, mu, N * 4, c->stream, "osc_iter: upload");
  if (s) return s;
  s = upload(c->in, pre, M * 4, c->stream, "osc_iter: upload");
  if (s) return s;
  s = upload(c->in2, post, M * 4, c->stream, "osc_iter: upload");
  if (s) return s;
  s = osc_dev_impl(c, c->out.as<float>(), kF32, c->in.as<float>(), c->in2.as<float>(), W, H,
                   nP, nSub, picks, angles, sad, geom, c->stream);
  if (s) return s;
  return finish(c, mu, c->out, N * 4, "osc_iter: download");
}

mexct_status mexct_tvmin3d_dev(mexct_ctx* ctx, const float* d_vol, int Nx,
                               int Ny, int Nz, float cval, int n_steps,
                               float* d_out, void* stream) {
  VALIDATE(tv_dev_impl(nullptr, d_vol, kF32, Nx, Ny, Nz, cval, n_steps, d_out, nullptr));
  CTX_OR_FAIL(c, "tvmin3d");
  return tv_dev_impl(c, d_vol, kF32, Nx, Ny, Nz, cval, n_steps, d_out, as_stream(stream));
}

mexct_status mexct_tvmin3d(mexct_ctx* ctx, const float* vol, int Nx, int Ny,
                           int Nz, float cval, int n_steps, float* out) {
  VALIDATE(tv_dev_impl(nullptr, vol, kF32, Nx, Ny, Nz, cval, n_steps, out, nullptr));
  CTX_OR_FAIL(c, "tvmin3d");
  const size_t N = (size_t)Nx * Ny * Nz;
  mexct_status s = upload(c->in, vol, N * 4, c->stream, "tvmin3d: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->out.ensure_async(N * 4, c->stream), "tvmin3d: workspace");
  s = tv_dev_impl(c, c->in.p, kF32, Nx, Ny, Nz, cval, n_steps, c->out.p, c->stream);
  if (s) return s;
  return finish(c, out, c->out, N * 4, "tvmin3d: download");
}

mexct_status mexct_prefilter_dev(mexct_ctx* ctx, const float* d_sino,
                                 const float* d_pre, int W, int H, int nP,
                                 const float* angles, int geom, float sad,
                                 int filter, float cutoff, float q,
                                 float* d_out, void* stream) {
  VALIDATE(prefilter_dev_impl(nullptr, d_sino, d_pre, W, H, nP, angles, geom, sad, filter,
                              cutoff, q, d_out, nullptr));
  CTX_OR_FAIL(c, "prefilter");
  return prefilter_dev_impl(c, d_sino, d_pre, W, H, nP, angles, geom, sad, filter, cutoff, q,
                            d_out, as_stream(stream));
}

mexct_status mexct_prefilter(mexct_ctx* ctx, const float* sino,
                             const float* pre, int W, int H, int nP,
                             const float* angles, int geom, float sad,
                             int filter, float cutoff, float q, float* out) {
  VALIDATE(prefilter_dev_impl(nullptr, sino, pre, W, H, nP, angles, geom, sad, filter, cutoff,
                              q, out, nullptr));
  CTX_OR_FAIL(c, "prefilter");
  const size_t M = (size_t)W * H * nP;
  mexct_status s = upload(c->in, sino, M * 4, c->stream, "prefilter: upload");
  if (s) return s;
  if (pre) {
    s = upload(c->in2, pre, M * 4, c->stream, "prefilter: upload");
    if (s) return s;
  }
  MEXCT_TRY_CUDA(c->out.ensure_async(M * 4, c->stream), "prefilter: workspace");
  s = prefilter_dev_impl(c, c->in.as<float>(), pre ? c->in2.as<float>() : nullptr, W, H, nP,
                         angles, geom, sad, filter, cutoff, q, c->out.as<float>(), c->stream);
  if (s) return s;
  return finish(c, out, c->out, M * 4, "prefilter: download");
}

mexct_status mexct_fbp(mexct_ctx* ctx, const float* pre, const float* post,
                       int W, int H, int nP, const float* angles, int geom,
                       float sad, int filter, float cutoff, float q,
                       float* recon) {
  if (!pre) return set_err(MEXCT_ERR_ARG, "fbp: NULL pointer");
  VALIDATE(prefilter_dev_impl(nullptr, post, pre, W, H, nP, angles, geom, sad, filter, cutoff,
                              q, recon, nullptr));
  CTX_OR_FAIL(c, "fbp");
  const size_t N = (size_t)W * W * H, M = (size_t)W * H * nP;
  mexct_status s = upload(c->in, post, M * 4, c->stream, "fbp: upload");
  if (s) return s;
  s = upload(c->in2, pre, M * 4, c->stream, "fbp: upload");
  if (s) return s;
  MEXCT_TRY_CUDA(c->in3.ensure_async(M * 4, c->stream), "fbp: workspace");
  MEXCT_TRY_CUDA(c->out.ensure_async(N * 4, c->stream), "fbp: workspace");
  s = prefilter_dev_impl(c, c->in.as<float>(), c->in2.as<float>(), W, H, nP, angles, geom, sad,
                         filter, cutoff, q, c->in3.as<float>(), c->stream);
  if (s) return s;
  s = bp_dev_impl(c, c->in3.p, kF32, W, H, nP, sad, angles, geom, c->out.p, kF32, c->stream);
  if (s) return s;
  return finish(c, recon, c->out, N * 4, "fbp: download");
}

}  // extern "C"
