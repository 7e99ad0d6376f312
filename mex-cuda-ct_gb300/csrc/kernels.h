// kernels.h -- launch interface between the host library and the kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "geom.cuh"

namespace mexct {

// Ray-driven projector launch (standard FP, general3D FP/BP, OSC FP).
struct RayArgs {
  int det_w, det_h;        // detector W x H
  int S, Z;                // volume S x S x Z
  float u0, v0;            // detector centre (W-1)/2, (H-1)/2
  float bx, by, bz;        // volume corner -S/2, -S/2, -Z/2
  float SR, RD, step;
  int nviews;              // views in this launch
  int view0, vstride;      // launch view i is global view view0 + i*vstride
  long long P;             // det_w * det_h
  int pts_per_view;        // general3D: per-view points
  float du, dv;            // pixel pitch at the isocentre (1: the reference's)
  float ou, ov;            // sub-pixel ray offset (0: the reference's)
  // Sub-volume FP (launch_fp_slab_sub): the padded tensors hold zrows padded
  // rows starting at full padded row zoff; samples whose z taps lie outside
  // [zlo, zhi) (tap space) read only zero rows and are skipped; accum: add to
  // the output instead of storing.
  int zoff, zrows, accum;
  float zlo, zhi;
  const float* pts;        // general3D slab FP: end points (launch_fp_slab_g3d)
  Trig trig[kMaxViews];
};

// Voxel-driven BP launch (standard BP, OSC dual BP).
struct VoxArgs {
  int W, H;       // volume W x W x H
  int nviews;
  float v0, SR;
  uint32_t hw;    // circle half width W/2 - 1 (unsigned, as the reference)
  int view0;      // launch view i reads sinogram slot view0 + i
  long long P;    // det_w * det_h
  // Detector of the decoupled-geometry BP (launch_bp_det): det_w x det_h
  // pixels, u centre hwd + 1 = det_w/2 (integer division), v centre
  // v0d = (det_h - 1)/2, reciprocal pitches inv_du, inv_dv.  The standard
  // launches ignore these fields: their detector is the volume's face.
  int det_w, det_h;
  float hwd, v0d, inv_du, inv_dv;
  // Sub-volume BP (launch_bp_sub): output slices zoff .. zoff + nzs - 1 of
  // the H-slice volume, from detector rows row0 .. row0 + nrows - 1.
  int zoff, nzs, row0, nrows;
  Trig trig[kMaxViews];
};

// Storage type tags.
enum Dtype { kF32 = 0, kF16 = 1, kBF16 = 2 };

cudaError_t launch_transpose_xy(const void* src, void* dst, int W, int H,
                                int dtype, cudaStream_t st);

cudaError_t launch_fp(int geom, bool border, const RayArgs& a,
                      const void* vol_x, const void* vol_y, int vol_type,
                      const float* pts, void* out, int out_type,
                      cudaStream_t st);

// Slab-staged FP (k_slab.cu): padded volumes in both layouts, TMA tensor maps
// over them, and the kernel.  With osc = true the kernel samples the
// zero-padded mu with step 0.5 and writes the OSC residuals instead; ot is
// then the storage of the residual views (kF32, or kF16 with FP32 mu, holding
// the residuals times e.rscale).
struct SlabEpi {
  const float* pre;  // OSC: pre/post counts and residual outputs (FP32, or FP16
  const float* post; // times rscale: the launch's residual type)
  void* rpre;        // residuals in the padded-sinogram layout of each view:
  void* rpost;       // [H+4][W+4] with a zero frame (border addressing)
  unsigned* err;     // set to non-zero when a bounded wait gave up
  int wait_us;       // limit of one wait: 0 = default (2 s), < 0 = give up at once
  double* obj;       // objective epilogue: one FP64 partial sum per CTA
  float rscale = 1.f;  // 16-bit residual views: residuals times this power of two
};
int slab_pitch(int W);
// Whether the slab FP kernels take views 2i and 2i+1 of a launch in one CTA
// (adjacent angles close enough that one slab box serves both bundles).
bool slab_pair_views(const RayArgs& a);
// CTAs of the slab FP kernels resident per SM (its launch bounds); persistent
// launches size their grids by it.
int slab_ctas_per_sm();
// Resident CTAs per SM of the cone FP32 slab kernel by the occupancy
// calculator (-1 on error).
int slab_resident_ctas();

// One problem of a batched FP launch (device-resident descriptor).
struct alignas(64) BatchFp {
  CUtensorMap tmx, tmy;       // over the problem's padded volumes
  int W, H, geom, nviews, Pf, tiles_u;
  float u0, v0, bx, by, bz, sad, step;
  long long item0;            // first work item: nviews * tiles items follow
  const void* px;
  const void* py;
  void* out;                  // sinogram (nviews, H, W)
  const Trig* trig;           // nviews entries (device)
  const void* vol;            // source volume (H, W, W) for the padding pass
  long long pad_item0;        // first padding item: ceil(Pf/32)^2 * (H+2) tiles
};

// One problem of a batched BP launch.

cudaError_t launch_fp_batch(const BatchFp* d_probs, int nprob, long long total,
                            unsigned long long* counter, unsigned* err, int ctas,
                            cudaStream_t st);
cudaError_t launch_pad_batch(const BatchFp* d_probs, int nprob, long long total,
                             cudaStream_t st);

cudaError_t launch_pad_volume(const void* src, int dtype, int W, int H, int Pf,
                              bool border, void* px, void* py, cudaStream_t st);
// TMA map over a padded volume (Pf x Ps x Pz) with the box shape of the slab
// kernel for projection geometry geom.
cudaError_t make_slab_tmap(CUtensorMap* map, const void* base, int dtype,
                           int Pf, int Ps, int Pz, int geom);
// OSC forward pass (border addressing, step 0.5) of a padded mu whose epilogue
// adds up the data-fidelity objective pre*e^-l + post*l of every detector
// pixel of the views in FP64: one partial per CTA into e.obj at index
// blockIdx.x * gridDim.y + blockIdx.y (views x tiles); nothing else is written.
cudaError_t launch_fp_slab_objective(int geom, const RayArgs& a, const CUtensorMap& mx,
                                     const CUtensorMap& my, const void* px, const void* py,
                                     int Pf, int vt, const SlabEpi& e, cudaStream_t st);
// Fixed-order FP64 sum of n partials into *out (one CTA; deterministic).
cudaError_t launch_sum_partials(const double* partials, long long n, double* out,
                                cudaStream_t st);
// out = sqrt(sum of parts[i]^2) over n norms of the parts of a volume, in
// index order; with scale non-null also scale = -c * (*cmul) / out (cmul
// may be null: factor 1).
cudaError_t launch_combine_norms(const double* parts, int n, double* out, float c,
                                 const double* cmul, float* scale, cudaStream_t st);

cudaError_t launch_fp_slab(int geom, bool border, bool osc, const RayArgs& a,
                           const CUtensorMap& mx, const CUtensorMap& my,
                           const void* px, const void* py, int Pf, int vt,
                           void* out, int ot, const SlabEpi& e,
                           cudaStream_t st);

// Slab FP (FP32) onto a decoupled detector (a.det_w, a.det_h, a.du, a.dv,
// a.ou, a.ov): par / fan rays interpolate in z, rays that miss the volume
// add nothing.
// general3D FP on the slab kernel (border addressing, FP32): rays from a.pts
// (6 planes of a.P points, per view when a.pts_per_view), per-tile boxes from
// bounds over all rays of the tile.
cudaError_t launch_fp_slab_g3d(const RayArgs& a, const CUtensorMap& mx, const CUtensorMap& my,
                               const void* px, const void* py, int Pf, float* out,
                               const SlabEpi& e, cudaStream_t st);

cudaError_t launch_fp_slab_det(int geom, const RayArgs& a, const CUtensorMap& mx,
                               const CUtensorMap& my, const void* px, const void* py, int Pf,
                               float* out, const SlabEpi& e, cudaStream_t st);

// Slab FP (FP32) of a z-slab of the volume (a.zoff, a.zrows, a.zlo, a.zhi,
// a.accum): the slab's padded tensors hold its slices with a clamp frame at
// the volume's own faces and zeros elsewhere (or a zero frame everywhere:
// border addressing), so the FPs of the slabs add up to the FP of the whole
// volume.
cudaError_t launch_fp_slab_sub(int geom, const RayArgs& a, const CUtensorMap& mx,
                               const CUtensorMap& my, const void* px, const void* py, int Pf,
                               float* out, const SlabEpi& e, cudaStream_t st);

// Padded layouts of a z-slab of nz slices (FP32): frame rows below / above
// the slab are zero where zero_lo / zero_hi (an inner slab face), else edge
// copies (the volume's own face, clamp addressing); with border the whole
// frame is zero (border addressing).
cudaError_t launch_pad_volume_sub(const float* src, int W, int nz, int Pf, bool zero_lo,
                                  bool zero_hi, float* px, float* py, cudaStream_t st,
                                  bool border = false);

cudaError_t launch_fp_tex(int geom, const RayArgs& a,
                          cudaTextureObject_t tex, float* out,
                          cudaStream_t st);

// Padded views for the voxel-driven BP: [nviews][H+4][W+4] texels, edge
// values replicated (clamp) in the two-texel frame.
constexpr int kSinoPad = 2;  // frame width of padded sinogram views
__host__ __device__ inline int sino_pad_pitch(int W) { return W + 2 * kSinoPad; }
size_t sino_pad_elems(int W, int H, int nviews);
// Launch shape of the BP: z voxels per thread (8 or 16), column rows per
// block (4 or 8), view blocks along grid z (1..64; > 1 needs an FP32
// partial-sum workspace of vblocks * W*W*H floats).
struct BpShape {
  int zc, rows, vblocks;
  // z-blocks (of zc slices) zb0 .. zb0 + nzb - 1 only (nzb = 0: all); with
  // one view block, a z range gets exactly the per-voxel operations of the
  // whole launch.
  int zb0 = 0, nzb = 0;
};
bool bp_shape_valid(const BpShape& s);

// Quad layout of the padded views (storage type stype: FP32 in 16-byte
// texels, FP16 / BF16 in 8-byte texels): texel (r, c) holds {P(r,c),
// P(r+1,c), P(r,c+1), P(r+1,c+1)} of the clamp-padded view P.
cudaError_t launch_pad_sino_quad(const void* in, int stype, int W, int H, int nviews, void* out,
                                 cudaStream_t st);
// BP of a.nviews views (view 0 of the launch first) from the quad layout, any
// geometry: cone reads one quad per voxel and view, par / fan (whose z rows
// are texel rows) one quad per z pair of voxels.  With accumulate the launch
// continues the sums stored in vol.
cudaError_t launch_bp_quad(int geom, const VoxArgs& a, const void* sino_quad, int stype,
                           void* vol, int vtype, bool accumulate, const BpShape& shp,
                           float* part, cudaStream_t st);

// Decoupled-detector BP from the quad layout (launch_pad_sino_quad, FP32) of
// a.det_w x a.det_h views.
cudaError_t launch_bp_det(int geom, const VoxArgs& a, const void* sino_quad, float* vol,
                          bool accumulate, cudaStream_t st);

// Sub-volume BP: slices a.zoff .. a.zoff + a.nzs - 1 (a W x W x a.nzs FP32
// slab) from detector rows a.row0 .. + a.nrows - 1 (which must hold every row
// the slab's columns reach: mexct_sub_rows) in the quad layout of the band.
// Per voxel the same operations as launch_bp_quad.
cudaError_t launch_bp_sub(int geom, const VoxArgs& a, const void* sino_quad, float* vol,
                          bool accumulate, cudaStream_t st);

// dst = w * src (first) or dst += w * src over n elements.
cudaError_t launch_add_scaled(const float* src, float* dst, long long n, float w, bool first,
                              cudaStream_t st);

// general3D ray-driven two-corner scatter BP (CUDAmex_general3D_BP.cu:61-188).
// Matched-adjoint general3D BP: the transpose of the general3D slab FP
// (accumulates into vol; no counterpart in the reference).
cudaError_t launch_g3d_bp_adjoint(const RayArgs& a, const float* sino, const float* pts,
                                  float* vol, cudaStream_t st);
cudaError_t launch_g3d_bp(const RayArgs& a, const float* sino,
                          const float* pts, float* vol, cudaStream_t st);

// OSC dual BP + update (CUDAmex_oscIter.cu:94-136,272-358); the subset FP with
// the residual epilogue (:140-271) is launch_fp_slab with osc = true.
// rpre/rpost: padded residual views (sino_pad_pitch layout, zero frame).
// With padx/pady non-null the updated mu is also written into the padded
// volumes of the slab FP (pitch Pf), so the next subset needs no padding pass.
// The OSC forward pass with the residual epilogue onto a decoupled detector
// (a.det_w, a.det_h, a.du, a.dv; one ray per pixel; FP32 mu) and the dual BP
// + update reading those residuals (no counterpart in the reference).
cudaError_t launch_fp_slab_osc_det(int geom, const RayArgs& a, const CUtensorMap& mx,
                                   const CUtensorMap& my, const void* px, const void* py, int Pf,
                                   const SlabEpi& e, cudaStream_t st);
cudaError_t launch_osc_bp_update_det(int geom, const VoxArgs& a, const float* rpre,
                                     const float* rpost, void* mu, int mt, void* padx,
                                     void* pady, int Pf, cudaStream_t st);
// Updates slices a.zoff .. a.zoff + a.nzs - 1 (a.zoff a multiple of 4) held
// at mu (and at slab-local rows of padx / pady).  dt: storage of the residual
// views (kF32, or kF16 with FP32 mu).
cudaError_t launch_osc_bp_update(int geom, const VoxArgs& a,
                                 const void* rpre, const void* rpost,
                                 void* mu, int mu_type, void* padx, void* pady, int Pf,
                                 cudaStream_t st, int dt = kF32);
// Residual views (padded quad layout) of nviews views from their line
// integrals l and counts pre / post, all W x H x nviews FP32.
cudaError_t launch_osc_residual(const float* l, const float* pre, const float* post, int W, int H,
                                int nviews, float* rpre, float* rpost, cudaStream_t st);

// TV (CUDAmex_TVmin_3D.cu:101-234).  tv_norm computes ||g||^2 (FP64 above the
// per-thread level) and the
// step scale -c/||g|| into *scale; tv_update writes y = x + scale*g(x).
size_t tv_partials_needed(int Nx, int Ny, int Nz);
// Whether the TV kernels' grid for this shape fits the launch limits
// (gridDim.y and gridDim.z at most 65535).
bool tv_shape_launchable(int Nx, int Ny, int Nz);
// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount,
// cached per device): grid-stride kernels size their grids by it.
int device_sms();
// Partial sums launch_ssd writes (one per CTA of its grid on the current device).
size_t ssd_partials_needed();
cudaError_t launch_tv_norm(const void* x, int x_type, int Nx, int Ny, int Nz,
                           float c, double* partials, unsigned* counter,
                           float* scale, double* norm, cudaStream_t st);
// As launch_tv_norm with c multiplied by the FP64 value at *cmul (device).
cudaError_t launch_tv_norm_scaled(const void* x, int x_type, int Nx, int Ny,
                                  int Nz, float c, const double* cmul,
                                  double* partials, unsigned* counter,
                                  float* scale, double* norm, cudaStream_t st);
cudaError_t launch_tv_update(const void* x, void* y, int x_type, int Nx,
                             int Ny, int Nz, const float* scale,
                             cudaStream_t st);

// Sum of squared differences in FP64 (OSC_TV_recon.m:65-67), deterministic.
cudaError_t launch_ssd(const void* a, const void* b, int dtype, long long n,
                       int zero_first, double* partials, unsigned* counter,
                       double* out, cudaStream_t st);
// NaN/Inf -> 0 in place (OSC_TV_recon.m:69-70).
cudaError_t launch_finite(void* x, int dtype, long long n, cudaStream_t st);
cudaError_t launch_fill(void* x, int dtype, long long n, float v,
                        cudaStream_t st);
cudaError_t launch_clamp_copy(const float* src, float* dst, long long n,
                              float eps, cudaStream_t st);
// *out = bits of the largest positive finite value of x (0 if none); *out must
// start at 0.
cudaError_t launch_max_nonneg(const float* x, long long n, unsigned* out, cudaStream_t st);
cudaError_t launch_convert(const void* src, int src_type, void* dst,
                           int dst_type, long long n, cudaStream_t st);

// FDK/FBP pre-filter (preFilterSinogram.m, parker_weight.m, FBP_recon.m).
struct FiltArgs {
  int W, H, nP, order, geom, log_input;
  float sad;
};
cudaError_t launch_prefilter(const FiltArgs& a, const float* sino,
                             const float* pre, const float* parker,
                             const float* dbeta, const float* kern,
                             float* out, cudaStream_t st);

}  // namespace mexct
