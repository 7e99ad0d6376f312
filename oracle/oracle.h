/*
 * oracle.h -- FP64 CPU restatement of the mex-cuda-CT projection-operator path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness checker for the
 * CUDA library in mex-cuda-ct_gb300/ and the timed CPU baseline.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may load
 * it; the product never links or calls it.
 *
 * Parity pinning: the reference (kurtishdekker/mex-cuda-CT) ships no tests,
 * golden vectors or fixtures, and its GPU kernels use texture references that
 * no longer compile with CUDA 13.  The oracle is therefore pinned by the
 * reference SOURCE (every function cites the file:line it restates) plus the
 * known-answer tests in tests/test_oracle_kat.py (chord lengths, constant
 * sinograms, trilinear hats, OSC fixed points, TV of constants).
 *
 * Arithmetic policy (stated once, used everywhere):
 *   - Discrete decisions of the reference (ray clipping, sample counts,
 *     general3D BP floor/ceil voxel indices and weights) are evaluated in IEEE
 *     binary32 exactly as the reference source writes them (no contraction:
 *     built with -ffp-contract=off), because they are discontinuous in the
 *     inputs and an FP64 evaluation would flip them.
 *   - Everything continuous (sample positions, trilinear/bilinear weights,
 *     ray sums, BP sums, exp, OSC update, TV gradient, norms, FFT filter) is
 *     FP64.
 *
 * Array layout: MATLAB column-major.  Volume index x + W*y + W*W*z,
 * sinogram index u + W*v + W*H*view.
 */
#ifndef MEXCT_ORACLE_H
#define MEXCT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Standard-geometry forward projection (CUDAmex_FP.cu:56-346, clamp address
 * mode, step 0.5 for geom 0/1 and 1.0 for geom 2).  out: [W,H,nP]. */
int orc_fp(const float* vol, int W, int H, float sad, const float* angles,
           int nP, int geom, double* out);

/* Standard-geometry voxel-driven backprojection (CUDAmex_BP.cu:44-221,
 * clamp address mode).  sino [W,H,nP] -> vol [W,W,H] (zeros outside circle). */
int orc_bp(const float* sino, int W, int H, int nP, float sad,
           const float* angles, int geom, double* vol);

/* Detector generalisation of orc_fp / orc_bp (no counterpart in the
 * reference): detector Wd x Hd pixels of pitch du, dv (voxels, at the
 * isocentre), FP with ss x ss rays per pixel averaged.  Wd = W, Hd = H,
 * du = dv = 1, ss = 1 are orc_fp / orc_bp exactly. */
int orc_fp_det(const float* vol, int W, int H, float sad, const float* angles,
               int nP, int geom, int Wd, int Hd, float du, float dv, int ss,
               double* out);
int orc_bp_det(const float* sino, int Wd, int Hd, int nP, float sad,
               const float* angles, int geom, int W, int H, float du, float dv,
               double* vol);

/* general3D forward projection (CUDAmex_general3D_FP.cu:59-150, border
 * address mode, step 0.5).  pts: [W,H,6] shared by every view
 * (pts_per_view=0) or [W,H,6,nP] (pts_per_view=1). out: [W,H,nP]. */
int orc_g3d_fp(const float* vol, int S, int Z, const float* angles,
               const float* pts, int W, int H, int nP, int pts_per_view,
               double* out);

/* general3D ray-driven 2-corner scatter backprojection
 * (CUDAmex_general3D_BP.cu:61-188).  vol: [S,S,Z]. */
int orc_g3d_bp(const float* sino, int W, int H, int nP, const float* angles,
               const float* pts, int pts_per_view, int S, int Z, double* vol);

/* The exact transpose of orc_g3d_fp (no counterpart in the reference). */
int orc_g3d_bp_matched(const float* sino, int W, int H, int nP, const float* angles,
                       const float* pts, int pts_per_view, int S, int Z, double* vol);

/* One OSC iteration over all subsets (CUDAmex_oscIter.cu:94-358,504-557):
 * mu [W,W,H] is updated in place (FP64 state); pre/post [W,H,nP] are NOT
 * modified.  picks: nSub int32 subset indices (0-based). */
int orc_osc_iter(double* mu, const float* pre, const float* post, int W,
                 int H, int nP, int nSub, const int32_t* picks,
                 const float* angles, float sad, int geom);

/* orc_osc_iter onto a decoupled detector (no counterpart in the reference):
 * pre/post [Wd,Hd,nP] of pitch du x dv, one ray per pixel centre. */
int orc_osc_iter_det(double* mu, const float* pre, const float* post, int W,
                     int H, int nP, int nSub, const int32_t* picks,
                     const float* angles, float sad, int geom, int Wd, int Hd,
                     float du, float dv);

/* The OSC forward pass alone (CUDAmex_oscIter.cu:140-259): step 0.5 for
 * every geometry, border addressing.  mu [W,W,H] -> out [W,H,nP]. */
int orc_osc_fp(const double* mu, int W, int H, float sad, const float* angles,
               int nP, int geom, double* out);

/* TV descent (CUDAmex_TVmin_3D.cu:101-234): n_steps of
 * x <- x - (c/||g||) g with the reference's 13-point TV gradient; border
 * voxels have g = 0.  vol is updated in place. */
int orc_tvmin3d(double* vol, int Nx, int Ny, int Nz, double c, int n_steps);

/* TV gradient only (for kernel-level checks).  g: [Nx,Ny,Nz]. */
int orc_tv_gradient(const double* vol, int Nx, int Ny, int Nz, double* g);

/* OSC_TV_recon.m driver (OSC_TV_recon.m:33-102).  first_picks[k] is the
 * 0-based first subset of iteration k (the reference draws it with randperm);
 * the rest of the order follows calcSubsetOrder.  mu_out: [W,W,H].
 * iter_cb (may be NULL) receives (k, mu) after every iteration. */
typedef void (*orc_iter_cb)(int k, const double* mu, void* user);
int orc_osc_tv(const float* pre, const float* post, int W, int H, int nP,
               const float* angles, float sad, int geom, int n_iter,
               double tv_const, int n_sub_init, int n_sub_final, double p_val,
               const int32_t* first_picks, double* mu_out, orc_iter_cb cb,
               void* user);

/* calcNumSubsets / calcSubsetOrder (OSC_TV_recon.m:76-102). */
int orc_num_subsets(int s_init, int s_final, double p_val, int max_iters,
                    int k);
int orc_subset_order(int n_sub, int first_pick, int32_t* picks);

/* parker_weight.m:29-72: the Parker window [nP][W] (view-major) in FP64 for a
 * W x W detector; q = 1 original Parker, q < 1 Wesarg's modified weights. */
int orc_parker_window(int W, int nP, const float* angles, int geom, double sad,
                      double q, double* out);

/* preFilterSinogram.m + parker_weight.m (FDK/FBP pre-filter).
 * filter: 0 none, 1 ramp, 2 shepp-logan, 3 cosine, 4 hamming, 5 hann.
 * geom 0 par3d, 1 fan3d, 2 cone3d.  Requires W == H (see parker_weight.m:225).
 * out: [W,H,nP] FP64. */
int orc_prefilter(const float* sino, int W, int H, int nP,
                  const float* angles, int geom, double sad, int filter,
                  double cutoff, double q, double* out);

/* Filter frequency response H (length order) of designFilter
 * (preFilterSinogram.m:95-152). Returns order, or <0 on error. */
int orc_filter_response(int W, int filter, double cutoff, double* H,
                        int cap);

/* Thread count used by the OpenMP loops (0 = OpenMP default). */
void orc_set_threads(int n);
int orc_get_threads(void);

/* Texture-fetch weights: 0 exact (default), 1 nearest 1/256, 2 truncated to
 * 1/256 -- an emulation of the 8-fractional-bit weights of CUDA's linear
 * texture filter, which the reference's tex2D/tex3D fetches use. */
void orc_set_tex_weights(int mode);
int orc_get_tex_weights(void);

/* Sample-position arithmetic of every FP / BP / OSC operator: 0 = FP64
 * positions p0 + k*d (default), 1 = the reference's binary32 incremental
 * stepping (`currentpoint += stepsize`, `proj_z += U`, binary32 column set-up).
 * Sums are FP64 in both modes. */
void orc_set_ref_steps(int mode);
int orc_get_ref_steps(void);

#ifdef __cplusplus
}
#endif
#endif
