/*
 * mexct.h -- C ABI of libmexct, a GB300 (sm_103a) implementation of the
 * mex-cuda-CT projection-operator path.
 *
 * Conventions shared by every entry point
 *   - Arrays are MATLAB column-major float32 ("single"):
 *       volume   [W,W,H]   index x + W*y + W*W*z
 *       sinogram [W,H,nP]  index u + W*v + W*H*view
 *       pts      [W,H,6]   planes x1,y1,z1,x2,y2,z2 (or [W,H,6,nP] per view)
 *   - Angles are float32 radians (MATLAB single), one per view.
 *   - geom: 0 parallel, 1 stacked fan, 2 cone (the reference's geomFlag).
 *   - Host entry points (no suffix) take host pointers, copy in, compute on
 *     the GPU and copy out before returning (the MEX gateway contract).
 *     Pinned host buffers give full-speed copies; pageable ones work too.
 *   - Device entry points (suffix _dev) take device pointers and a CUDA
 *     stream (cudaStream_t passed as void*, NULL = legacy default stream);
 *     they are stream-ordered and return without synchronising.
 *   - ctx may be NULL: a per-device default context is used.
 *   - Every call returns a mexct_status; mexct_last_error() gives the text of
 *     the last failure on the calling thread.  Nothing aborts, longjmps or
 *     resets the device (the reference's CUDAmex_oscIter.cu:582 calls
 *     cudaDeviceReset; this library never does).
 */
#ifndef MEXCT_H
#define MEXCT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int mexct_status;
#define MEXCT_OK 0
#define MEXCT_ERR_ARG 1         /* invalid argument (dims, geom, null, ...) */
#define MEXCT_ERR_CUDA 2        /* CUDA runtime error */
#define MEXCT_ERR_OOM 3         /* device allocation failed */
#define MEXCT_ERR_UNSUPPORTED 4 /* valid in the reference but not supported */
#define MEXCT_ERR_TIMEOUT 5     /* a bounded device-side wait gave up */
#define MEXCT_ERR_BUDGET 6      /* request exceeds the admission budget */
#define MEXCT_ERR_IO 7          /* a file cannot be read, written or parsed */

/* Storage types for the _ex entry points. */
#define MEXCT_F32 0
#define MEXCT_F16 1
#define MEXCT_BF16 2

/* FP implementation variants for the _ex entry points. */
#define MEXCT_FP_EXPLICIT 0 /* FP32 trilinear, TMA slab-staged (parity path) */
#define MEXCT_FP_TEXTURE 1  /* hardware 3D texture: the reference's arithmetic, bit for bit */
#define MEXCT_FP_RAY 2      /* FP32 trilinear, one ray per thread via L1 */
#define MEXCT_FP_AUTO 3     /* EXPLICIT or RAY, from the context's shape table */

typedef struct mexct_ctx mexct_ctx;

const char* mexct_last_error(void);
const char* mexct_version(void);

/* Context: owns the stream used by host entry points, grow-only device
 * workspaces and the autotune cache.  One context per device and thread
 * (or serialise calls on a shared one). */
mexct_status mexct_ctx_create(int device, mexct_ctx** out);
mexct_status mexct_ctx_destroy(mexct_ctx* ctx);
/* Release the context's workspaces (they are re-created on demand). */
mexct_status mexct_ctx_trim(mexct_ctx* ctx);

/* Bounded waits (no counterpart in the reference).  The slab forward projector
 * waits on its shared-memory copies with a wall-clock limit; a wait that runs
 * out records a flag in the context's device error word and the CTA samples
 * from global memory instead, so the result is unchanged and nothing hangs.
 * set_wait_limit: us > 0 limit per wait in microseconds, 0 give up at once
 * (diagnostics: every wait that is not already satisfied falls back), < 0 the
 * default (2 s).  device_errors: the error word's flags (bit 0: a wait gave
 * up; bit 1: a copy issued before that did not land within 2 s either), read
 * with a blocking copy once the covered work has finished (e.g. after
 * synchronising its stream); clear != 0 zeroes it. */
mexct_status mexct_ctx_set_wait_limit(mexct_ctx* ctx, int us);
mexct_status mexct_ctx_device_errors(mexct_ctx* ctx, unsigned* flags, int clear);

/* ---- MEX-equivalent host entry points --------------------------------- */

/* fp = CUDAmex_FP(vol, SAD, angles, nProj, geomFlag)
 * Replaces projection_kernels/CUDAmex_FP.cu:350-477 (kernels :56-346).
 * vol [W,W,H] -> out [W,H,nP].  Clamp addressing; step 0.5 (par, fan) or 1.0
 * (cone).  Every detector row is computed (the reference skips rows
 * iy >= 32*ceil(W/32), CUDAmex_FP.cu:432-440). */
mexct_status mexct_fp(mexct_ctx* ctx, const float* vol, int W, int H,
                      float sad, const float* angles, int nP, int geom,
                      float* out);

/* bp = CUDAmex_BP(sino, SAD, angles, geomFlag)
 * Replaces projection_kernels/CUDAmex_BP.cu:223-324 (kernels :44-221).
 * sino [W,H,nP] -> vol [W,W,H] (zero outside the circle h = W/2-1). */
mexct_status mexct_bp(mexct_ctx* ctx, const float* sino, int W, int H,
                      int nP, float sad, const float* angles, int geom,
                      float* vol);

/* fp = CUDAmex_general3D_FP(vol, angles, pts, nProj)
 * Replaces projection_kernels/CUDAmex_general3D_FP.cu:154-252 (kernel
 * :59-150).  vol [S,S,Z], pts [W,H,6] shared by all views (pts_per_view=0,
 * the reference's form) or [W,H,6,nP] (pts_per_view=1, an extension for
 * helical scans).  Border addressing, step 0.5. */
mexct_status mexct_g3d_fp(mexct_ctx* ctx, const float* vol, int S, int Z,
                          const float* angles, const float* pts, int W,
                          int H, int nP, int pts_per_view, float* out);

/* bp = CUDAmex_general3D_BP(sino, angles, pts, S, Z)
 * Replaces projection_kernels/CUDAmex_general3D_BP.cu:194-282 (kernel
 * :61-188): ray-driven two-corner scatter, transcribed exactly. */
mexct_status mexct_g3d_bp(mexct_ctx* ctx, const float* sino, int W, int H,
                          int nP, const float* angles, const float* pts,
                          int pts_per_view, int S, int Z, float* vol);

/* CUDAmex_oscIter(mu, pre, post, nSub, subsetPicks, angles, SAD, geomFlag)
 * Replaces iterative_reconstruction/CUDAmex_oscIter.cu:362-584 (kernels
 * :94-358).  mu [W,W,H] is updated in place; pre/post [W,H,nP] are NOT
 * modified (the reference overwrites them, :527-528). */
mexct_status mexct_osc_iter(mexct_ctx* ctx, float* mu, const float* pre,
                            const float* post, int W, int H, int nP,
                            int nSub, const int32_t* picks,
                            const float* angles, float sad, int geom);

/* out = CUDAmex_TVmin_3D(vol, c)
 * Replaces iterative_reconstruction/CUDAmex_TVmin_3D.cu:162-246 (kernel
 * :101-158, thrust norm/saxpy :221-234).  n_steps = 20 in the reference.
 * Border gradient is 0 (the reference leaves it uninitialised); the
 * gradient norm is reduced in FP64. */
mexct_status mexct_tvmin3d(mexct_ctx* ctx, const float* vol, int Nx, int Ny,
                           int Nz, float c, int n_steps, float* out);

/* filteredSino = preFilterSinogram(sino, geom, angles, filter, cutoff, q)
 * Replaces fbp_reconstruction/preFilterSinogram.m:1-90 and
 * parker_weight.m:1-98.  filter: 0 none, 1 ramp, 2 shepp-logan, 3 cosine,
 * 4 hamming, 5 hann.  Requires W == H and nP >= 2, as the reference does.
 * log_input != 0 first applies FBP_recon.m:26-28 (sino = -log(post/pre),
 * NaN/Inf -> 0) with sino = post and pre_or_null = pre. */
mexct_status mexct_prefilter(mexct_ctx* ctx, const float* sino,
                             const float* pre_or_null, int W, int H, int nP,
                             const float* angles, int geom, float sad,
                             int filter, float cutoff, float q, float* out);

/* weightedSino = parker_weight(sino, angles, geom, q)
 * Replaces fbp_reconstruction/parker_weight.m:1-79 (its printed notes left
 * out): the (modified) Parker window per view and row element u of a W x W
 * detector, computed in FP64 from MATLAB's double SAD and q, rounded to
 * single and multiplied into the single sinogram as the reference does.
 * Host only (no GPU).  W != H: MEXCT_ERR_UNSUPPORTED (the reference's repmat
 * needs a square detector). */
mexct_status mexct_parker_weight(const float* sino, int W, int H, int nP,
                                 const float* angles, int geom, double sad,
                                 double q, float* out);

/* recon = FBP_recon(pre, post, angles, geom, filter, cutoff, q)
 * Replaces fbp_reconstruction/FBP_recon.m:1-41 on the device: log
 * transform, pre-filter and BP with no host round trip. */
mexct_status mexct_fbp(mexct_ctx* ctx, const float* pre, const float* post,
                       int W, int H, int nP, const float* angles, int geom,
                       float sad, int filter, float cutoff, float q,
                       float* recon);

/* ---- device-pointer twins (stream-ordered) ---------------------------- */

mexct_status mexct_fp_dev(mexct_ctx* ctx, const float* d_vol, int W, int H,
                          float sad, const float* angles, int nP, int geom,
                          float* d_out, void* stream);
mexct_status mexct_bp_dev(mexct_ctx* ctx, const float* d_sino, int W, int H,
                          int nP, float sad, const float* angles, int geom,
                          float* d_vol, void* stream);
mexct_status mexct_g3d_fp_dev(mexct_ctx* ctx, const float* d_vol, int S,
                              int Z, const float* angles, const float* d_pts,
                              int W, int H, int nP, int pts_per_view,
                              float* d_out, void* stream);
mexct_status mexct_g3d_bp_dev(mexct_ctx* ctx, const float* d_sino, int W,
                              int H, int nP, const float* angles,
                              const float* d_pts, int pts_per_view, int S,
                              int Z, float* d_vol, void* stream);

/* Matched-adjoint general3D BP (no counterpart in the reference: its BP,
 * CUDAmex_general3D_BP.cu:61-188, deposits into two corners with shifted
 * weights and is not the transpose of its FP; its eight-corner form is left
 * commented out at :172-179).  The exact transpose of mexct_g3d_fp of this
 * library: the same rays and FP32 sample positions, the eight trilinear taps
 * of each sample, p*0.5*w into each tap inside the volume, so that
 * <g3d_fp(x), y> = <x, g3d_bp_matched(y)> up to FP32 rounding (what iterative
 * solvers with a gradient need).  Arguments as mexct_g3d_bp / _dev. */
mexct_status mexct_g3d_bp_matched(mexct_ctx* ctx, const float* sino, int W, int H,
                                  int nP, const float* angles, const float* pts,
                                  int pts_per_view, int S, int Z, float* vol);
mexct_status mexct_g3d_bp_matched_dev(mexct_ctx* ctx, const float* d_sino, int W,
                                      int H, int nP, const float* angles,
                                      const float* d_pts, int pts_per_view, int S,
                                      int Z, float* d_vol, void* stream);
mexct_status mexct_osc_iter_dev(mexct_ctx* ctx, float* d_mu,
                                const float* d_pre, const float* d_post,
                                int W, int H, int nP, int nSub,
                                const int32_t* picks, const float* angles,
                                float sad, int geom, void* stream);
mexct_status mexct_tvmin3d_dev(mexct_ctx* ctx, const float* d_vol, int Nx,
                               int Ny, int Nz, float c, int n_steps,
                               float* d_out, void* stream);
mexct_status mexct_prefilter_dev(mexct_ctx* ctx, const float* d_sino,
                                 const float* d_pre_or_null, int W, int H,
                                 int nP, const float* angles, int geom,
                                 float sad, int filter, float cutoff,
                                 float q, float* d_out, void* stream);

/* Extended FP/BP: storage type of the volume and sinogram (MEXCT_F32,
 * MEXCT_F16, MEXCT_BF16; accumulation is always FP32) and the FP variant
 * (MEXCT_FP_EXPLICIT, MEXCT_FP_RAY, MEXCT_FP_AUTO, or MEXCT_FP_TEXTURE with
 * FP32 storage only). */
mexct_status mexct_fp_dev_ex(mexct_ctx* ctx, const void* d_vol, int vol_type,
                             int W, int H, float sad, const float* angles,
                             int nP, int geom, void* d_out, int out_type,
                             int variant, void* stream);
mexct_status mexct_bp_dev_ex(mexct_ctx* ctx, const void* d_sino,
                             int sino_type, int W, int H, int nP, float sad,
                             const float* angles, int geom, void* d_vol,
                             int vol_type, void* stream);

/* Resident CTAs per SM of the cone FP32 slab kernel (256 threads, 57 KB of
 * shared memory each) on the current device, by the occupancy calculator:
 * 4 on a GB300. */
mexct_status mexct_fp_slab_occupancy(int* ctas_per_sm);

/* ---- decoupled detector ----------------------------------------------- */

/* No counterpart in the reference, whose detector is always the volume's
 * face: W x H pixels of unit pitch, one ray through each pixel centre
 * (CUDAmex_FP.cu:378-379, CUDAmex_BP.cu:73,249).  Here the detector is
 * det_w x det_h pixels of pitch du x dv (voxel units at the isocentre), with
 * its centre where the reference puts it: u0 = (det_w - 1)/2 for the rays,
 * det_w/2 (integer division) for BP's u coordinate, (det_h - 1)/2 in v.
 * ss >= 1: FP traces ss x ss rays per pixel at sub-pixel offsets
 * (k + 0.5)/ss - 0.5 and returns their mean.  det_w = W, det_h = H,
 * du = dv = 1, ss = 1 gives what mexct_fp_dev / mexct_bp_dev give. */
typedef struct mexct_detector {
  int det_w, det_h;  /* pixels, >= 1 each */
  float du, dv;      /* pitch, > 0 */
  int ss;            /* FP rays per pixel side, 1..8 */
} mexct_detector;

/* FP32 volume W x W x H (x fastest) to an FP32 sinogram det_w x det_h x nP
 * (the slab kernel; ss x ss launches for ss > 1). */
mexct_status mexct_fp_det_dev(mexct_ctx* ctx, const float* d_vol, int W, int H,
                              float sad, const float* angles, int nP,
                              int geom, const mexct_detector* det,
                              float* d_out, void* stream);
/* FP32 sinogram det_w x det_h x nP to an FP32 volume W x W x H (voxel-driven,
 * bilinear in u and v for every geometry; ss is ignored). */
mexct_status mexct_bp_det_dev(mexct_ctx* ctx, const float* d_sino,
                              const mexct_detector* det, int nP, float sad,
                              const float* angles, int geom, int W, int H,
                              float* d_vol, void* stream);

/* Host-array forms of the two above (MATLAB layouts, as mexct_fp / mexct_bp:
 * vol [W, W, H], sinogram [det_w, det_h, nP], both x / u fastest): one
 * upload, the device operator, one download, synchronous. */
mexct_status mexct_fp_det(mexct_ctx* ctx, const float* vol, int W, int H, float sad,
                          const float* angles, int nP, int geom,
                          const mexct_detector* det, float* out);
mexct_status mexct_bp_det(mexct_ctx* ctx, const float* sino,
                          const mexct_detector* det, int nP, float sad,
                          const float* angles, int geom, int W, int H, float* vol);

/* One OSC iteration (as mexct_osc_iter_dev) with the scanner's detector
 * decoupled from the volume (no counterpart in the reference, whose oscIter
 * ties the detector to the volume's face): pre/post are FP32 counts on a
 * det_w x det_h x nP detector of pitch du x dv; the forward pass casts one ray
 * per pixel centre (det->ss must be 1) with the residual epilogue, and the
 * dual BP interpolates the residuals in u and v for every geometry.  FP32 mu
 * [W,W,H] is updated in place.  det_w = W, det_h = H, du = dv = 1 is the
 * reference's detector. */
mexct_status mexct_osc_iter_det_dev(mexct_ctx* ctx, float* d_mu, const float* d_pre,
                                    const float* d_post, const mexct_detector* det,
                                    int W, int H, int nP, int nSub,
                                    const int32_t* picks, const float* angles,
                                    float sad, int geom, void* stream);

/* ---- sub-volumes and out-of-core FP / BP --------------------------------- */

/* No counterpart in the reference (its oscIter keeps whole volumes on the
 * device; sub-volume reconstruction of larger images is a TODO at
 * iterative_reconstruction/CUDAmex_oscIter.cu:28-29).  A slab is slices
 * z0 .. z0 + nz - 1 of a W x W x H volume (x fastest), standard detector
 * (W x H, pitch 1).
 *
 * mexct_sub_rows: the detector rows row0 .. row0 + nrows - 1 that the BP of a
 * slab reads (par / fan: the slab's own rows; cone: a wider band).
 * mexct_fp_sub_dev: FP of a device slab (W x W x nz) into the device sinogram
 * (W x H x nP): the FP of the volume with every other slice zero, the clamp
 * frame kept at the volume's own faces; accumulate != 0 adds to d_sino, so
 * the FPs of the slabs of a volume add up to its FP (FP32 rounding apart).
 * mexct_bp_sub_dev: BP into a device slab from detector rows row0 .. row0 +
 * nrows - 1 of every view (device array W x nrows x nP; the rows must hold
 * those mexct_sub_rows names); each voxel gets the operations of the
 * whole-volume BP, so the slabs of a volume are its BP (with one view block,
 * MEXCT_TUNE_FIXED, bit for bit).  accumulate != 0 continues the sums stored
 * in d_slab view by view, so the BPs of consecutive view chunks of a
 * sinogram accumulate to its one-call BP bit for bit. */
mexct_status mexct_sub_rows(int W, int H, float sad, int geom, int z0, int nz,
                            int* row0, int* nrows);
mexct_status mexct_fp_sub_dev(mexct_ctx* ctx, const float* d_slab, int W, int H,
                              int z0, int nz, float sad, const float* angles,
                              int nP, int geom, float* d_sino, int accumulate,
                              void* stream);
mexct_status mexct_bp_sub_dev(mexct_ctx* ctx, const float* d_rows, int row0,
                              int nrows, int W, int H, int nP, float sad,
                              const float* angles, int geom, int z0, int nz,
                              float* d_slab, int accumulate, void* stream);

/* FP / BP of host arrays (the layouts of mexct_fp / mexct_bp) whose device
 * working set is kept within budget_bytes: the volume passes through the
 * device in slabs, the sinogram in view chunks (FP) or row bands (BP).
 * MEXCT_ERR_BUDGET if not even one slice and one view fit.  The context's
 * workspaces grow to the working set and are kept (mexct_ctx_trim frees them). */
mexct_status mexct_fp_ooc(mexct_ctx* ctx, const float* vol, int W, int H,
                          float sad, const float* angles, int nP, int geom,
                          size_t budget_bytes, float* sino);
mexct_status mexct_bp_ooc(mexct_ctx* ctx, const float* sino, int W, int H,
                          int nP, float sad, const float* angles, int geom,
                          size_t budget_bytes, float* vol);

/* ---- scanner data files -------------------------------------------------- */

/* No counterpart in the reference (its .vff / .mat data are read in MATLAB and
 * kept out of the repository, .gitignore:14-16).  Arrays are float32,
 * column-major, as the entry points take them.
 *
 * MAT-file Level 5 (MATLAB save up to -v7, compressed or not, either byte
 * order): mexct_mat_list writes the variable names, '\n'-separated;
 * mexct_mat_info gives a variable's dimensions (name NULL or "": the first
 * numeric one); mexct_mat_read converts its real part (any numeric class) to
 * float32, count = the product of the dimensions.  -v7.3 files (HDF5, which
 * MATLAB needs for arrays above 2 GB) are read by the same three calls: the
 * root group's numeric and logical datasets (complex: the real part),
 * contiguous, compact or chunked with deflate / shuffle / Fletcher-32; other
 * HDF5 features give MEXCT_ERR_UNSUPPORTED.  mexct_mat_write writes one
 * single-precision variable, creating the file or (append != 0) adding to it
 * (see mexct_mat_write_ex for the format).
 *
 * VFF ("ncaa" header, single-band raster slices, big-endian data; bits 8
 * unsigned, 16 signed, 32 float): mexct_vff_info gives the size X, Y, Z (Z = 1
 * for rank 2), spacing and bits; mexct_vff_read converts to float32 (x
 * fastest); mexct_vff_write writes bits 16 (rounded, saturated) or 32. */
mexct_status mexct_mat_list(const char* path, char* names, size_t capacity);
mexct_status mexct_mat_info(const char* path, const char* name, int* ndims,
                            long long* dims);
mexct_status mexct_mat_read(const char* path, const char* name, float* out,
                            long long count);
mexct_status mexct_mat_write(const char* path, const char* name,
                             const float* data, int ndims,
                             const long long* dims, int append);
/* mexct_mat_write with the file format chosen: MEXCT_MAT_V5 (Level 5, at most
 * 4 GiB per variable), MEXCT_MAT_V73 (-v7.3 / HDF5: a contiguous single
 * dataset with MATLAB_class "single", as MATLAB writes it; appending relinks
 * the root group at the end of the file) or MEXCT_MAT_AUTO (what
 * mexct_mat_write does: the format of the file appended to, else -v7.3 for a
 * variable of 2 GB or more, which MATLAB reads only from -v7.3). */
#define MEXCT_MAT_AUTO 0
#define MEXCT_MAT_V5 5
#define MEXCT_MAT_V73 73
mexct_status mexct_mat_write_ex(const char* path, const char* name,
                                const float* data, int ndims,
                                const long long* dims, int append, int format);
mexct_status mexct_vff_info(const char* path, int* dims, float* spacing,
                            int* bits);
mexct_status mexct_vff_read(const char* path, float* out, long long count);
mexct_status mexct_vff_write(const char* path, const float* data,
                             const int* dims, const float* spacing, int bits);

/* ---- launch shapes and autotuning -------------------------------------- */

/* No counterpart in the reference (its kernels have one fixed launch shape).
 *
 * Every FP and BP call belongs to a shape class: operator, geometry, W, H,
 * the view count rounded up to a power of two, and the input / output
 * storage types.  A context keeps one launch shape per class.
 * FP: variant, MEXCT_FP_EXPLICIT (TMA slab kernel) or MEXCT_FP_RAY (one ray
 *     per thread); both compute the exact FP32 form.  Used by mexct_fp,
 *     mexct_fp_dev and mexct_fp_dev_ex with MEXCT_FP_AUTO.
 * BP: zc = z voxels per thread (8 or 16), rows = voxel rows per 32-column
 *     block (4 or 8), vblocks = view blocks (1..64) whose FP32 partial sums
 *     are added in block order; used by every BP entry point.
 * Shapes change only the rounding of the FP32 sums (vblocks) or nothing at
 * all (zc, rows, variant). */
typedef struct mexct_shape {
  int variant;               /* FP */
  int zc, rows, vblocks;     /* BP */
} mexct_shape;

#define MEXCT_OP_FP 0
#define MEXCT_OP_BP 1

/* Modes for a class without a table entry. */
#define MEXCT_TUNE_FIXED 0     /* FP slab kernel; BP zc 16, rows 8, 1 view block */
#define MEXCT_TUNE_HEURISTIC 1 /* default: view blocks so small volumes fill the GPU */
#define MEXCT_TUNE_AUTO 2      /* the first call of the class times every candidate
                                  shape on its own data and keeps the fastest (a call
                                  made during stream capture uses the heuristic) */
mexct_status mexct_ctx_set_tune_mode(mexct_ctx* ctx, int mode);

/* Pin (set) or read the shape of one class.  get returns the entry if there
 * is one (ms = the tuned time in milliseconds, NaN if pinned, tuned = 1 if
 * chosen by timing), else the shape the current mode would start from with
 * tuned = -1. */
mexct_status mexct_shape_set(mexct_ctx* ctx, int op, int geom, int W, int H,
                             int nP, int in_type, int out_type,
                             const mexct_shape* shape);
mexct_status mexct_shape_get(mexct_ctx* ctx, int op, int geom, int W, int H,
                             int nP, int in_type, int out_type,
                             mexct_shape* shape, double* ms, int* tuned);
/* Drop every table entry of the context. */
mexct_status mexct_shape_clear(mexct_ctx* ctx);

/* Tune one class now: time every candidate shape on these device buffers
 * (the output is overwritten; on return it holds the result of the best
 * shape), record the fastest and return it.  Must not run during stream
 * capture. */
mexct_status mexct_autotune_fp(mexct_ctx* ctx, const void* d_vol, int vol_type,
                               int W, int H, float sad, const float* angles,
                               int nP, int geom, void* d_out, int out_type,
                               void* stream, mexct_shape* best, double* best_ms);
mexct_status mexct_autotune_bp(mexct_ctx* ctx, const void* d_sino,
                               int sino_type, int W, int H, int nP, float sad,
                               const float* angles, int geom, void* d_vol,
                               int vol_type, void* stream, mexct_shape* best,
                               double* best_ms);

/* ---- allocation-free variant ------------------------------------------ */

/* TV descent for callers that cannot allocate device memory while they run.
 * This entry point has no counterpart in the reference.
 *
 * It returns the same volume as mexct_tvmin3d_dev. Its scratch is one fixed
 * array compiled into the library (about 8.5 MiB, kept by every GPU that
 * loads the library until the process exits), so it never calls cudaMalloc
 * or cudaFree. That suits a serving loop that reserves its whole HBM budget
 * at start-up, where an allocation on the request path can synchronise the
 * device and stall other streams. It also suits a host whose GPU memory is
 * held by another allocator (MATLAB's gpuArray pool, for one).
 *
 * - The caller passes the input and output volumes (device pointers, float32,
 *   Nx*Ny*Nz voxels; d_vol == d_out is allowed).
 * - It runs on the current device and the given stream.
 * - Volumes above 2^21 voxels (e.g. 128^3) are rejected with
 *   MEXCT_ERR_UNSUPPORTED. So is a shape that needs more than 65536 reduction
 *   partials, or a launch grid beyond 65535 tiles in y or z.
 * - Every call looks up the array's device address for the current device
 *   and context. The first call on a device also loads the library's device
 *   code there: make that first call before any stream capture.
 * - All calls share the array. Calls that overlap on the GPU race. */
mexct_status mexct_tvmin3d_dev_noalloc(const float* d_vol, int Nx, int Ny,
                                       int Nz, float c, int n_steps,
                                       float* d_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MEXCT_H */
