/*
 * mexct_solver.h -- device-resident OSC-TV solver of libmexct (C ABI).
 * Conventions as in mexct.h.
 */
#ifndef MEXCT_SOLVER_H
#define MEXCT_SOLVER_H
#include "mexct.h"
#ifdef __cplusplus
extern "C" {
#endif

/* ---- device-resident OSC-TV (OSC_TV_recon.m on the GPU) --------------- */

/* A solver keeps mu, mu_old, pre and post resident on the device and runs
 * iterative_reconstruction/OSC_TV_recon.m:33-74 without host round trips:
 * per iteration the subset count (calcNumSubsets, :76-78) and order
 * (calcSubsetOrder, :80-102, with the randperm first pick given), one OSC
 * iteration, and from k = 2 the FP64 step norm d_a, 20 TV steps with
 * c = TV_constant*d_a and NaN/Inf -> 0.  Storage of mu may be MEXCT_F32
 * or MEXCT_BF16 (pre/post stay FP32: counts exceed FP16 range; every sum
 * accumulates in FP32, every norm in FP64).  MEXCT_F16 mu is accepted but
 * underflows the initial mu = 1e-10 (below FP16's smallest subnormal), so the
 * multiplicative update stays at 0.  BF16 mu (8-bit mantissa) lands ~1e-1 from
 * the FP32 iterates after 20 iterations: outside a 1e-3 accuracy bound.  The
 * low-precision form near it keeps mu and the counts in FP32 and stores the
 * residual views in FP16 (mexct_osctv_create_ex). */
typedef struct mexct_osctv mexct_osctv;

typedef struct mexct_osctv_params {
  int n_iter;          /* numIter */
  float tv_const;      /* TV_constant */
  int n_sub_init;      /* numSubsInit */
  int n_sub_final;     /* numSubsFinal */
  float p_val;         /* pVal */
  int use_graph;       /* capture each iteration as a CUDA graph (cached) */
  int objective;       /* also compute the FP64 data-fidelity objective */
} mexct_osctv_params;

/* pre/post: device [W,H,nP] float32 counts (copied; inputs untouched).
 * mu starts at 1e-10 (OSC_TV_recon.m:33). */
mexct_status mexct_osctv_create(mexct_ctx* ctx, const float* d_pre,
                                const float* d_post, int W, int H, int nP,
                                const float* angles, float sad, int geom,
                                int mu_type, void* stream,
                                mexct_osctv** out);
/* As mexct_osctv_create, with the storage of the residual views (the OSC
 * forward pass's pre e^-l - post and pre e^-l l, read by the dual BP) chosen:
 * MEXCT_F32, or MEXCT_F16 (FP32 mu only) holding the residuals times one power
 * of two that brings the largest count into (2^14, 2^15] (FP16 cannot hold
 * counts above 65504, and small intensities would fall into its subnormal
 * range; the update num/den does not depend on a common scale of the two
 * residuals).  The counts stay FP32: rounding them to FP16 moves the
 * reconstruction itself.  Every sum accumulates in FP32, every norm in FP64. */
mexct_status mexct_osctv_create_ex(mexct_ctx* ctx, const float* d_pre,
                                   const float* d_post, int W, int H, int nP,
                                   const float* angles, float sad, int geom,
                                   int mu_type, int data_type, void* stream,
                                   mexct_osctv** out);
/* Run iterations k0+1 .. k0+n (k0 = iterations already run); first_picks
 * holds one 0-based first subset per iteration of this call. */
mexct_status mexct_osctv_run(mexct_osctv* s, const mexct_osctv_params* p,
                             const int32_t* first_picks, int n, void* stream);
/* Current mu as float32 into device memory (W*W*H). */
mexct_status mexct_osctv_mu(mexct_osctv* s, float* d_out, void* stream);
/* Iterations run so far, the last d_a and the last objective (NaN if off). */
mexct_status mexct_osctv_stats(mexct_osctv* s, int* iters, double* d_a,
                               double* objective);
/* Checkpoint / resume: the full state (mu, mu_old, iteration count, the
 * pre/post element-0 switch) to/from host memory of mexct_osctv_state_bytes. */
size_t mexct_osctv_state_bytes(const mexct_osctv* s);
mexct_status mexct_osctv_snapshot(mexct_osctv* s, void* host, void* stream);
mexct_status mexct_osctv_restore(mexct_osctv* s, const void* host,
                                 void* stream);
mexct_status mexct_osctv_destroy(mexct_osctv* s);

/* recon = OSC_TV_recon(pre, post, angles, geom, numIter, TV_constant,
 * numSubsInit, numSubsFinal, pVal) with host arrays (one call, FP32 mu).
 * Replaces iterative_reconstruction/OSC_TV_recon.m:1-74. */
mexct_status mexct_osc_tv_recon(mexct_ctx* ctx, const float* pre,
                                const float* post, int W, int H, int nP,
                                const float* angles, float sad, int geom,
                                int n_iter, float tv_const, int n_sub_init,
                                int n_sub_final, float p_val,
                                const int32_t* first_picks, float* recon);

/* OSC_TV_recon out of core: as mexct_osc_tv_recon, with mu in host memory
 * streaming through the device in z-slabs, using at most budget_bytes of
 * device memory (no counterpart in the reference, which lists sub-volume
 * reconstruction of larger images as a TODO: CUDAmex_oscIter.cu:28-29).
 * The slab is the whole volume when it fits, else the thickest multiple of 4
 * slices that does (*slab_planes, if non-NULL); the views of the largest
 * subset and the slab buffers must fit (MEXCT_ERR_BUDGET otherwise).  Per
 * voxel the operations are the in-core solver's; a subset's line integrals
 * are FP32 sums of the slabs' parts and the FP64 norms are combined slab by
 * slab.  Host memory: 2 volumes and the clamped counts, pinned. */
mexct_status mexct_osc_tv_recon_ooc(mexct_ctx* ctx, const float* pre,
                                    const float* post, int W, int H, int nP,
                                    const float* angles, float sad, int geom,
                                    int n_iter, float tv_const,
                                    int n_sub_init, int n_sub_final,
                                    float p_val, const int32_t* first_picks,
                                    size_t budget_bytes, float* recon,
                                    int* slab_planes);

/* The slab thickness (slices) and device bytes mexct_osc_tv_recon_ooc uses
 * for a problem within budget_bytes (host-side; MEXCT_ERR_BUDGET if no slab
 * fits). */
mexct_status mexct_osc_tv_ooc_plan(int W, int H, int nP, int geom, int n_iter,
                                   int n_sub_init, int n_sub_final,
                                   float p_val, size_t budget_bytes,
                                   int* slab_planes, size_t* device_bytes);

/* Subset schedule helpers (OSC_TV_recon.m:76-102). */
int mexct_num_subsets(int s_init, int s_final, float p_val, int max_iters,
                      int k);
mexct_status mexct_subset_order(int n_sub, int first_pick, int32_t* picks);

#ifdef __cplusplus
}
#endif
#endif /* MEXCT_SOLVER_H */
