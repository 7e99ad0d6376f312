/*
 * mexct_batch.h -- batched FP / BP over many independent problems of
 * different sizes and geometries (C ABI of libmexct; conventions as in
 * mexct.h).  No counterpart in the reference, which runs one problem per MEX
 * call; each problem computes exactly what mexct_fp_dev / mexct_bp_dev compute
 * for it (CUDAmex_FP.cu:56-346, CUDAmex_BP.cu:44-221).
 */
#ifndef MEXCT_BATCH_H
#define MEXCT_BATCH_H
#include "mexct.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct mexct_problem {
  int W, H, nP, geom;   /* volume W x W x H, detector W x H, views, geomFlag */
  float sad;
  const float* angles;  /* host, nP float32 radians */
  const float* d_vol;   /* device FP32 volume [W,W,H] (input of FP) */
  float* d_sino;        /* device FP32 sinogram [W,H,nP] (FP output, BP input) */
  float* d_rec;         /* device FP32 volume [W,W,H] (BP output) */
} mexct_problem;

typedef struct mexct_batch mexct_batch;

/* Plan a batch: per-problem padded buffers and device descriptors (uploads
 * synchronously).  The device pointers must stay valid while it is used. */
mexct_status mexct_batch_create(mexct_ctx* ctx, const mexct_problem* probs, int n,
                                mexct_batch** out);
/* FP of every problem: one batched padding launch + one persistent launch.
 * Stream-ordered, no host work, capturable in a CUDA graph. */
mexct_status mexct_batch_fp(mexct_batch* b, void* stream);
/* BP of every problem (d_sino -> d_rec): per problem a padding launch and its
 * BP launches (quad / pair view layouts, one view block), fanned out over 8
 * streams by fork / join events on `stream`, so a capture records them as
 * concurrent graph branches.  Stream-ordered, no host work. */
mexct_status mexct_batch_bp(mexct_batch* b, void* stream);
mexct_status mexct_batch_destroy(mexct_batch* b);

#ifdef __cplusplus
}
#endif
#endif /* MEXCT_BATCH_H */
