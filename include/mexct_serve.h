/*
 * mexct_serve.h -- request server of libmexct (C ABI; conventions as in
 * mexct.h).  No counterpart in the reference, which runs one blocking MEX call
 * at a time and resets the device after each OSC iteration.
 *
 * A server owns `slots` worker threads, each with its own context (stream and
 * workspaces).  Submitted FDK (FBP_recon.m) or OSC-TV (OSC_TV_recon.m)
 * requests queue in arrival order and are admitted to a free slot as soon as
 * their HBM footprint fits the budget next to the requests already running
 * (first fit in arrival order), so work of different sizes overlaps on the
 * device.  Results are the same as the one-request entry points
 * (mexct_fbp / mexct_osc_tv_recon): every kernel of these paths is
 * deterministic and independent of what else runs.
 */
#ifndef MEXCT_SERVE_H
#define MEXCT_SERVE_H
#include "mexct.h"
#ifdef __cplusplus
extern "C" {
#endif

#define MEXCT_REQ_FDK 0
#define MEXCT_REQ_OSCTV 1

typedef struct mexct_request {
  int kind;              /* MEXCT_REQ_FDK or MEXCT_REQ_OSCTV */
  int W, H, nP, geom;    /* detector W x H (volume W x W x H), views, geomFlag */
  float sad;
  int mu_type;           /* OSC-TV storage of mu: MEXCT_F32 or MEXCT_BF16 */
  const float* angles;   /* host, nP float32 radians */
  const float* pre;      /* host [W,H,nP] counts */
  const float* post;     /* host [W,H,nP] counts */
  float* recon;          /* host [W,W,H] output, written before completion */
  int filter;            /* FDK: filter (0..5), cutoff, Parker q */
  float cutoff, q;
  int n_iter;            /* OSC-TV: numIter, TV_constant, subsets, pVal */
  float tv_const;
  int n_sub_init, n_sub_final;
  float p_val;
  const int32_t* first_picks; /* OSC-TV: n_iter 0-based first subsets */
  double simulate_s;     /* > 0: no GPU work, the slot is held this long */
  int data_type;         /* OSC-TV: storage of the residual views, MEXCT_F32
                            (0 counts as F32) or MEXCT_F16 (FP32 mu only) */
} mexct_request;

typedef struct mexct_server mexct_server;

typedef struct mexct_server_stats {
  long long submitted, completed, failed, rejected;
  size_t bytes_in_use, peak_bytes, budget;
  int max_concurrent;
} mexct_server_stats;

/* HBM footprint the server charges a request (bytes). */
size_t mexct_request_bytes(const mexct_request* r);

/* device -1 creates a host-only server that accepts only simulated requests
 * (for testing admission and scheduling without a GPU). */
mexct_status mexct_server_create(int device, int slots, size_t hbm_budget,
                                 mexct_server** out);
/* Queue a request; host arrays must stay valid until it completes.  A request
 * whose footprint exceeds the whole budget is rejected (MEXCT_ERR_BUDGET). */
mexct_status mexct_server_submit(mexct_server* s, const mexct_request* r,
                                 unsigned long long* ticket);
/* Wait up to timeout_s (< 0: forever) for a ticket.  On completion returns
 * MEXCT_OK and fills the request's status and its queue / run / total seconds;
 * MEXCT_ERR_TIMEOUT if still pending. */
mexct_status mexct_server_wait(mexct_server* s, unsigned long long ticket,
                               double timeout_s, mexct_status* result,
                               double* queue_s, double* run_s, double* total_s);
mexct_status mexct_server_stats_get(mexct_server* s, mexct_server_stats* out);
/* Drain the queue, join the workers, free everything. */
mexct_status mexct_server_destroy(mexct_server* s);

#ifdef __cplusplus
}
#endif
#endif /* MEXCT_SERVE_H */
