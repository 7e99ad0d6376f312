// recon = CUDAmex_OSC_TV_recon(pre, post, scanAngles, SAD, geomFlag, numIter,
//                              TV_constant, numSubsInit, numSubsFinal, pVal,
//                              firstPicks [, deviceBudgetBytes])
// [recon, slabPlanes] = CUDAmex_OSC_TV_recon(..., deviceBudgetBytes)
//
// The whole OSC_TV_recon.m driver (iterative_reconstruction/OSC_TV_recon.m:1-74)
// in one call on the device: mu, the counts and every subset's FP / dual BP stay
// resident, and the 20 TV steps follow each iteration from the second on.  The
// driver's geom struct becomes SAD and geomFlag (0 par3d, 1 fan3d, 2 cone3d, as
// its dispatch at :51-59), and its per-iteration random first subset
// (randperm at :82) is passed in: firstPicks is int32 with one 0-based entry per
// iteration (the rest of each iteration's order follows :83-102).  pre / post
// are single [W, H, nP] and are not modified; recon is single [W, W, H].
// With deviceBudgetBytes, mu stays in host memory and streams through the
// device in z-slabs within that many bytes (sub-volume reconstruction, a TODO
// of the reference at CUDAmex_oscIter.cu:28-29); the optional second output is
// the slab thickness in slices.
#include "gateway.h"
#include "mexct_solver.h"

MEXCT_GATEWAY(CUDAmex_OSC_TV_recon) {
  const char* fn = "CUDAmex_OSC_TV_recon";
  mexgw::require_nrhs(nrhs, 11, 12, fn);
  if (nlhs > (nrhs == 12 ? 2 : 1))
    mexErrMsgIdAndTxt("mexct:nlhs", "%s: too many outputs", fn);
  mexgw::require_single(prhs[0], fn, "pre");
  mexgw::require_single(prhs[1], fn, "post");
  mexgw::require_single(prhs[2], fn, "scanAngles");
  if (!mxIsInt32(prhs[10])) mexErrMsgIdAndTxt("mexct:class", "%s: firstPicks must be int32", fn);
  const size_t W = mexgw::dim(prhs[1], 0), H = mexgw::dim(prhs[1], 1), nP = mexgw::dim(prhs[1], 2);
  if (mxGetNumberOfDimensions(prhs[0]) > 3 || mxGetNumberOfDimensions(prhs[1]) > 3 ||
      mexgw::dim(prhs[0], 0) != W || mexgw::dim(prhs[0], 1) != H || mexgw::dim(prhs[0], 2) != nP)
    mexErrMsgIdAndTxt("mexct:dims", "%s: pre and post must both be W x H x nP", fn);
  if (mxGetNumberOfElements(prhs[2]) < nP)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: too few angles", fn);
  const int numIter = (int)mxGetScalar(prhs[5]);
  if (numIter < 1) mexErrMsgIdAndTxt("mexct:invalidInput", "%s: numIter must be >= 1", fn);
  if (mxGetNumberOfElements(prhs[10]) < (size_t)numIter)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: firstPicks needs one entry per iteration", fn);
  double budget = 0.0;
  if (nrhs == 12) {
    budget = mxGetScalar(prhs[11]);
    if (!(budget >= 1.0) || budget > 9.0e18)
      mexErrMsgIdAndTxt("mexct:invalidInput", "%s: deviceBudgetBytes must be a positive byte count",
                        fn);
  }
  const int w = mexgw::as_int(W, fn, "W"), h = mexgw::as_int(H, fn, "H");
  const int np = mexgw::as_int(nP, fn, "nP");
  const mwSize dims[3] = {W, W, H};
  plhs[0] = mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
  const float* pre = (const float*)mxGetData(prhs[0]);
  const float* post = (const float*)mxGetData(prhs[1]);
  const float* ang = (const float*)mxGetData(prhs[2]);
  const float sad = (float)mxGetScalar(prhs[3]);
  const int geom = (int)mxGetScalar(prhs[4]);
  const float tv = (float)mxGetScalar(prhs[6]);
  const int s0 = (int)mxGetScalar(prhs[7]), s1 = (int)mxGetScalar(prhs[8]);
  const float pval = (float)mxGetScalar(prhs[9]);
  const int32_t* picks = (const int32_t*)mxGetData(prhs[10]);
  float* recon = (float*)mxGetData(plhs[0]);
  if (nrhs == 12) {
    int planes = 0;
    mexgw::check(mexct_osc_tv_recon_ooc(nullptr, pre, post, w, h, np, ang, sad, geom, numIter, tv,
                                        s0, s1, pval, picks, (size_t)budget, recon, &planes),
                 fn);
    if (nlhs > 1) {
      const mwSize one[2] = {1, 1};
      plhs[1] = mxCreateNumericArray(2, one, mxDOUBLE_CLASS, mxREAL);
      *(double*)mxGetData(plhs[1]) = (double)planes;
    }
  } else {
    mexgw::check(mexct_osc_tv_recon(nullptr, pre, post, w, h, np, ang, sad, geom, numIter, tv, s0,
                                    s1, pval, picks, recon),
                 fn);
  }
}
