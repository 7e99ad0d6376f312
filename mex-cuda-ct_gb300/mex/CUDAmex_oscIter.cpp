// CUDAmex_oscIter(mu, pre, post, numSubsets, subsetPicks, angles, SAD, geomFlag)
// MEX gateway with the argument list of
// iterative_reconstruction/CUDAmex_oscIter.cu:362-390.  No output: mu (single
// [W, W, H]) is updated in place as in the reference; pre/post (single
// [W, H, nP]) are left unchanged; subsetPicks is int32 (0-based).
#include "gateway.h"

MEXCT_GATEWAY(CUDAmex_oscIter) {
  (void)nlhs;
  (void)plhs;
  const char* fn = "CUDAmex_oscIter";
  mexgw::require_nrhs(nrhs, 8, 8, fn);
  mexgw::require_single(prhs[0], fn, "reconVol");
  mexgw::require_single(prhs[1], fn, "preScan");
  mexgw::require_single(prhs[2], fn, "postScan");
  mexgw::require_single(prhs[5], fn, "scanAngles");
  if (!mxIsInt32(prhs[4])) mexErrMsgIdAndTxt("mexct:class", "%s: subsetPicks must be int32", fn);
  const size_t W = mexgw::dim(prhs[0], 0), H = mexgw::dim(prhs[0], 2);
  if (mexgw::dim(prhs[0], 1) != W) mexErrMsgIdAndTxt("mexct:dims", "%s: reconVol must be W x W x H", fn);
  if (mexgw::dim(prhs[1], 0) != W || mexgw::dim(prhs[1], 1) != H ||
      mexgw::dim(prhs[2], 0) != W || mexgw::dim(prhs[2], 1) != H ||
      mexgw::dim(prhs[1], 2) != mexgw::dim(prhs[2], 2))
    mexErrMsgIdAndTxt("mexct:dims", "%s: preScan/postScan must be W x H x nP", fn);
  const size_t nP = mexgw::dim(prhs[1], 2);
  const int nSub = (int)mxGetScalar(prhs[3]);
  if (nSub <= 0) mexErrMsgIdAndTxt("mexct:invalidInput", "%s: numSubsets must be > 0", fn);
  if (mxGetNumberOfElements(prhs[4]) < (size_t)nSub)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: subsetPicks has fewer than numSubsets entries", fn);
  if (mxGetNumberOfElements(prhs[5]) < nP)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: too few angles", fn);
  mexgw::check(mexct_osc_iter(nullptr, (float*)mxGetData(prhs[0]),
                              (const float*)mxGetData(prhs[1]), (const float*)mxGetData(prhs[2]),
                              mexgw::as_int(W, fn, "W"), mexgw::as_int(H, fn, "H"),
                              mexgw::as_int(nP, fn, "nP"), nSub,
                              (const int32_t*)mxGetData(prhs[4]), (const float*)mxGetData(prhs[5]),
                              (float)mxGetScalar(prhs[6]), (int)mxGetScalar(prhs[7])),
               fn);
}
