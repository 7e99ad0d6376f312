// fp = CUDAmex_FP(vol, SAD, angles, nProj, geomFlag)
// MEX gateway with the argument list of projection_kernels/CUDAmex_FP.cu:350-376.
// vol: single [W, W, H]; SAD: scalar; angles: single [nProj]; geomFlag 0/1/2
// (optional: 0 when omitted, where the reference reads an undefined prhs[4]).
// Output: single [W, H, nProj].
#include "gateway.h"

MEXCT_GATEWAY(CUDAmex_FP) {
  (void)nlhs;
  const char* fn = "CUDAmex_FP";
  mexgw::require_nrhs(nrhs, 4, 5, fn);
  mexgw::require_single(prhs[0], fn, "the volume");
  mexgw::require_single(prhs[2], fn, "angles");
  const size_t W = mexgw::dim(prhs[0], 0), W1 = mexgw::dim(prhs[0], 1), H = mexgw::dim(prhs[0], 2);
  if (W != W1) mexErrMsgIdAndTxt("mexct:dims", "%s: volume must be W x W x H", fn);
  const double np = mxGetScalar(prhs[3]);
  if (!(np >= 0)) mexErrMsgIdAndTxt("mexct:invalidInput", "%s: nProj must be >= 0", fn);
  const int nP = (int)np;
  if (mxGetNumberOfElements(prhs[2]) < (size_t)nP)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: %d angles for %d projections", fn,
                      (int)mxGetNumberOfElements(prhs[2]), nP);
  const int geom = nrhs > 4 ? (int)mxGetScalar(prhs[4]) : 0;
  const mwSize dims[3] = {W, H, (mwSize)nP};
  plhs[0] = mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
  mexgw::check(mexct_fp(nullptr, (const float*)mxGetData(prhs[0]), mexgw::as_int(W, fn, "W"),
                        mexgw::as_int(H, fn, "H"), (float)mxGetScalar(prhs[1]),
                        (const float*)mxGetData(prhs[2]), nP, geom, (float*)mxGetData(plhs[0])),
               fn);
}
