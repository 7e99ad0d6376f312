// bp = CUDAmex_BP(projections, SAD, angles, geomFlag)
// MEX gateway with the argument list of projection_kernels/CUDAmex_BP.cu:223-245.
// projections: single [W, H, nP]; output: single [W, W, H].
#include "gateway.h"

MEXCT_GATEWAY(CUDAmex_BP) {
  (void)nlhs;
  const char* fn = "CUDAmex_BP";
  mexgw::require_nrhs(nrhs, 4, 4, fn);
  mexgw::require_single(prhs[0], fn, "projections");
  mexgw::require_single(prhs[2], fn, "angles");
  const size_t W = mexgw::dim(prhs[0], 0), H = mexgw::dim(prhs[0], 1), nP = mexgw::dim(prhs[0], 2);
  if (mxGetNumberOfElements(prhs[2]) < nP)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: %d angles for %d projections", fn,
                      (int)mxGetNumberOfElements(prhs[2]), (int)nP);
  const mwSize dims[3] = {W, W, H};
  plhs[0] = mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
  mexgw::check(mexct_bp(nullptr, (const float*)mxGetData(prhs[0]), mexgw::as_int(W, fn, "W"),
                        mexgw::as_int(H, fn, "H"), mexgw::as_int(nP, fn, "nP"),
                        (float)mxGetScalar(prhs[1]), (const float*)mxGetData(prhs[2]),
                        (int)mxGetScalar(prhs[3]), (float*)mxGetData(plhs[0])),
               fn);
}
