// bp = CUDAmex_general3D_BP(projections, angles, pts, M, N)
// MEX gateway with the argument list of
// projection_kernels/CUDAmex_general3D_BP.cu:194-229.
// projections: single [W, H, nP]; pts: single [W, H, 6] (or per view
// [W, H, 6, nP]); output: single [M, M, N].
#include "gateway.h"

MEXCT_GATEWAY(CUDAmex_general3D_BP) {
  (void)nlhs;
  const char* fn = "CUDAmex_general3D_BP";
  mexgw::require_nrhs(nrhs, 5, 5, fn);
  mexgw::require_single(prhs[0], fn, "projections");
  mexgw::require_single(prhs[1], fn, "angles");
  mexgw::require_single(prhs[2], fn, "pts");
  const size_t W = mexgw::dim(prhs[0], 0), H = mexgw::dim(prhs[0], 1), nP = mexgw::dim(prhs[0], 2);
  if (mexgw::dim(prhs[2], 0) != W || mexgw::dim(prhs[2], 1) != H || mexgw::dim(prhs[2], 2) != 6)
    mexErrMsgIdAndTxt("mexct:dims", "%s: pts must be W x H x 6 matching the projections", fn);
  const size_t pv = mexgw::dim(prhs[2], 3);
  const int per_view = pv > 1 ? 1 : 0;
  if (per_view && pv < nP) mexErrMsgIdAndTxt("mexct:dims", "%s: pts has too few views", fn);
  if (mxGetNumberOfElements(prhs[1]) < nP)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: too few angles", fn);
  const double m = mxGetScalar(prhs[3]), n = mxGetScalar(prhs[4]);
  if (!(m >= 1) || !(n >= 1)) mexErrMsgIdAndTxt("mexct:invalidInput", "%s: M, N must be >= 1", fn);
  const mwSize dims[3] = {(mwSize)m, (mwSize)m, (mwSize)n};
  plhs[0] = mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
  mexgw::check(mexct_g3d_bp(nullptr, (const float*)mxGetData(prhs[0]), mexgw::as_int(W, fn, "W"),
                            mexgw::as_int(H, fn, "H"), mexgw::as_int(nP, fn, "nP"),
                            (const float*)mxGetData(prhs[1]), (const float*)mxGetData(prhs[2]),
                            per_view, (int)m, (int)n, (float*)mxGetData(plhs[0])),
               fn);
}
