// fp = CUDAmex_general3D_FP(vol, angles, pts, nProj)
// MEX gateway with the argument list of
// projection_kernels/CUDAmex_general3D_FP.cu:154-189.
// vol: single [S, S, Z]; pts: single [W, H, 6] (or [W, H, 6, nProj], one set of
// rays per view); output: single [W, H, nProj].
#include "gateway.h"

MEXCT_GATEWAY(CUDAmex_general3D_FP) {
  (void)nlhs;
  const char* fn = "CUDAmex_general3D_FP";
  mexgw::require_nrhs(nrhs, 4, 4, fn);
  mexgw::require_single(prhs[0], fn, "the volume");
  mexgw::require_single(prhs[1], fn, "angles");
  mexgw::require_single(prhs[2], fn, "pts");
  const size_t S = mexgw::dim(prhs[0], 0), Z = mexgw::dim(prhs[0], 2);
  const size_t W = mexgw::dim(prhs[2], 0), H = mexgw::dim(prhs[2], 1);
  if (mexgw::dim(prhs[2], 2) != 6)
    mexErrMsgIdAndTxt("mexct:dims", "%s: pts must be W x H x 6 (x1,y1,z1,x2,y2,z2)", fn);
  const double np = mxGetScalar(prhs[3]);
  if (!(np >= 0)) mexErrMsgIdAndTxt("mexct:invalidInput", "%s: nProj must be >= 0", fn);
  const int nP = (int)np;
  const size_t pv = mexgw::dim(prhs[2], 3);
  const int per_view = pv > 1 ? 1 : 0;
  if (per_view && pv < (size_t)nP)
    mexErrMsgIdAndTxt("mexct:dims", "%s: pts has %d views, %d requested", fn, (int)pv, nP);
  if (mxGetNumberOfElements(prhs[1]) < (size_t)nP)
    mexErrMsgIdAndTxt("mexct:invalidInput", "%s: too few angles", fn);
  const mwSize dims[3] = {W, H, (mwSize)nP};
  plhs[0] = mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
  mexgw::check(mexct_g3d_fp(nullptr, (const float*)mxGetData(prhs[0]), mexgw::as_int(S, fn, "S"),
                            mexgw::as_int(Z, fn, "Z"), (const float*)mxGetData(prhs[1]),
                            (const float*)mxGetData(prhs[2]), mexgw::as_int(W, fn, "W"),
                            mexgw::as_int(H, fn, "H"), nP, per_view,
                            (float*)mxGetData(plhs[0])),
               fn);
}
