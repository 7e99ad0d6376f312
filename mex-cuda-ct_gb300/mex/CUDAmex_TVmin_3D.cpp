// image_out = CUDAmex_TVmin_3D(image_in, tvConst)
// MEX gateway with the argument list of
// iterative_reconstruction/CUDAmex_TVmin_3D.cu:162-185: exactly two arguments,
// 20 TV-descent steps (the reference's hard-coded count).
#include "gateway.h"

MEXCT_GATEWAY(CUDAmex_TVmin_3D) {
  (void)nlhs;
  const char* fn = "CUDAmex_TVmin_3D";
  mexgw::require_nrhs(nrhs, 2, 2, fn);
  mexgw::require_single(prhs[0], fn, "image_in");
  const size_t nx = mexgw::dim(prhs[0], 0), ny = mexgw::dim(prhs[0], 1), nz = mexgw::dim(prhs[0], 2);
  const mwSize dims[3] = {nx, ny, nz};
  plhs[0] = mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
  mexgw::check(mexct_tvmin3d(nullptr, (const float*)mxGetData(prhs[0]), mexgw::as_int(nx, fn, "Nx"),
                             mexgw::as_int(ny, fn, "Ny"), mexgw::as_int(nz, fn, "Nz"),
                             (float)mxGetScalar(prhs[1]), 20, (float*)mxGetData(plhs[0])),
               fn);
}
