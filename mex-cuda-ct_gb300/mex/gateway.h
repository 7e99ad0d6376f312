// gateway.h -- shared helpers of the mexct MEX gateways.
//
// Each gateway keeps the reference's MATLAB name, argument list and array
// layout and forwards to the host entry point of libmexct (include/mexct.h).
// Unlike the reference, the gateways check argument count, class and shape
// and turn every library status into a MATLAB error with id "mexct:*".
#pragma once

#include <stddef.h>
#include <stdint.h>

#include "mex.h"
#include "mexct.h"

#ifdef MEXCT_STUB
#define MEXCT_GATEWAY(name) \
  extern "C" void mexFunction_##name(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[])
#else
#define MEXCT_GATEWAY(name) \
  void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[])
#endif

namespace mexgw {

inline void require_single(const mxArray* a, const char* fn, const char* what) {
  if (!a || !mxIsSingle(a))
    mexErrMsgIdAndTxt("mexct:class", "%s: %s must be single (float32)", fn, what);
}

inline void require_nrhs(int nrhs, int lo, int hi, const char* fn) {
  if (nrhs < lo || nrhs > hi) {
    if (lo == hi)
      mexErrMsgIdAndTxt("mexct:nrhs", "%s: %d arguments expected, got %d", fn, lo, nrhs);
    mexErrMsgIdAndTxt("mexct:nrhs", "%s: %d to %d arguments expected, got %d", fn, lo, hi, nrhs);
  }
}

// Dimension i of a MATLAB array (1 beyond the stored dimensions).
inline size_t dim(const mxArray* a, int i) {
  return (mwSize)i < mxGetNumberOfDimensions(a) ? mxGetDimensions(a)[i] : 1;
}

inline int as_int(size_t v, const char* fn, const char* what) {
  if (v > (size_t)0x7fffffff) mexErrMsgIdAndTxt("mexct:size", "%s: %s too large", fn, what);
  return (int)v;
}

inline void check(mexct_status s, const char* fn) {
  if (s == MEXCT_OK) return;
  const char* id = "mexct:cuda";
  switch (s) {
    case MEXCT_ERR_ARG: id = "mexct:invalidInput"; break;
    case MEXCT_ERR_OOM: id = "mexct:outOfMemory"; break;
    case MEXCT_ERR_UNSUPPORTED: id = "mexct:unsupported"; break;
    case MEXCT_ERR_TIMEOUT: id = "mexct:timeout"; break;
    case MEXCT_ERR_BUDGET: id = "mexct:budget"; break;
    default: break;
  }
  mexErrMsgIdAndTxt(id, "%s: %s", fn, mexct_last_error());
}

}  // namespace mexgw
