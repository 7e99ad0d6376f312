/*
 * mex.h (stub) -- the subset of MATLAB's MEX C API that the mexct gateways
 * use, for building and testing the gateways without MATLAB.
 *
 * With MATLAB present, the gateways compile against MATLAB's own mex.h
 * instead (mexcuda or mex with MATLAB's include path).  In this stub:
 *   - arrays are column-major buffers with a class id and dimensions;
 *   - mexErrMsgTxt / mexErrMsgIdAndTxt throw mexstub::MexError (MATLAB
 *     longjmps back to the prompt; the stub unwinds back to mxs_call()).
 */
#ifndef MEXCT_MEXSTUB_MEX_H
#define MEXCT_MEXSTUB_MEX_H

#include <stddef.h>
#include <stdint.h>

typedef size_t mwSize;
typedef size_t mwIndex;

typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxDOUBLE_CLASS = 6,
  mxSINGLE_CLASS = 7,
  mxINT32_CLASS = 12,
} mxClassID;

typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct mxArray_tag mxArray;

#ifdef __cplusplus
extern "C" {
#endif

void* mxGetData(const mxArray* a);
const mwSize* mxGetDimensions(const mxArray* a);
mwSize mxGetNumberOfDimensions(const mxArray* a);
size_t mxGetNumberOfElements(const mxArray* a);
double mxGetScalar(const mxArray* a);
mxClassID mxGetClassID(const mxArray* a);
int mxIsSingle(const mxArray* a);
int mxIsInt32(const mxArray* a);
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls,
                              mxComplexity cplx);
void mexErrMsgTxt(const char* msg);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
void mexWarnMsgTxt(const char* msg);
int mexPrintf(const char* fmt, ...);

#ifdef __cplusplus
}
#endif

#endif
