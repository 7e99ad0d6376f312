// mexstub.cpp -- MEX API stub (mxArray shim) plus a C ABI that lets tests and
// tools create arrays and invoke the gateways by name, as MATLAB would.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "mex.h"

struct mxArray_tag {
  mxClassID cls = mxUNKNOWN_CLASS;
  std::vector<mwSize> dims;
  std::vector<unsigned char> data;
};

namespace mexstub {
struct MexError : std::runtime_error {
  std::string id;
  MexError(const std::string& i, const std::string& m) : std::runtime_error(m), id(i) {}
};
thread_local std::string g_msg, g_id;
}  // namespace mexstub

static size_t elem_size(mxClassID c) {
  switch (c) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxINT32_CLASS: return 4;
    default: return 1;
  }
}

extern "C" {

void* mxGetData(const mxArray* a) { return a ? (void*)a->data.data() : nullptr; }
const mwSize* mxGetDimensions(const mxArray* a) { return a->dims.data(); }
mwSize mxGetNumberOfDimensions(const mxArray* a) { return a->dims.size(); }
size_t mxGetNumberOfElements(const mxArray* a) {
  size_t n = 1;
  for (mwSize d : a->dims) n *= d;
  return n;
}
mxClassID mxGetClassID(const mxArray* a) { return a->cls; }
int mxIsSingle(const mxArray* a) { return a->cls == mxSINGLE_CLASS; }
int mxIsInt32(const mxArray* a) { return a->cls == mxINT32_CLASS; }

double mxGetScalar(const mxArray* a) {
  if (!a || a->data.empty()) return 0.0;
  switch (a->cls) {
    case mxDOUBLE_CLASS: return *(const double*)a->data.data();
    case mxSINGLE_CLASS: return *(const float*)a->data.data();
    case mxINT32_CLASS: return *(const int32_t*)a->data.data();
    default: return 0.0;
  }
}

mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls,
                              mxComplexity) {
  mxArray* a = new mxArray_tag();
  a->cls = cls;
  a->dims.assign(dims, dims + ndim);
  // MATLAB drops trailing singleton dimensions beyond the second.
  while (a->dims.size() > 2 && a->dims.back() == 1) a->dims.pop_back();
  while (a->dims.size() < 2) a->dims.push_back(1);
  a->data.assign(mxGetNumberOfElements(a) * elem_size(cls), 0);
  return a;
}

void mexErrMsgTxt(const char* msg) { throw mexstub::MexError("", msg ? msg : ""); }

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw mexstub::MexError(id ? id : "", buf);
}

void mexWarnMsgTxt(const char* msg) { fprintf(stderr, "Warning: %s\n", msg); }

int mexPrintf(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int n = vprintf(fmt, ap);
  va_end(ap);
  return n;
}

// ---- harness C ABI ---------------------------------------------------------
typedef void (*mex_fn)(int, mxArray**, int, const mxArray**);
void mexFunction_CUDAmex_FP(int, mxArray**, int, const mxArray**);
void mexFunction_CUDAmex_BP(int, mxArray**, int, const mxArray**);
void mexFunction_CUDAmex_general3D_FP(int, mxArray**, int, const mxArray**);
void mexFunction_CUDAmex_general3D_BP(int, mxArray**, int, const mxArray**);
void mexFunction_CUDAmex_oscIter(int, mxArray**, int, const mxArray**);
void mexFunction_CUDAmex_TVmin_3D(int, mxArray**, int, const mxArray**);
void mexFunction_CUDAmex_OSC_TV_recon(int, mxArray**, int, const mxArray**);

mxArray* mxs_create(int cls, int ndim, const size_t* dims, const void* data) {
  mxArray* a = mxCreateNumericArray((mwSize)ndim, (const mwSize*)dims, (mxClassID)cls, mxREAL);
  if (data && !a->data.empty()) std::memcpy(a->data.data(), data, a->data.size());
  return a;
}
void mxs_destroy(mxArray* a) { delete a; }
void* mxs_data(mxArray* a) { return mxGetData(a); }
int mxs_class(const mxArray* a) { return (int)a->cls; }
int mxs_ndim(const mxArray* a) { return (int)a->dims.size(); }
size_t mxs_dim(const mxArray* a, int i) { return i < (int)a->dims.size() ? a->dims[i] : 1; }
const char* mxs_error(void) { return mexstub::g_msg.c_str(); }
const char* mxs_error_id(void) { return mexstub::g_id.c_str(); }

// Invoke a gateway by its MATLAB name.  Returns 0 on success, 1 when the
// gateway raised a MATLAB error (text via mxs_error), 2 for an unknown name.
int mxs_call(const char* name, int nlhs, mxArray** plhs, int nrhs, const mxArray** prhs) {
  static const std::map<std::string, mex_fn> table = {
      {"CUDAmex_FP", mexFunction_CUDAmex_FP},
      {"CUDAmex_BP", mexFunction_CUDAmex_BP},
      {"CUDAmex_general3D_FP", mexFunction_CUDAmex_general3D_FP},
      {"CUDAmex_general3D_BP", mexFunction_CUDAmex_general3D_BP},
      {"CUDAmex_oscIter", mexFunction_CUDAmex_oscIter},
      {"CUDAmex_TVmin_3D", mexFunction_CUDAmex_TVmin_3D},
      {"CUDAmex_OSC_TV_recon", mexFunction_CUDAmex_OSC_TV_recon},
  };
  auto it = table.find(name ? name : "");
  if (it == table.end()) return 2;
  mexstub::g_msg.clear();
  mexstub::g_id.clear();
  try {
    it->second(nlhs, plhs, nrhs, prhs);
  } catch (const mexstub::MexError& e) {
    mexstub::g_msg = e.what();
    mexstub::g_id = e.id;
    return 1;
  }
  return 0;
}

}  // extern "C"
