/*
 * ref_launch.cu -- host launcher for the reference's own CUDA kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  It loads the cubins that oracle/ref_build.py
 * compiles, unmodified, from the reference's .cu files and runs their kernels
 * on the GPU with the host-side steps of the reference's mexFunction gateways
 * restated here (MATLAB is absent, and the gateways' host code was built for
 * x86 MEX hosts).  Its outputs are the reference outputs that pin the FP64
 * oracle and the CUDA library (tests/golden/make_ref_golden.py); it is also
 * timed beside the library on the same GPU.  Nothing in the product links or
 * calls it.
 *
 * What is the reference's and what is restated:
 *   - every kernel is the reference's own compiled code, launched with the
 *     reference's grid, block and argument values;
 *   - texture and surface references (removed in CUDA 12) are objects here,
 *     created with the reference's address mode, linear filtering and
 *     unnormalised coordinates, their handles written into the __device__
 *     variables that oracle/ref_compat.h gives each reference;
 *   - per-view loops, copies and synchronisations follow the gateways line by
 *     line (cited per function), with the deprecated cudaMemcpyToArray /
 *     FromArray written as their cudaMemcpy2D*Array equivalents;
 *   - the angle's sine and cosine are the correctly rounded binary32 values
 *     of the binary32 angle (the gateways call the host C library's sincosf,
 *     whose last bit depends on that library);
 *   - deviations, each in code the reference leaves undefined or harmful:
 *     the TV gradient buffer is zeroed once before the descent (the reference
 *     never writes its border and reads whatever cudaMalloc returned), and the
 *     OSC gateway's closing cudaDeviceReset (CUDAmex_oscIter.cu:582) is left
 *     out, since it would destroy every other allocation of the process.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/functional.h>
#include <thrust/transform.h>
#include <thrust/transform_reduce.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

namespace {

char g_err[1024] = "";
std::string g_dir;
double g_last_ms = 0.0;

#define RT(x)                                                                                  \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess) {                                                                   \
      snprintf(g_err, sizeof g_err, "%s: %s (line %d)", #x, cudaGetErrorString(e_), __LINE__); \
      return 1;                                                                                \
    }                                                                                          \
  } while (0)

#define DR(x)                                                                     \
  do {                                                                            \
    CUresult r_ = (x);                                                            \
    if (r_ != CUDA_SUCCESS) {                                                     \
      const char* s_ = "?";                                                       \
      cuGetErrorString(r_, &s_);                                                  \
      snprintf(g_err, sizeof g_err, "%s: %s (line %d)", #x, s_, __LINE__);        \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

#define CK(x)          \
  do {                 \
    if ((x) != 0) {    \
      return 1;        \
    }                  \
  } while (0)

struct Module {
  const char* file;
  CUmodule mod;
};
Module g_fp = {"ref_fp.cubin", nullptr}, g_bp = {"ref_bp.cubin", nullptr},
       g_g3fp = {"ref_g3d_fp.cubin", nullptr}, g_g3bp = {"ref_g3d_bp.cubin", nullptr},
       g_osc = {"ref_osc.cubin", nullptr}, g_tv = {"ref_tv.cubin", nullptr};

int load(Module& m) {
  if (m.mod) return 0;
  RT(cudaFree(nullptr));  // make the runtime's primary context current
  std::string p = g_dir + "/" + m.file;
  DR(cuModuleLoad(&m.mod, p.c_str()));
  return 0;
}

int kernel(Module& m, const char* mangled, CUfunction* f) {
  CK(load(m));
  DR(cuModuleGetFunction(f, m.mod, mangled));
  return 0;
}

// Write an object handle into the first 8 bytes of a reference's __device__
// texture / surface variable (ref_compat.h keeps the handle first).
int set_handle(Module& m, const char* var, unsigned long long h) {
  CK(load(m));
  CUdeviceptr p;
  size_t sz = 0;
  DR(cuModuleGetGlobal(&p, &sz, m.mod, var));
  if (sz < sizeof h) {
    snprintf(g_err, sizeof g_err, "device variable %s has %zu bytes", var, sz);
    return 1;
  }
  DR(cuMemcpyHtoD(p, &h, sizeof h));
  return 0;
}

int launch(CUfunction f, dim3 g, dim3 b, void** args) {
  DR(cuLaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, 0, nullptr, args, nullptr));
  return 0;
}

int tex_object(cudaArray_t a, cudaTextureAddressMode am, cudaTextureObject_t* t) {
  cudaResourceDesc rd;
  memset(&rd, 0, sizeof rd);
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = a;
  cudaTextureDesc td;
  memset(&td, 0, sizeof td);
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = am;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 0;
  RT(cudaCreateTextureObject(t, &rd, &td, nullptr));
  return 0;
}

int surf_object(cudaArray_t a, cudaSurfaceObject_t* s) {
  cudaResourceDesc rd;
  memset(&rd, 0, sizeof rd);
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = a;
  RT(cudaCreateSurfaceObject(s, &rd));
  return 0;
}

void trig(float beta, float* s, float* c) {
  *s = (float)std::sin((double)beta);
  *c = (float)std::cos((double)beta);
}

unsigned nblocks32(unsigned n) { return n % 32 == 0 ? n / 32 : n / 32 + 1; }

// Host volume [W,W,H] (x fastest) into / out of a 3D array, as the gateways'
// cudaMemcpy3D with make_cudaPitchedPtr(vol, W*4, H, W) does.
int vol_to_array(const float* v, cudaArray_t a, size_t W, size_t H) {
  cudaMemcpy3DParms p;
  memset(&p, 0, sizeof p);
  p.srcPtr = make_cudaPitchedPtr((void*)v, W * sizeof(float), W, W);
  p.dstArray = a;
  p.extent = make_cudaExtent(W, W, H);
  p.kind = cudaMemcpyHostToDevice;
  RT(cudaMemcpy3D(&p));
  return 0;
}

int array_to_vol(cudaArray_t a, float* v, size_t W, size_t H) {
  cudaMemcpy3DParms p;
  memset(&p, 0, sizeof p);
  p.srcArray = a;
  p.dstPtr = make_cudaPitchedPtr((void*)v, W * sizeof(float), W, W);
  p.extent = make_cudaExtent(W, W, H);
  p.kind = cudaMemcpyDeviceToHost;
  RT(cudaMemcpy3D(&p));
  return 0;
}

struct Timer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  ~Timer() {
    g_last_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};

// thrust functors of CUDAmex_TVmin_3D.cu:69-90 (x*x and a*x + y), restated.
struct sq_f {
  __host__ __device__ float operator()(const float& x) const { return x * x; }
};
struct saxpy_f {
  const float a;
  explicit saxpy_f(float a_) : a(a_) {}
  __host__ __device__ float operator()(const float& x, const float& y) const { return a * x + y; }
};

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err; }
double ref_last_ms(void) { return g_last_ms; }

int ref_init(const char* cubin_dir) {
  g_dir = cubin_dir;
  int n = 0;
  RT(cudaGetDeviceCount(&n));
  if (n < 1) {
    snprintf(g_err, sizeof g_err, "no CUDA device");
    return 1;
  }
  return 0;
}

/* CUDAmex_FP gateway, CUDAmex_FP.cu:350-477.  vol [W,W,H] -> out [W,H,nP]. */
int ref_fp(const float* vol, int W_, int H_, float D, const float* ang, int nP, int geom, float* out) {
  Timer tm;
  static const char* names[3] = {"_Z21forwardProjKernel_parPfffffffffffjjjjj",
                                 "_Z21forwardProjKernel_fanPfffffffffffjjjjj",
                                 "_Z22forwardProjKernel_conePfffffffffffjjjjj"};
  if (geom < 0 || geom > 2) {
    snprintf(g_err, sizeof g_err, "invalid geometry");
    return 1;
  }
  CUfunction f;
  CK(kernel(g_fp, names[geom], &f));
  unsigned width = W_, height = H_;
  float u0 = float(W_ - 1) / 2, v0 = float(H_ - 1) / 2;  // :378-379
  float* projection = nullptr;
  size_t pbytes = (size_t)width * height * sizeof(float);
  RT(cudaMalloc(&projection, pbytes));
  RT(cudaMemset(projection, 0, pbytes));
  cudaChannelFormatDesc cd = cudaCreateChannelDesc<float>();
  cudaArray_t arr;
  RT(cudaMalloc3DArray(&arr, &cd, make_cudaExtent(width, width, height), 0));
  cudaTextureObject_t tex;
  CK(tex_object(arr, cudaAddressModeClamp, &tex));  // :405-409
  CK(set_handle(g_fp, "reconTex", tex));
  CK(vol_to_array(vol, arr, width, height));
  float bx = -(float)width / 2.0, by = -(float)width / 2.0, bz = -(float)height / 2.0;  // :424-426
  float voxel = 1.0f;
  unsigned isx = width, isy = width, isz = height;
  dim3 block(32, 32), grid(nblocks32(width), nblocks32(width));  // :432-440
  for (int p = 0; p < nP; ++p) {
    float s, c;
    trig(ang[p], &s, &c);
    void* args[] = {&projection, &bx, &by, &bz, &u0, &v0, &s, &c, &D, &D, &voxel,
                    &isx, &isy, &isz, &width, &height};
    CK(launch(f, grid, block, args));
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(out + (size_t)p * width * height, projection, pbytes, cudaMemcpyDeviceToHost));
  }
  cudaDestroyTextureObject(tex);
  cudaFreeArray(arr);
  cudaFree(projection);
  return 0;
}

/* CUDAmex_BP gateway, CUDAmex_BP.cu:223-324.  sino [W,H,nP] -> vol [W,W,H]. */
int ref_bp(const float* sino, int W_, int H_, int nP, float D, const float* ang, int geom, float* vol) {
  Timer tm;
  static const char* names[3] = {"_Z18backprojKernel_parPfffffjj", "_Z18backprojKernel_fanPfffffjj",
                                 "_Z19backprojKernel_conePfffffjj"};
  if (geom < 0 || geom > 2) {
    snprintf(g_err, sizeof g_err, "invalid geometry");
    return 1;
  }
  CUfunction f;
  CK(kernel(g_bp, names[geom], &f));
  unsigned width = W_, height = H_;
  float v0 = float(H_ - 1) / 2;  // :246
  float* output = nullptr;
  size_t vbytes = (size_t)width * width * height * sizeof(float);
  RT(cudaMalloc(&output, vbytes));
  RT(cudaMemset(output, 0, vbytes));
  cudaChannelFormatDesc cd = cudaCreateChannelDesc<float>();
  cudaArray_t arr;
  RT(cudaMallocArray(&arr, &cd, width, height));
  cudaTextureObject_t tex;
  CK(tex_object(arr, cudaAddressModeClamp, &tex));  // :269-273
  CK(set_handle(g_bp, "projtex", tex));
  dim3 block(32, 32), grid(nblocks32(width), nblocks32(width));  // :276-284
  for (int p = 0; p < nP; ++p) {
    float s, c;
    trig(ang[p], &s, &c);
    RT(cudaMemcpy2DToArray(arr, 0, 0, sino + (size_t)p * width * height, width * sizeof(float),
                           width * sizeof(float), height, cudaMemcpyHostToDevice));
    void* args[] = {&output, &v0, &s, &c, &D, &width, &height};
    CK(launch(f, grid, block, args));
    RT(cudaDeviceSynchronize());
  }
  RT(cudaMemcpy(vol, output, vbytes, cudaMemcpyDeviceToHost));
  cudaDestroyTextureObject(tex);
  cudaFreeArray(arr);
  cudaFree(output);
  return 0;
}

/* CUDAmex_general3D_FP gateway, CUDAmex_general3D_FP.cu:154-252.
 * vol [S,S,Z], pts [W,H,6] -> out [W,H,nP]. */
int ref_g3d_fp(const float* vol, int S_, int Z_, const float* ang, const float* pts, int W_, int H_, int nP,
               float* out) {
  Timer tm;
  CUfunction f;
  CK(kernel(g_g3fp, "_Z17forwardProjKernelPfS_ffffffjjjjj", &f));
  unsigned width = W_, height = H_, side = S_, nsl = Z_;
  float bx = -(float)side / 2.0, by = bx, bz = -(float)nsl / 2.0, voxel = 1.0f;  // :174-177
  dim3 block(32, 32), grid((int)std::ceil(width / 32.f), (int)std::ceil(height / 32.f));  // :179-180
  size_t pbytes = (size_t)width * height * sizeof(float);
  float *projection = nullptr, *dpts = nullptr;
  RT(cudaMalloc(&projection, pbytes));
  RT(cudaMemset(projection, 0, pbytes));
  RT(cudaMalloc(&dpts, pbytes * 6));
  RT(cudaMemcpy(dpts, pts, pbytes * 6, cudaMemcpyHostToDevice));
  cudaChannelFormatDesc cd = cudaCreateChannelDesc<float>();
  cudaArray_t arr;
  RT(cudaMalloc3DArray(&arr, &cd, make_cudaExtent(side, side, nsl), 0));
  cudaTextureObject_t tex;
  CK(tex_object(arr, cudaAddressModeBorder, &tex));  // :217-221
  CK(set_handle(g_g3fp, "reconTex", tex));
  CK(vol_to_array(vol, arr, side, nsl));
  for (int p = 0; p < nP; ++p) {
    float s, c;
    trig(ang[p], &s, &c);
    void* args[] = {&projection, &dpts, &bx, &by, &bz, &s, &c, &voxel, &side, &side, &nsl, &width, &height};
    CK(launch(f, grid, block, args));
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(out + (size_t)p * width * height, projection, pbytes, cudaMemcpyDeviceToHost));
  }
  cudaDestroyTextureObject(tex);
  cudaFreeArray(arr);
  cudaFree(projection);
  cudaFree(dpts);
  return 0;
}

/* CUDAmex_general3D_BP gateway, CUDAmex_general3D_BP.cu:194-282.
 * sino [W,H,nP], pts [W,H,6] -> vol [S,S,Z] (float atomics: summation order
 * varies from run to run). */
int ref_g3d_bp(const float* sino, int W_, int H_, int nP, const float* ang, const float* pts, int S_, int Z_,
               float* vol) {
  Timer tm;
  CUfunction f;
  CK(kernel(g_g3bp, "_Z14backProjKernelPfS_S_ffffffjjjjjj", &f));
  unsigned width = W_, height = H_, side = S_, nsl = Z_, nproj = nP;
  float bx = -(float)side / 2.0, by = bx, bz = -(float)nsl / 2.0, voxel = 1.0f;  // :215-218
  dim3 block(32, 32), grid((int)std::ceil(width / 32.f), (int)std::ceil(height / 32.f));  // :220-221
  size_t pbytes = (size_t)width * height * sizeof(float);
  size_t vbytes = (size_t)side * side * nsl * sizeof(float);
  float *projection = nullptr, *dpts = nullptr, *output = nullptr;
  RT(cudaMalloc(&projection, pbytes));
  RT(cudaMemset(projection, 0, pbytes));
  RT(cudaMalloc(&dpts, pbytes * 6));
  RT(cudaMemcpy(dpts, pts, pbytes * 6, cudaMemcpyHostToDevice));
  RT(cudaMalloc(&output, vbytes));
  RT(cudaMemset(output, 0, vbytes));
  for (int p = 0; p < nP; ++p) {
    float s, c;
    trig(ang[p], &s, &c);
    RT(cudaMemcpy(projection, sino + (size_t)p * width * height, pbytes, cudaMemcpyHostToDevice));
    void* args[] = {&output, &projection, &dpts, &bx, &by, &bz, &s, &c, &voxel,
                    &side, &side, &nsl, &width, &height, &nproj};
    CK(launch(f, grid, block, args));
    RT(cudaDeviceSynchronize());
  }
  RT(cudaMemcpy(vol, output, vbytes, cudaMemcpyDeviceToHost));
  cudaFree(output);
  cudaFree(projection);
  cudaFree(dpts);
  return 0;
}

/* CUDAmex_oscIter gateway, CUDAmex_oscIter.cu:362-584.  mu [W,W,H] updated in
 * place; pre / post [W,H,nP] are overwritten with the residual views of the
 * last pass, as the gateway does (:527-528). */
int ref_osc_iter(float* mu, float* pre, float* post, int W_, int H_, int nP, int nSub, const int32_t* picks,
                 const float* ang, float D, int geom) {
  Timer tm;
  CUfunction fzero, fupd, ffp, fbp;
  CK(kernel(g_osc, "_Z18oscSetCorrTermZerojj", &fzero));
  CK(kernel(g_osc, "_Z19oscIterUpdateKerneljj", &fupd));
  CK(kernel(g_osc, "_Z24oscIterForwardProjKernelffffffffffjjjjji", &ffp));
  CK(kernel(g_osc, "_Z21oscIterBackProjKernelffffjji", &fbp));
  unsigned width = W_, height = H_;
  float u0 = float(W_ - 1) / 2, v0 = float(H_ - 1) / 2;  // :401-402
  cudaChannelFormatDesc cd = cudaCreateChannelDesc<float>();
  cudaArray_t pre_a, post_a, rec_a, num_a, den_a;
  RT(cudaMallocArray(&pre_a, &cd, width, height, cudaArraySurfaceLoadStore));
  RT(cudaMallocArray(&post_a, &cd, width, height, cudaArraySurfaceLoadStore));
  cudaExtent ext = make_cudaExtent(width, width, height);
  RT(cudaMalloc3DArray(&rec_a, &cd, ext, cudaArraySurfaceLoadStore));
  RT(cudaMalloc3DArray(&num_a, &cd, ext, cudaArraySurfaceLoadStore));
  RT(cudaMalloc3DArray(&den_a, &cd, ext, cudaArraySurfaceLoadStore));
  cudaTextureObject_t pre_t, post_t, rec_t;
  CK(tex_object(pre_a, cudaAddressModeBorder, &pre_t));  // :417-425
  CK(tex_object(post_a, cudaAddressModeBorder, &post_t));
  CK(tex_object(rec_a, cudaAddressModeBorder, &rec_t));  // :458-462
  cudaSurfaceObject_t pre_s, post_s, rec_s, num_s, den_s;
  CK(surf_object(pre_a, &pre_s));
  CK(surf_object(post_a, &post_s));
  CK(surf_object(rec_a, &rec_s));
  CK(surf_object(num_a, &num_s));
  CK(surf_object(den_a, &den_s));
  CK(set_handle(g_osc, "preScanProjTex", pre_t));
  CK(set_handle(g_osc, "postScanProjTex", post_t));
  CK(set_handle(g_osc, "reconTex", rec_t));
  CK(set_handle(g_osc, "preSurf", pre_s));
  CK(set_handle(g_osc, "postSurf", post_s));
  CK(set_handle(g_osc, "reconSurf", rec_s));
  CK(set_handle(g_osc, "correctionVolumeNumeratorSurf", num_s));
  CK(set_handle(g_osc, "correctionVolumeDenominatorSurf", den_s));
  CK(vol_to_array(mu, rec_a, width, height));
  float bx = -(float)width / 2.0, by = -(float)width / 2.0, bz = -(float)height / 2.0;  // :483-485
  float voxel = 1.0f;
  unsigned isx = width, isy = width, isz = height;
  dim3 block(32, 32), grid(nblocks32(width), nblocks32(width));  // :492-500
  size_t pix = (size_t)width * height, prow = width * sizeof(float);
  {
    void* args[] = {&width, &height};
    CK(launch(fzero, grid, block, args));  // :504
  }
  for (int si = 0; si < nSub; ++si) {
    int sel = picks[si];
    for (int p = sel; p < nP; p += nSub) {  // :509-531
      float s, c;
      trig(ang[p], &s, &c);
      RT(cudaMemcpy2DToArray(pre_a, 0, 0, pre + p * pix, prow, prow, height, cudaMemcpyHostToDevice));
      RT(cudaMemcpy2DToArray(post_a, 0, 0, post + p * pix, prow, prow, height, cudaMemcpyHostToDevice));
      void* args[] = {&bx, &by, &bz, &u0, &v0, &s, &c, &D, &D, &voxel, &isx, &isy, &isz, &width, &height, &geom};
      CK(launch(ffp, grid, block, args));
      RT(cudaDeviceSynchronize());
      RT(cudaMemcpy2DFromArray(pre + p * pix, prow, pre_a, 0, 0, prow, height, cudaMemcpyDeviceToHost));
      RT(cudaMemcpy2DFromArray(post + p * pix, prow, post_a, 0, 0, prow, height, cudaMemcpyDeviceToHost));
    }
    for (int p = sel; p < nP; p += nSub) {  // :533-546
      float s, c;
      trig(ang[p], &s, &c);
      RT(cudaMemcpy2DToArray(pre_a, 0, 0, pre + p * pix, prow, prow, height, cudaMemcpyHostToDevice));
      RT(cudaMemcpy2DToArray(post_a, 0, 0, post + p * pix, prow, prow, height, cudaMemcpyHostToDevice));
      void* args[] = {&v0, &s, &c, &D, &width, &height, &geom};
      CK(launch(fbp, grid, block, args));
      RT(cudaDeviceSynchronize());
    }
    void* args[] = {&width, &height};
    CK(launch(fupd, grid, block, args));  // :549
    RT(cudaDeviceSynchronize());
  }
  CK(array_to_vol(rec_a, mu, width, height));  // :564-570
  cudaDestroyTextureObject(pre_t);
  cudaDestroyTextureObject(post_t);
  cudaDestroyTextureObject(rec_t);
  cudaDestroySurfaceObject(pre_s);
  cudaDestroySurfaceObject(post_s);
  cudaDestroySurfaceObject(rec_s);
  cudaDestroySurfaceObject(num_s);
  cudaDestroySurfaceObject(den_s);
  cudaFreeArray(rec_a);
  cudaFreeArray(num_a);
  cudaFreeArray(den_a);
  cudaFreeArray(pre_a);
  cudaFreeArray(post_a);
  return 0;
}

/* CUDAmex_TVmin_3D gateway, CUDAmex_TVmin_3D.cu:162-246: 20 descent steps with
 * the reference's thrust reduction and SAXPY.  in/out [Nx,Ny,Nz]. */
int ref_tvmin3d(const float* in, int Nx_, int Ny_, int Nz_, float tv_const, float* out) {
  Timer tm;
  CUfunction f;
  CK(kernel(g_tv, "_Z16tvGradientKernelPfS_jjj", &f));
  unsigned nx = Nx_, ny = Ny_, nz = Nz_;
  size_t numel = (size_t)nx * ny * nz, bytes = numel * sizeof(float);
  float *output = nullptr, *input = nullptr;
  RT(cudaMalloc(&output, bytes));
  RT(cudaMemset(output, 0, bytes));  // border of the gradient: 0 (never written by the kernel)
  RT(cudaMalloc(&input, bytes));
  RT(cudaMemcpy(input, in, bytes, cudaMemcpyHostToDevice));
  dim3 block(32, 32, 1), grid(nblocks32(nx), nblocks32(ny), nz);  // :199-219
  for (int i = 0; i < 20; ++i) {
    void* args[] = {&output, &input, &nx, &ny, &nz};
    CK(launch(f, grid, block, args));
    thrust::device_ptr<float> o = thrust::device_pointer_cast(output);
    thrust::device_ptr<float> x = thrust::device_pointer_cast(input);
    float magnitude = std::sqrt(thrust::transform_reduce(o, o + numel, sq_f(), 0.0, thrust::plus<float>()));
    thrust::transform(o, o + numel, x, x, saxpy_f(-tv_const / magnitude));
  }
  RT(cudaMemcpy(out, input, bytes, cudaMemcpyDeviceToHost));
  cudaFree(output);
  cudaFree(input);
  return 0;
}

}  // extern "C"
