/*
 * ref_compat.h -- force-included (nvcc -include) when the reference's own
 * CUDA sources are compiled, unmodified, into sm_103a cubins for the oracle's
 * reference runs (oracle/ref_build.py).  TEST INFRASTRUCTURE ONLY.
 *
 * CUDA 12 removed texture and surface references (`texture<T,dim,mode>`,
 * `surface<void,dim>`, cudaBindTextureToArray, ...).  The reference files
 * projection_kernels/CUDAmex_FP.cu:40, CUDAmex_BP.cu:39,
 * CUDAmex_general3D_FP.cu:43 and iterative_reconstruction/CUDAmex_oscIter.cu:84-91
 * declare such references at file scope and fetch through them in device code.
 * This header turns each declaration into a __device__ variable that holds a
 * texture / surface OBJECT handle, and gives the legacy fetch functions
 * overloads that forward to the object forms.  The reference's kernels then
 * compile exactly as written; the host launcher (oracle/ref_launch.cu) creates
 * the objects with the address and filter modes the reference's host code sets
 * and writes the handles into those variables before each launch.
 *
 * Differences from the legacy references, both in code paths the reference
 * never exercises with in-range indices:
 *   - surface reads and writes use cudaBoundaryModeZero (an out-of-range
 *     access is dropped) instead of the legacy default cudaBoundaryModeTrap;
 *   - the host-side bind/unbind functions exist only so that the reference's
 *     mexFunction parses; the cubin build compiles device code only, and they
 *     are never called.
 */
#ifndef MEXCT_REF_COMPAT_H
#define MEXCT_REF_COMPAT_H

#include <cuda_runtime.h>
#include <cuda.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* The legacy texture reference became a plain aggregate: handle first, then the
   fields the reference's host code assigns (never read). */
template <class T, int DIM, cudaTextureReadMode MODE = cudaReadModeElementType>
struct mexct_ref_texture {
  cudaTextureObject_t obj;
  int normalized;
  cudaTextureFilterMode filterMode;
  cudaTextureAddressMode addressMode[3];
  cudaChannelFormatDesc channelDesc;
};

template <class T, int DIM>
struct mexct_ref_surface {
  cudaSurfaceObject_t obj;
};

template <class T, cudaTextureReadMode M>
__device__ __forceinline__ T tex3D(const mexct_ref_texture<T, 3, M>& t, float x, float y, float z) {
  return tex3D<T>(t.obj, x, y, z);
}

template <class T, cudaTextureReadMode M>
__device__ __forceinline__ T tex2D(const mexct_ref_texture<T, 2, M>& t, float x, float y) {
  return tex2D<T>(t.obj, x, y);
}

template <class V, class T>
__device__ __forceinline__ void surf3Dwrite(V val, const mexct_ref_surface<T, 3>& s, int x, int y, int z,
                                            cudaSurfaceBoundaryMode = cudaBoundaryModeZero) {
  surf3Dwrite<V>(val, s.obj, x, y, z, cudaBoundaryModeZero);
}

template <class V, class T>
__device__ __forceinline__ void surf3Dread(V* out, const mexct_ref_surface<T, 3>& s, int x, int y, int z,
                                           cudaSurfaceBoundaryMode = cudaBoundaryModeZero) {
  surf3Dread<V>(out, s.obj, x, y, z, cudaBoundaryModeZero);
}

template <class V, class T>
__device__ __forceinline__ void surf2Dwrite(V val, const mexct_ref_surface<T, 2>& s, int x, int y,
                                            cudaSurfaceBoundaryMode = cudaBoundaryModeZero) {
  surf2Dwrite<V>(val, s.obj, x, y, cudaBoundaryModeZero);
}

template <class V, class T>
__device__ __forceinline__ void surf2Dread(V* out, const mexct_ref_surface<T, 2>& s, int x, int y,
                                           cudaSurfaceBoundaryMode = cudaBoundaryModeZero) {
  surf2Dread<V>(out, s.obj, x, y, cudaBoundaryModeZero);
}

/* Host-side names of the removed API, for parsing only (device-only build). */
template <class T, int D, cudaTextureReadMode M>
static inline cudaError_t cudaBindTextureToArray(const mexct_ref_texture<T, D, M>&, const cudaArray*,
                                                 const cudaChannelFormatDesc&) {
  return cudaErrorNotSupported;
}
template <class T, int D, cudaTextureReadMode M>
static inline cudaError_t cudaUnbindTexture(const mexct_ref_texture<T, D, M>&) {
  return cudaErrorNotSupported;
}
template <class T, int D>
static inline cudaError_t cudaBindSurfaceToArray(const mexct_ref_surface<T, D>&, const cudaArray*) {
  return cudaErrorNotSupported;
}
template <class T, int D>
static inline cudaError_t cudaBindSurfaceToArray(const mexct_ref_surface<T, D>&, const cudaArray*,
                                                 const cudaChannelFormatDesc&) {
  return cudaErrorNotSupported;
}

/* Removed runtime entry points the reference's host code names. */
#define cudaThreadSynchronize cudaDeviceSynchronize

/* File-scope `texture<...> name;` / `surface<...> name;` become __device__
   variables that hold object handles (defined after every system header). */
#define texture __device__ mexct_ref_texture
#define surface __device__ mexct_ref_surface

#endif
