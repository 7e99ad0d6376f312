// geom.cuh -- device-side geometry and sampling shared by the mexct kernels.
//
// Ray set-up (end points, clip to the volume box, entry point, per-step
// vector, sample count) is evaluated in binary32 with explicitly rounded
// operations (__fadd_rn/__fmul_rn/__fmaf_rn/...), so that the compiler can
// neither contract nor reorder it, and takes exactly the discrete decisions
// the reference takes (CUDAmex_FP.cu:82-137 and its copies in the other
// operators).  The reference is built with nvcc -O3 and fused multiply-add on
// (compile.m:25), so its multiply-adds here are fmas; which product of each
// sum is fused was pinned against outputs of the reference's own kernels run
// on a GB300: a general3D BP's voxel indices and weights reproduce to 1e-7
// only with these fmas, and the texture FP variant, which samples as the
// reference does, reproduces the reference's FP output bit for bit.
// Sampling and accumulation are plain FP32 with FMAs: they are continuous in
// the inputs.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mexct {

constexpr int kMaxViews = 2048;  // views per launch (trig table in params)

struct Trig {
  float s, c;
};

// ---- storage types -------------------------------------------------------
__device__ __forceinline__ float ldf(const float* p) { return __ldg(p); }
__device__ __forceinline__ float ldf(const __half* p) {
  return __half2float(__ldg(p));
}
__device__ __forceinline__ float ldf(const __nv_bfloat16* p) {
  return __bfloat162float(__ldg(p));
}
__device__ __forceinline__ float ldp(const float* p) { return *p; }
__device__ __forceinline__ float ldp(const __half* p) {
  return __half2float(*p);
}
__device__ __forceinline__ float ldp(const __nv_bfloat16* p) {
  return __bfloat162float(*p);
}
__device__ __forceinline__ void stf(float* p, float v) { *p = v; }
__device__ __forceinline__ void stf(__half* p, float v) {
  *p = __float2half_rn(v);
}
__device__ __forceinline__ void stf(__nv_bfloat16* p, float v) {
  *p = __float2bfloat16_rn(v);
}

// ---- binary32 ray set-up ---------------------------------------------------
struct Ray {
  float cx, cy, cz;  // clipped entry point
  float dx, dy, dz;  // per-step displacement
  int n;             // samples of while(travelled < distance)
};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// One axis of the slab clip: alpha of the planes b and -b, or NaN when the
// ray is parallel to them (|d| < 1e-5 compared in double, as written).
__device__ __forceinline__ void slab(float s, float e, float b, float& lo,
                                     float& hi) {
  const float d = fsub(e, s);
  float a1, a2;
  if ((double)fabsf(d) >= 1e-5) {
    a1 = fdiv(fsub(b, s), d);
    a2 = fdiv(fsub(-b, s), d);
  } else {
    a1 = __int_as_float(0x7fffffff);
    a2 = a1;
  }
  lo = fminf(a1, a2);
  hi = fmaxf(a1, a2);
}

// CUDAmex_FP.cu:82-137.
__device__ __forceinline__ Ray clip_ray(float sx, float sy, float sz, float ex,
                                        float ey, float ez, float bx, float by,
                                        float bz, float step) {
  float xlo, xhi, ylo, yhi, zlo, zhi;
  slab(sx, ex, bx, xlo, xhi);
  slab(sy, ey, by, ylo, yhi);
  slab(sz, ez, bz, zlo, zhi);
  const float amin = fmaxf(0.f, fmaxf(xlo, fmaxf(ylo, zlo)));
  const float amax = fminf(1.f, fminf(xhi, fminf(yhi, zhi)));
  const float ddx = fsub(ex, sx), ddy = fsub(ey, sy), ddz = fsub(ez, sz);
  Ray r;
  r.cx = ffma(amin, ddx, sx);
  r.cy = ffma(amin, ddy, sy);
  r.cz = ffma(amin, ddz, sz);
  const float px = ffma(amax, ddx, sx);
  const float py = ffma(amax, ddy, sy);
  const float pz = ffma(amax, ddz, sz);
  const float qx = fsub(px, r.cx), qy = fsub(py, r.cy), qz = fsub(pz, r.cz);
  const float dist = __fsqrt_rn(ffma(qz, qz, ffma(qx, qx, fmul(qy, qy))));
  r.dx = fmul(fdiv(qx, dist), step);
  r.dy = fmul(fdiv(qy, dist), step);
  r.dz = fmul(fdiv(qz, dist), step);
  // Number of k >= 0 with k*step < dist (dist/step is exact for step 0.5 and
  // 1).  NaN, non-positive or infinite distance: no sample.
  if (!(dist > 0.f) || isinf(dist)) {
    r.n = 0;
  } else {
    r.n = (int)ceilf(fdiv(dist, step));
  }
  return r;
}

// Whether the segment s -> e meets the volume box [b, -b] per axis (no
// counterpart in the reference, whose rays all pass through the box: each
// crosses the isocentre plane at a point 0.5 voxel or more inside it).  The
// clip above leaves an axis the ray runs parallel to open and marches a ray
// that misses the box between two points outside it; the decoupled detector
// drops such rays instead.  The per-axis alphas are the clip's own.
__device__ __forceinline__ bool hits_box(const float* s, const float* e, float bx, float by,
                                         float bz) {
  const float b[3] = {bx, by, bz};
  float amin = 0.f, amax = 1.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float lo, hi;
    slab(s[i], e[i], b[i], lo, hi);
    if (lo != lo) {  // parallel to the axis' planes: inside or not at all
      if (fabsf(s[i]) > -b[i]) return false;
    } else {
      amin = fmaxf(amin, lo);
      amax = fminf(amax, hi);
    }
  }
  return amin <= amax;
}

// Standard-geometry ray end points (CUDAmex_FP.cu:64-77 par, :162-175 cone,
// :259-272 fan; CUDAmex_oscIter.cu:152-187).  Detector generalisation (no
// counterpart in the reference): pixel pitch du, dv at the isocentre and a
// sub-pixel offset ou, ov; du = dv = 1, ou = ov = 0 give the reference's
// binary32 operations exactly (adding 0 and multiplying by 1 are exact).
// Fused as the reference's build fuses them: in the parallel geometry u*sinB
// and u*cosB appear in both end points, are rounded once and shared, and the
// other product of each sum is fused; in fan and cone u appears only in the
// detector end point, fused as fma(-RD, cosB, -(u*sinB)) and
// fma(u, cosB, -RD*sinB).
template <int GEOM>
__device__ __forceinline__ void std_ray(int ix, int iy, float u0, float v0,
                                        float sb, float cb, float SR, float RD,
                                        float* s, float* e, float du = 1.0f,
                                        float dv = 1.0f, float ou = 0.0f,
                                        float ov = 0.0f) {
  float u, v;
  const float du0 = fmul(fsub(fadd((float)ix, ou), u0), du);
  const float dv0 = fmul(fsub(fadd((float)iy, ov), v0), dv);
  if (GEOM == 0) {
    u = du0;
    v = dv0;
    const float usb = fmul(u, sb), ucb = fmul(u, cb);
    s[0] = ffma(SR, cb, -usb);
    s[1] = ffma(SR, sb, ucb);
    s[2] = v;
    e[0] = ffma(-RD, cb, -usb);
    e[1] = ffma(-RD, sb, ucb);
    e[2] = v;
    return;
  } else if (GEOM == 1) {
    u = fdiv(fmul(du0, fadd(SR, RD)), SR);
    v = dv0;
    s[0] = fmul(SR, cb);
    s[1] = fmul(SR, sb);
    s[2] = v;
  } else {
    u = fdiv(fmul(du0, fadd(SR, RD)), SR);
    v = fdiv(fmul(dv0, fadd(SR, RD)), SR);
    s[0] = fmul(SR, cb);
    s[1] = fmul(SR, sb);
    s[2] = 0.0f;
  }
  e[0] = ffma(-RD, cb, -fmul(u, sb));
  e[1] = ffma(u, cb, fmul(-RD, sb));
  e[2] = v;
}

// general3D ray end points rotated by the view angle
// (CUDAmex_general3D_FP.cu:71-77, CUDAmex_general3D_BP.cu:73-79), fused as the
// reference's build fuses them: x' = fma(x, cosB, -(y*sinB)),
// y' = fma(y, cosB, x*sinB).
__device__ __forceinline__ void g3d_ray(const float* pts, long long pix,
                                        long long P, float sb, float cb,
                                        float* s, float* e) {
  const float x1 = __ldg(pts + pix), y1 = __ldg(pts + pix + P),
              z1 = __ldg(pts + pix + 2 * P);
  const float x2 = __ldg(pts + pix + 3 * P), y2 = __ldg(pts + pix + 4 * P),
              z2 = __ldg(pts + pix + 5 * P);
  s[0] = ffma(x1, cb, -fmul(y1, sb));
  s[1] = ffma(y1, cb, fmul(x1, sb));
  s[2] = z1;
  e[0] = ffma(x2, cb, -fmul(y2, sb));
  e[1] = ffma(y2, cb, fmul(x2, sb));
  e[2] = z2;
}

// ---- FP32 texture-equivalent sampling -----------------------------------
// Unnormalised coordinates, texel centre at i + 0.5, linear filter with exact
// FP32 weights.  Clamp: indices clamped to the edge.  Border: 0 outside.
struct Tap {
  int i0, i1;   // indices to load (always in range)
  float w0, w1; // weights (border: zero for out-of-range taps)
};

template <bool BORDER>
__device__ __forceinline__ Tap tap(float c, int n) {
  // Bound the coordinate so floor() fits an int; the result is unchanged.
  c = fminf(fmaxf(c, -4.0f), (float)n + 4.0f) - 0.5f;
  const float f = floorf(c);
  const float a = c - f;
  const int i = (int)f;
  Tap t;
  t.i0 = min(max(i, 0), n - 1);
  t.i1 = min(max(i + 1, 0), n - 1);
  t.w0 = 1.0f - a;
  t.w1 = a;
  if (BORDER) {
    if (i < 0 || i >= n) t.w0 = 0.f;
    if (i + 1 < 0 || i + 1 >= n) t.w1 = 0.f;
  }
  return t;
}

// Trilinear sample of a volume stored with a fast axis (nf), a slow axis
// (ns) and z (nz): index f + nf*(s + ns*z).
template <bool BORDER, typename T>
__device__ __forceinline__ float tri(const T* __restrict__ v, int nf, int ns,
                                     int nz, float cf, float cs, float cz) {
  const Tap a = tap<BORDER>(cf, nf);
  const Tap b = tap<BORDER>(cs, ns);
  const Tap g = tap<BORDER>(cz, nz);
  const size_t sz = (size_t)nf * ns;
  const T* p00 = v + (size_t)g.i0 * sz + (size_t)b.i0 * nf;
  const T* p01 = v + (size_t)g.i0 * sz + (size_t)b.i1 * nf;
  const T* p10 = v + (size_t)g.i1 * sz + (size_t)b.i0 * nf;
  const T* p11 = v + (size_t)g.i1 * sz + (size_t)b.i1 * nf;
  const float r00 = a.w0 * ldf(p00 + a.i0) + a.w1 * ldf(p00 + a.i1);
  const float r01 = a.w0 * ldf(p01 + a.i0) + a.w1 * ldf(p01 + a.i1);
  const float r10 = a.w0 * ldf(p10 + a.i0) + a.w1 * ldf(p10 + a.i1);
  const float r11 = a.w0 * ldf(p11 + a.i0) + a.w1 * ldf(p11 + a.i1);
  return g.w0 * (b.w0 * r00 + b.w1 * r01) + g.w1 * (b.w0 * r10 + b.w1 * r11);
}

// Circle of reconstruction with the reference's unsigned arithmetic
// (CUDAmex_BP.cu:73-77).
__device__ __forceinline__ bool in_circle(int ix, int iy, uint32_t hw) {
  const uint32_t dx = (uint32_t)ix - hw, dy = (uint32_t)iy - hw;
  return (uint32_t)(dx * dx + dy * dy) < (uint32_t)(hw * hw);
}

}  // namespace mexct
