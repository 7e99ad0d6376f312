// k_proj.cu -- ray-per-thread forward projectors (general3D FP, the
// MEXCT_FP_RAY and MEXCT_FP_TEXTURE variants), voxel-driven backprojectors
// (standard BP, OSC dual BP + update, batched BP) and the general3D scatter
// backprojector for sm_103a.  The standard and OSC forward projections run
// in the slab kernel of k_slab.cu.
//
// Ray-per-thread FP (CUDAmex_FP.cu:56-346, CUDAmex_general3D_FP.cu:59-150)
//   One thread per detector pixel; a warp owns 32 consecutive pixels of one
//   detector row, a CTA a 32x8 pixel tile of one view.  blockIdx.x is the
//   view, so CTAs that are resident together march the same detector tile at
//   neighbouring angles through the same part of the volume (L2 reuse).
//   Samples are explicit FP32 trilinear fetches (the texture unit's 8-bit
//   filter weights would miss a 1e-5 tolerance).  The volume is kept in two
//   layouts, x-fastest and y-fastest: a view whose rays run mostly along x
//   reads the y-fastest copy, so the 32 lanes of a warp (neighbouring u, i.e.
//   neighbouring y) touch consecutive addresses.
//
// Backprojection (CUDAmex_BP.cu:44-221)
//   One thread per (x, y) voxel column and a chunk of ZC voxels along z held
//   in registers across all views (or a block of views), each warp on an 8x4
//   patch of columns; per-view geometry comes from the kernel parameter block
//   (constant bank); the projection taps come through L1 from the views laid
//   out once as quads (a texel's 2x2 bilinear footprint in 16 bytes); the
//   volume is written once.
#include <algorithm>
#include <type_traits>
#include <cstdio>

#include "kernels.h"

namespace mexct {

template <typename T>
struct DT;
template <>
struct DT<float> {
  static constexpr int id = kF32;
};
template <>
struct DT<__half> {
  static constexpr int id = kF16;
};
template <>
struct DT<__nv_bfloat16> {
  static constexpr int id = kBF16;
};

// ---------------------------------------------------------------------------
// xy transpose (x-fastest <-> y-fastest), 32x32 tiles per z slice.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) transpose_xy_kernel(
    const T* __restrict__ src, T* __restrict__ dst, int W) {
  __shared__ T tile[32][33];
  const size_t zoff = (size_t)blockIdx.z * W * W;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int x = x0 + threadIdx.x, y = y0 + j;
    if (x < W && y < W) tile[j][threadIdx.x] = src[zoff + (size_t)y * W + x];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int y = y0 + threadIdx.x, x = x0 + j;
    if (x < W && y < W) dst[zoff + (size_t)x * W + y] = tile[threadIdx.x][j];
  }
}

cudaError_t launch_transpose_xy(const void* src, void* dst, int W, int H,
                                int dtype, cudaStream_t st) {
  dim3 blk(32, 8), grd((W + 31) / 32, (W + 31) / 32, H);
  switch (dtype) {
    case kF32:
      transpose_xy_kernel<float>
          <<<grd, blk, 0, st>>>((const float*)src, (float*)dst, W);
      break;
    case kF16:
      transpose_xy_kernel<__half>
          <<<grd, blk, 0, st>>>((const __half*)src, (__half*)dst, W);
      break;
    default:
      transpose_xy_kernel<__nv_bfloat16><<<grd, blk, 0, st>>>(
          (const __nv_bfloat16*)src, (__nv_bfloat16*)dst, W);
      break;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Ray march: sum of n trilinear samples at c + k*d (texture coordinates).
// ---------------------------------------------------------------------------
template <bool BORDER, typename T>
__device__ __forceinline__ float march(const T* __restrict__ v, int nf,
                                       int ns, int nz, float cf, float cs,
                                       float cz, float df, float ds, float dz,
                                       int n) {
  float a0 = 0.f, a1 = 0.f;
  int k = 0;
  for (; k + 1 < n; k += 2) {
    const float k0 = (float)k, k1 = (float)(k + 1);
    a0 += tri<BORDER>(v, nf, ns, nz, fmaf(k0, df, cf), fmaf(k0, ds, cs),
                      fmaf(k0, dz, cz));
    a1 += tri<BORDER>(v, nf, ns, nz, fmaf(k1, df, cf), fmaf(k1, ds, cs),
                      fmaf(k1, dz, cz));
  }
  if (k < n) {
    const float k0 = (float)k;
    a0 += tri<BORDER>(v, nf, ns, nz, fmaf(k0, df, cf), fmaf(k0, ds, cs),
                      fmaf(k0, dz, cz));
  }
  return a0 + a1;
}

// Build the binary32 ray of detector pixel (ix, iy) of launch view `view`.
// GEOM 0/1/2: standard geometries; GEOM 3: general3D points.
template <int GEOM>
__device__ __forceinline__ Ray make_ray(const RayArgs& A, int view, int ix,
                                        int iy, const float* __restrict__ pts) {
  const Trig t = A.trig[view];
  float s[3], e[3];
  if (GEOM < 3) {
    std_ray<GEOM>(ix, iy, A.u0, A.v0, t.s, t.c, A.SR, A.RD, s, e, A.du, A.dv, A.ou, A.ov);
  } else {
    const long long pix = (long long)iy * A.det_w + ix;
    const float* p =
        pts + (A.pts_per_view ? (size_t)6 * A.P * (A.view0 + view * A.vstride) : 0);
    g3d_ray(p, pix, A.P, t.s, t.c, s, e);
  }
  return clip_ray(s[0], s[1], s[2], e[0], e[1], e[2], A.bx, A.by, A.bz,
                  A.step);
}

// Warp-uniform choice of the volume layout: the y-fastest copy when the rays
// of this warp run mostly along x.
template <int GEOM>
__device__ __forceinline__ bool pick_y_layout(const RayArgs& A, int view,
                                              const Ray& r, bool valid,
                                              bool have_y) {
  if (!have_y) return false;
  if (GEOM < 3) {
    const Trig t = A.trig[view];
    return fabsf(t.c) >= fabsf(t.s);
  }
  const bool live = valid && r.n > 0;
  const unsigned all = __ballot_sync(0xffffffffu, live);
  const unsigned xs =
      __ballot_sync(0xffffffffu, live && fabsf(r.dx) >= fabsf(r.dy));
  return all != 0u && 2 * __popc(xs) >= __popc(all);
}

template <int GEOM, bool BORDER, typename TV, typename TO>
__global__ void __launch_bounds__(256) fp_kernel(
    const __grid_constant__ RayArgs A, const TV* __restrict__ vx,
    const TV* __restrict__ vy, const float* __restrict__ pts,
    TO* __restrict__ out) {
  const int view = blockIdx.x;
  const int tiles_u = (A.det_w + 31) >> 5;
  const int ix = (blockIdx.y % tiles_u) * 32 + threadIdx.x;
  const int iy = (blockIdx.y / tiles_u) * blockDim.y + threadIdx.y;
  const bool valid = ix < A.det_w && iy < A.det_h;
  const Ray r = make_ray<GEOM>(A, view, min(ix, A.det_w - 1),
                               min(iy, A.det_h - 1), pts);
  const bool use_y = pick_y_layout<GEOM>(A, view, r, valid, vy != nullptr);
  if (!valid) return;
  const float cx = r.cx - A.bx, cy = r.cy - A.by, cz = r.cz - A.bz;
  float acc;
  if (use_y)
    acc = march<BORDER>(vy, A.S, A.S, A.Z, cy, cx, cz, r.dy, r.dx, r.dz, r.n);
  else
    acc = march<BORDER>(vx, A.S, A.S, A.Z, cx, cy, cz, r.dx, r.dy, r.dz, r.n);
  stf(out + (size_t)(A.view0 + view * A.vstride) * A.P + (size_t)iy * A.det_w + ix,
      acc * A.step);
}

template <int GEOM, bool BORDER, typename TV, typename TO>
static void fp_go(const RayArgs& a, const void* vx, const void* vy,
                  const float* pts, void* out, cudaStream_t st) {
  const int tiles = ((a.det_w + 31) / 32) * ((a.det_h + 7) / 8);
  dim3 blk(32, 8), grd(a.nviews, tiles);
  fp_kernel<GEOM, BORDER, TV, TO><<<grd, blk, 0, st>>>(
      a, (const TV*)vx, (const TV*)vy, pts, (TO*)out);
}

template <int GEOM, bool BORDER>
static cudaError_t fp_types(const RayArgs& a, const void* vx, const void* vy,
                            int vt, const float* pts, void* out, int ot,
                            cudaStream_t st) {
  if (vt == kF32 && ot == kF32)
    fp_go<GEOM, BORDER, float, float>(a, vx, vy, pts, out, st);
  else if (vt == kF16 && ot == kF16)
    fp_go<GEOM, BORDER, __half, __half>(a, vx, vy, pts, out, st);
  else if (vt == kF16 && ot == kF32)
    fp_go<GEOM, BORDER, __half, float>(a, vx, vy, pts, out, st);
  else if (vt == kBF16 && ot == kBF16)
    fp_go<GEOM, BORDER, __nv_bfloat16, __nv_bfloat16>(a, vx, vy, pts, out,
                                                       st);
  else if (vt == kBF16 && ot == kF32)
    fp_go<GEOM, BORDER, __nv_bfloat16, float>(a, vx, vy, pts, out, st);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_fp(int geom, bool border, const RayArgs& a,
                      const void* vx, const void* vy, int vt,
                      const float* pts, void* out, int ot, cudaStream_t st) {
  if (a.nviews <= 0) return cudaSuccess;
  // the ray-per-thread form serves MEXCT_FP_RAY for the standard geometries
  // (clamp addressing); general3D and the OSC FP use the slab kernel
  if (border) return cudaErrorInvalidValue;
  switch (geom) {
    case 0: return fp_types<0, false>(a, vx, vy, vt, pts, out, ot, st);
    case 1: return fp_types<1, false>(a, vx, vy, vt, pts, out, ot, st);
    case 2: return fp_types<2, false>(a, vx, vy, vt, pts, out, ot, st);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// Hardware-texture FP variant: the reference's own sampling path, reproduced
// operation for operation (CUDAmex_FP.cu:137-148, :235-246, :332-343): one
// thread per ray, the texture unit's trilinear filter (8-bit weights), the
// sample point advanced by `currentpoint += stepsize` in binary32, the
// texture coordinate `currentpoint - b` in binary32, and one FP32 running
// sum `dval += tex * stepsize`.  With the ray set-up of geom.cuh this gives
// the reference's output bit for bit; it sits ~1e-4 from the FP64 oracle
// (8-bit weights, binary32 stepping), where the slab kernel sits at 1e-7.
// ---------------------------------------------------------------------------
template <int GEOM>
__global__ void __launch_bounds__(256) fp_tex_kernel(
    const __grid_constant__ RayArgs A, cudaTextureObject_t tex,
    float* __restrict__ out) {
  const int view = blockIdx.x;
  const int tiles_u = (A.det_w + 31) >> 5;
  const int ix = (blockIdx.y % tiles_u) * 32 + threadIdx.x;
  const int iy = (blockIdx.y / tiles_u) * blockDim.y + threadIdx.y;
  if (ix >= A.det_w || iy >= A.det_h) return;
  const Ray r = make_ray<GEOM>(A, view, ix, iy, nullptr);
  float cx = r.cx, cy = r.cy, cz = r.cz, acc = 0.f;
#pragma unroll 4
  for (int k = 0; k < r.n; ++k) {
    const float t = tex3D<float>(tex, fsub(cx, A.bx), fsub(cy, A.by), fsub(cz, A.bz));
    acc = ffma(t, A.step, acc);
    cx = fadd(cx, r.dx);
    cy = fadd(cy, r.dy);
    cz = fadd(cz, r.dz);
  }
  out[(size_t)(A.view0 + view * A.vstride) * A.P + (size_t)iy * A.det_w + ix] = acc;
}

cudaError_t launch_fp_tex(int geom, const RayArgs& a, cudaTextureObject_t tex,
                          float* out, cudaStream_t st) {
  if (a.nviews <= 0) return cudaSuccess;
  const int tiles = ((a.det_w + 31) / 32) * ((a.det_h + 7) / 8);
  dim3 blk(32, 8), grd(a.nviews, tiles);
  switch (geom) {
    case 0: fp_tex_kernel<0><<<grd, blk, 0, st>>>(a, tex, out); break;
    case 1: fp_tex_kernel<1><<<grd, blk, 0, st>>>(a, tex, out); break;
    case 2: fp_tex_kernel<2><<<grd, blk, 0, st>>>(a, tex, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Voxel-driven BP.  Per view: s, t and U of the column (CUDAmex_BP.cu:79-94,
// :137-154, :199-212), then the projection column is sampled along z.
// ---------------------------------------------------------------------------
template <int GEOM>
struct ColGeom {
  float w, py, pz0, dpz;
};

// Projection coordinates of column (x, y) for one view (CUDAmex_BP.cu:
// 88-190).  Detector generalisation: u centre hwd + 1, v centre v0d,
// reciprocal pitches inv_du, inv_dv; the defaults (hwd = hw, v0d = v0,
// inv_du = inv_dv = 1) are the reference's operations exactly.
template <int GEOM>
__device__ __forceinline__ ColGeom<GEOM> col_geom(float x, float y, Trig t,
                                                  float SR, float v0,
                                                  float hwd, float v0d, float inv_du,
                                                  float inv_dv) {
  ColGeom<GEOM> g;
  const float s = fmaf(x, t.c, y * t.s);
  const float tt = fmaf(-x, t.s, y * t.c);
  if (GEOM == 0) {
    g.w = 1.f;
    g.py = fmaf(tt, inv_du, hwd) + 1.f;
    g.pz0 = fmaf(-v0, inv_dv, v0d) + 0.5f;
    g.dpz = inv_dv;
  } else {
    const float U = SR / (SR - s);
    g.w = U * U;
    g.py = fmaf(tt, U * inv_du, hwd) + 1.f;
    if (GEOM == 1) {
      g.pz0 = fmaf(-v0, inv_dv, v0d) + 0.5f;
      g.dpz = inv_dv;
    } else {
      const float Uv = U * inv_dv;
      g.pz0 = fmaf(-v0, Uv, v0d) + 0.5f;
      g.dpz = Uv;
    }
  }
  return g;
}

// Sample one projection along a voxel column: acc[j] += w * B(py, pz(z0+j)).
// Par/fan columns hit texel rows exactly (pz = iz + 0.5): one row, no v
// interpolation.
template <int GEOM, bool BORDER, int ZC, typename TS>
__device__ __forceinline__ void bp_column(const TS* __restrict__ p, int W,
                                          int H, int z0,
                                          const ColGeom<GEOM>& g,
                                          float* acc) {
  const Tap tu = tap<BORDER>(g.py, W);
  const float w0 = g.w * tu.w0, w1 = g.w * tu.w1;
  if (GEOM < 2) {
#pragma unroll
    for (int j = 0; j < ZC; ++j) {
      const int row = min(z0 + j, H - 1);
      const TS* r = p + (size_t)row * W;
      acc[j] = fmaf(w0, ldf(r + tu.i0), fmaf(w1, ldf(r + tu.i1), acc[j]));
    }
  } else {
#pragma unroll
    for (int j = 0; j < ZC; ++j) {
      const float pz = fmaf((float)(z0 + j), g.dpz, g.pz0);
      const Tap tv = tap<BORDER>(pz, H);
      const TS* r0 = p + (size_t)tv.i0 * W;
      const TS* r1 = p + (size_t)tv.i1 * W;
      const float a = fmaf(w0, ldf(r0 + tu.i0), w1 * ldf(r0 + tu.i1));
      const float b = fmaf(w0, ldf(r1 + tu.i0), w1 * ldf(r1 + tu.i1));
      acc[j] = fmaf(tv.w0, a, fmaf(tv.w1, b, acc[j]));
    }
  }
}


// ---------------------------------------------------------------------------
// Backprojection from padded views.  Each view is laid out once in [H+4][W+4]
// texels with two extra rows and columns on every side holding the edge
// values (clamp addressing; the OSC residual views keep a zero frame, border
// addressing).  A tap index then only needs clamping into [-2, n] -- both
// taps of an index outside the image read frame values, which is what the
// clamp / border texture fetch returns -- instead of clamping both taps of
// both axes into the image.
// ---------------------------------------------------------------------------
size_t sino_pad_elems(int W, int H, int nviews) {
  return (size_t)sino_pad_pitch(W) * (H + 2 * kSinoPad) * nviews;
}

// Quad layout of the clamp-padded views (every BP): padded texel (r, c) of
// view v -> {P(r,c), P(r+1,c), P(r,c+1), P(r+1,c+1)} (column c's two rows,
// then column c+1's) with P(r, c) = the view's pixel (clamp(c - kSinoPad),
// clamp(r - kSinoPad)) (the clamp texture fetch's frame).  FP32 views: a float4 per
// texel; FP16 / BF16 views: the four 16-bit values in a uint2 (x: P(r,c) |
// P(r+1,c) << 16, y: column c+1), converted to FP32 exactly as a 16-bit
// load is.
template <typename S> struct QuadT;
template <> struct QuadT<float> {
  using T = float4;
  static __device__ __forceinline__ T make(float a, float b, float c, float d) {
    return make_float4(a, b, c, d);
  }
  static __device__ __forceinline__ float4 get(const T* p) { return __ldg(p); }
};
// 16-bit values as bits (make) and back to float in registers (get; the
// conversions are exact for both types)
__device__ __forceinline__ uint32_t bits16(__half h) { return __half_as_ushort(h); }
__device__ __forceinline__ uint32_t bits16(__nv_bfloat16 h) { return __bfloat16_as_ushort(h); }
// Two packed 16-bit values (low half first) to FP32 in one paired conversion
// (exact, as the scalar conversions are).
template <typename H16> __device__ __forceinline__ float2 pair_from_bits16(uint32_t u);
template <> __device__ __forceinline__ float2 pair_from_bits16<__half>(uint32_t u) {
  return __half22float2(*reinterpret_cast<const __half2*>(&u));
}
template <> __device__ __forceinline__ float2 pair_from_bits16<__nv_bfloat16>(uint32_t u) {
  return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u));
}
template <typename H16> struct QuadT16 {
  using T = uint2;
  static __device__ __forceinline__ T make(H16 a, H16 b, H16 c, H16 d) {
    return make_uint2(bits16(a) | (bits16(b) << 16), bits16(c) | (bits16(d) << 16));
  }
  static __device__ __forceinline__ float4 get(const T* p) {
    const uint2 q = __ldg(p);
    const float2 lo = pair_from_bits16<H16>(q.x), hi = pair_from_bits16<H16>(q.y);
    return make_float4(lo.x, lo.y, hi.x, hi.y);
  }
};
template <> struct QuadT<__half> : QuadT16<__half> {};
template <> struct QuadT<__nv_bfloat16> : QuadT16<__nv_bfloat16> {};

// Marker type of the BP kernels' view pointer: views in the quad layout of
// storage type S.
template <typename S> struct QuadLayout {};
template <typename T> struct IsQuad : std::false_type {};
template <typename S> struct IsQuad<QuadLayout<S>> : std::true_type { using Storage = S; };

template <typename S>
__global__ void __launch_bounds__(256) pad_sino_quad_kernel(const S* __restrict__ in, int W,
                                                            int H,
                                                            typename QuadT<S>::T* __restrict__ out,
                                                            int Wp) {
  const int c = blockIdx.x * 32 + threadIdx.x;
  const int r = blockIdx.y * 8 + threadIdx.y;
  const int v = blockIdx.z;
  const int Hp = H + 2 * kSinoPad;
  if (c >= Wp || r >= Hp) return;
  const S* view = in + (size_t)v * W * H;
  const int x0 = min(max(c - kSinoPad, 0), W - 1), x1 = min(max(c + 1 - kSinoPad, 0), W - 1);
  const int y0 = min(max(r - kSinoPad, 0), H - 1), y1 = min(max(r + 1 - kSinoPad, 0), H - 1);
  out[((size_t)v * Hp + r) * Wp + c] =
      QuadT<S>::make(view[(size_t)y0 * W + x0], view[(size_t)y1 * W + x0],
                     view[(size_t)y0 * W + x1], view[(size_t)y1 * W + x1]);
}

cudaError_t launch_pad_sino_quad(const void* in, int stype, int W, int H, int nviews, void* out,
                                 cudaStream_t st) {
  if (nviews <= 0) return cudaSuccess;
  const int Wp = sino_pad_pitch(W);
  dim3 blk(32, 8), grd((Wp + 31) / 32, (H + 2 * kSinoPad + 7) / 8, nviews);
#define QPAD(S)                                                                           \
  pad_sino_quad_kernel<S><<<grd, blk, 0, st>>>(static_cast<const S*>(in), W, H,           \
                                               static_cast<typename QuadT<S>::T*>(out), Wp)
  if (stype == kF32) QPAD(float);
  else if (stype == kF16) QPAD(__half);
  else if (stype == kBF16) QPAD(__nv_bfloat16);
  else return cudaErrorInvalidValue;
#undef QPAD
  return cudaGetLastError();
}

// A voxel column's samples of one padded view: acc[j] += w * B(py, pz_j) for
// the column's z voxels z0 + j (CUDAmex_BP.cu:88-190).  g.py / g.pz0 are
// texture coordinates (texel centres at i + 0.5); B is bilinear in FP32 with
// the taps of the padded view P: u tap iu = floor(py - 0.5) (coordinate
// bounded so floor fits an int, index clamped into the frame), w0 = w (1 -
// au), w1 = w au; per voxel a = fma(w0, P(r, iu), w1 P(r, iu+1)), b the same
// on row r + 1, acc = fma(1 - az, a, fma(az, b, acc)).  W x H is the detector;
// roff: the view holds detector rows roff .. roff + H - 1 (a band of a
// taller detector, launch_bp_sub), taps are computed in whole-detector rows.
//
// Cone column over a quad-layout view (launch_pad_sino_quad): texel (r, c)
// holds the bilinear footprint {P(r,c), P(r+1,c), P(r,c+1), P(r+1,c+1)} of
// the padded view P, so each voxel's four taps are one 16-byte load whose
// halves (columns c and c+1) feed the packed u lerps of both rows.  pz is
// interpolated: r = floor(pz - 0.5), az its fraction.
template <int ZC, typename S = float, int GEOM = 2>
__device__ __forceinline__ void bp_column_quad(const typename QuadT<S>::T* __restrict__ p, int W,
                                               int H, int Wp, int z0, const ColGeom<GEOM>& g,
                                               float* acc, int roff = 0) {
  const float cu = fminf(fmaxf(g.py, -4.0f), (float)W + 4.0f) - 0.5f;
  const float fu = floorf(cu);
  const float au = cu - fu;
  const int iu = min(max((int)fu, -kSinoPad), W) + kSinoPad;
  const float w0 = g.w * (1.0f - au), w1 = g.w * au;
  const typename QuadT<S>::T* col = p + iu;
  static_assert(ZC % 2 == 0, "ZC must be even");
  const float2 w02 = make_float2(w0, w0), w12 = make_float2(w1, w1);
  const float pz0 = g.pz0 - 0.5f;
  const float2 dpz2 = make_float2(g.dpz, g.dpz), pz02 = make_float2(pz0, pz0);
#pragma unroll
  for (int j = 0; j < ZC; j += 2) {
    const float2 zz = make_float2((float)(z0 + j), (float)(z0 + j + 1));
    const float2 cz = __ffma2_rn(zz, dpz2, pz02);
    const float2 fz = make_float2(floorf(cz.x), floorf(cz.y));
    const float2 az = __fadd2_rn(cz, make_float2(-fz.x, -fz.y));
    const int i0 = min(max(__float2int_rz(fz.x) - roff, -kSinoPad), H) + kSinoPad;
    const int i1 = min(max(__float2int_rz(fz.y) - roff, -kSinoPad), H) + kSinoPad;
    const float4 q0 = QuadT<S>::get(col + (size_t)i0 * Wp);
    const float4 q1 = QuadT<S>::get(col + (size_t)i1 * Wp);
    // (a, b) of one voxel: the u lerps of rows r and r+1, one packed pair of
    // operations on the quad's two halves (columns c and c+1)
    const float2 ab0 = __ffma2_rn(w02, make_float2(q0.x, q0.y), __fmul2_rn(w12, make_float2(q0.z, q0.w)));
    const float2 ab1 = __ffma2_rn(w02, make_float2(q1.x, q1.y), __fmul2_rn(w12, make_float2(q1.z, q1.w)));
    const float2 omaz = __fadd2_rn(make_float2(1.0f, 1.0f), make_float2(-az.x, -az.y));
    acc[j] = fmaf(omaz.x, ab0.x, fmaf(az.x, ab0.y, acc[j]));
    acc[j + 1] = fmaf(omaz.y, ab1.x, fmaf(az.y, ab1.y, acc[j + 1]));
  }
}

// Par / fan column over a quad-layout view: the column's z rows are texel
// rows, so the quad at row r holds column c's rows r and r+1 and column c+1's,
// i.e. both voxels of a z pair as register pairs: one 16-byte load and two
// packed operations per pair.  Row r = min(z, H - 1) with weight 1 (az = 0:
// acc = fma(w0, P(r, iu), fma(w1, P(r, iu+1), acc))); the layout clamps row
// r + 1 exactly as min(z + 1, H - 1) does.
template <int GEOM, int ZC, typename S = float>
__device__ __forceinline__ void bp_column_quadrows(const typename QuadT<S>::T* __restrict__ p,
                                                   int W, int H, int Wp, int z0,
                                                   const ColGeom<GEOM>& g, float* acc,
                                                   int roff = 0) {
  const float cu = fminf(fmaxf(g.py, -4.0f), (float)W + 4.0f) - 0.5f;
  const float fu = floorf(cu);
  const float au = cu - fu;
  const int iu = min(max((int)fu, -kSinoPad), W) + kSinoPad;
  const float w0 = g.w * (1.0f - au), w1 = g.w * au;
  const typename QuadT<S>::T* col = p + iu;
  static_assert(ZC % 2 == 0, "ZC must be even");
  const float2 w02 = make_float2(w0, w0), w12 = make_float2(w1, w1);
#pragma unroll
  for (int j = 0; j < ZC; j += 2) {
    const float4 q = QuadT<S>::get(col + (size_t)(min(z0 + j - roff, H - 1) + kSinoPad) * Wp);
    const float2 t = __ffma2_rn(w02, make_float2(q.x, q.y),
                                __ffma2_rn(w12, make_float2(q.z, q.w),
                                           make_float2(acc[j], acc[j + 1])));
    acc[j] = t.x;
    acc[j + 1] = t.y;
  }
}

// Launch shape (BpShape): ZC z voxels per thread, blocks of 32 x rows
// columns, and the views split into vblocks blocks along grid z.  With
// vblocks > 1 every view block writes FP32 partial sums to part[vb][voxel]
// and bp_reduce_kernel adds them in block order (deterministic).
// MODE 0: the reference's detector; 1: decoupled detector (launch_bp_det);
// 2: a z-slab of the volume from a band of detector rows (launch_bp_sub).
template <int GEOM, int ZC, typename TS, typename TV, int MODE = 0>
// Cone columns take 16 bilinear taps per z pair; bounding registers to 64 keeps
// 4 CTAs (32 warps) per SM resident, 5% faster at 512^3 x 720 than the 66
// registers / 3 CTAs the compiler picks unbounded.  Par/fan columns need no
// bound.
__global__ void __launch_bounds__(256, GEOM == 2 ? 4 : 1) bp_pad_kernel(const __grid_constant__ VoxArgs A,
                                                     const TS* __restrict__ sino, int Wp,
                                                     TV* __restrict__ vol, int accumulate,
                                                     int nz, int vblocks,
                                                     float* __restrict__ part, int zb0) {
  // A block covers 32 x blockDim.y columns (blockDim.y = 4 or 8, one warp per
  // threadIdx.y); each warp takes an 8 x 4 patch of them, whose projections
  // span fewer detector texels at every view than a 32 x 1 row: fewer L1
  // wavefronts per quad load.
  const int w = threadIdx.y, lane = threadIdx.x;
  const int ix = blockIdx.x * 32 + 8 * (w & 3) + (lane & 7);
  const int iy = blockIdx.y * blockDim.y + 4 * (w >> 2) + (lane >> 3);
  const int zb = zb0 + blockIdx.z % nz, vb = blockIdx.z / nz;  // nz: z-blocks of the launch
  const int z0 = zb * ZC;
  if (ix >= A.W || iy >= A.W) return;
  const int vbeg = (int)((long long)A.nviews * vb / vblocks);
  const int vend = (int)((long long)A.nviews * (vb + 1) / vblocks);
  const int nzo = MODE == 2 ? A.nzs : A.H;  // output slices
  const bool cont = accumulate && vblocks == 1;
  float acc[ZC];
#pragma unroll
  for (int j = 0; j < ZC; ++j) acc[j] = 0.f;
  if (in_circle(ix, iy, A.hw)) {
    // Accumulating launches continue the stored sums view by view, so views
    // split over several launches give the one-launch result bit for bit.
    if (cont) {
      const size_t sz = (size_t)A.W * A.W;
      const TV* o = vol + (size_t)iy * A.W + ix + (size_t)z0 * sz;
#pragma unroll
      for (int j = 0; j < ZC; ++j)
        if (z0 + j < nzo) acc[j] = ldp(o + (size_t)j * sz);
    }
    const float x = (float)ix - ((float)A.hw + 0.5f);
    const float y = (float)iy - ((float)A.hw + 0.5f);
    static_assert(IsQuad<TS>::value, "views in the quad layout");
    using S = typename IsQuad<TS>::Storage;
    const auto* q = reinterpret_cast<const typename QuadT<S>::T*>(sino);
    if constexpr (MODE == 1) {
      // decoupled detector: every geometry interpolates in v
      const size_t vstride = (size_t)Wp * (A.det_h + 2 * kSinoPad);
      for (int v = vbeg; v < vend; ++v) {
        const ColGeom<GEOM> g =
            col_geom<GEOM>(x, y, A.trig[v], A.SR, A.v0, A.hwd, A.v0d, A.inv_du, A.inv_dv);
        bp_column_quad<ZC, S, GEOM>(q + (size_t)v * vstride, A.det_w, A.det_h, Wp, z0, g, acc);
      }
    } else {
      // MODE 0: the whole detector; MODE 2: a band of rows row0 .. row0 +
      // nrows - 1 of it for the slab's voxels zoff + z (taps in whole-detector
      // rows, offset by row0)
      const int rows = MODE == 2 ? A.nrows : A.H;
      const int zg = MODE == 2 ? A.zoff + z0 : z0;
      const int roff = MODE == 2 ? A.row0 : 0;
      const size_t vstride = (size_t)Wp * (rows + 2 * kSinoPad);
      for (int v = vbeg; v < vend; ++v) {
        const ColGeom<GEOM> g = col_geom<GEOM>(x, y, A.trig[v], A.SR, A.v0, (float)A.hw, A.v0,
                                               1.f, 1.f);
        if constexpr (GEOM == 2)
          bp_column_quad<ZC, S>(q + (size_t)v * vstride, A.W, rows, Wp, zg, g, acc, roff);
        else  // par / fan: the z rows are texel rows
          bp_column_quadrows<GEOM, ZC, S>(q + (size_t)v * vstride, A.W, rows, Wp, zg, g, acc,
                                          roff);
      }
    }
  }
  else if (cont) {
    return;  // outside the circle: the stored sums stand
  }
  const size_t base = (size_t)iy * A.W + ix;
  const size_t sz = (size_t)A.W * A.W;
  TV* const out = vol + base + (size_t)z0 * sz;
  if (vblocks > 1) {
    float* pp = part + (size_t)vb * sz * A.H + base;
#pragma unroll
    for (int j = 0; j < ZC; ++j)
      if (z0 + j < A.H) pp[(size_t)(z0 + j) * sz] = acc[j];
    return;
  }
#pragma unroll
  for (int j = 0; j < ZC; ++j) {
    if (z0 + j < nzo) {
      stf(out + (size_t)j * sz, acc[j]);
    }
  }
}

template <typename TV>
__global__ void __launch_bounds__(256) bp_reduce_kernel(const float* __restrict__ part,
                                                        int vblocks, long long N,
                                                        TV* __restrict__ vol, int accumulate) {
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < N; i += (long long)gridDim.x * 256) {
    float s = accumulate ? ldp(vol + i) : 0.f;
    for (int b = 0; b < vblocks; ++b) s += part[(size_t)b * N + i];
    stf(vol + i, s);
  }
}


template <int GEOM, int ZC, typename TS, typename TV>
static cudaError_t bp_pad_go(const VoxArgs& a, const void* sino, int Wp, void* vol, bool accum,
                             const BpShape& shp, float* part, cudaStream_t st) {
  const int nzall = (a.H + ZC - 1) / ZC;
  if (shp.zb0 < 0 || shp.zb0 >= nzall || (shp.vblocks > 1 && (shp.zb0 > 0 || shp.nzb > 0)))
    return cudaErrorInvalidValue;
  const int nz = shp.nzb > 0 ? std::min(shp.nzb, nzall - shp.zb0) : nzall - shp.zb0;
  dim3 blk(32, shp.rows), grd((a.W + 31) / 32, (a.W + shp.rows - 1) / shp.rows,
                              nz * shp.vblocks);
  bp_pad_kernel<GEOM, ZC, TS, TV><<<grd, blk, 0, st>>>(a, (const TS*)sino, Wp, (TV*)vol,
                                                       accum ? 1 : 0, nz, shp.vblocks, part,
                                                       shp.zb0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || shp.vblocks == 1) return e;
  const long long N = (long long)a.W * a.W * a.H;
  const int ctas = (int)std::min<long long>((N + 255) / 256, 16ll * device_sms());
  bp_reduce_kernel<TV><<<ctas, 256, 0, st>>>(part, shp.vblocks, N, (TV*)vol, accum ? 1 : 0);
  return cudaGetLastError();
}

template <int GEOM, typename TS, typename TV>
static cudaError_t bp_pad_zc(const VoxArgs& a, const void* sino, int Wp, void* vol, bool accum,
                             const BpShape& shp, float* part, cudaStream_t st) {
  if (shp.zc == 8) return bp_pad_go<GEOM, 8, TS, TV>(a, sino, Wp, vol, accum, shp, part, st);
  return bp_pad_go<GEOM, 16, TS, TV>(a, sino, Wp, vol, accum, shp, part, st);
}

bool bp_shape_valid(const BpShape& s) {
  return (s.zc == 8 || s.zc == 16) && (s.rows == 4 || s.rows == 8) && s.vblocks >= 1 &&
         s.vblocks <= 64;
}

template <int GEOM>
static cudaError_t bp_quad_types(const VoxArgs& a, const void* sino_quad, int stype, int Wp,
                                 void* vol, int vtype, bool accumulate, const BpShape& shp,
                                 float* part, cudaStream_t st) {
  using QF = QuadLayout<float>;
  using QH = QuadLayout<__half>;
  using QB = QuadLayout<__nv_bfloat16>;
  if (stype == kF32 && vtype == kF32)
    return bp_pad_zc<GEOM, QF, float>(a, sino_quad, Wp, vol, accumulate, shp, part, st);
  if (stype == kF32 && vtype == kF16)
    return bp_pad_zc<GEOM, QF, __half>(a, sino_quad, Wp, vol, accumulate, shp, part, st);
  if (stype == kF32 && vtype == kBF16)
    return bp_pad_zc<GEOM, QF, __nv_bfloat16>(a, sino_quad, Wp, vol, accumulate, shp, part, st);
  if (stype == kF16 && vtype == kF16)
    return bp_pad_zc<GEOM, QH, __half>(a, sino_quad, Wp, vol, accumulate, shp, part, st);
  if (stype == kF16 && vtype == kF32)
    return bp_pad_zc<GEOM, QH, float>(a, sino_quad, Wp, vol, accumulate, shp, part, st);
  if (stype == kBF16 && vtype == kBF16)
    return bp_pad_zc<GEOM, QB, __nv_bfloat16>(a, sino_quad, Wp, vol, accumulate, shp, part, st);
  if (stype == kBF16 && vtype == kF32)
    return bp_pad_zc<GEOM, QB, float>(a, sino_quad, Wp, vol, accumulate, shp, part, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_bp_quad(int geom, const VoxArgs& a, const void* sino_quad, int stype,
                           void* vol, int vtype, bool accumulate, const BpShape& shp,
                           float* part, cudaStream_t st) {
  if (!bp_shape_valid(shp) || (shp.vblocks > 1 && !part)) return cudaErrorInvalidValue;
  const int Wp = sino_pad_pitch(a.W);
  switch (geom) {
    case 0: return bp_quad_types<0>(a, sino_quad, stype, Wp, vol, vtype, accumulate, shp, part, st);
    case 1: return bp_quad_types<1>(a, sino_quad, stype, Wp, vol, vtype, accumulate, shp, part, st);
    case 2: return bp_quad_types<2>(a, sino_quad, stype, Wp, vol, vtype, accumulate, shp, part, st);
    default: return cudaErrorInvalidValue;
  }
}

// Decoupled-detector BP: FP32 det_w x det_h views in the quad layout
// (launch_pad_sino_quad), blocks of 32 x 4 columns, every geometry
// interpolating in v.
cudaError_t launch_bp_det(int geom, const VoxArgs& a, const void* sino_quad, float* vol,
                          bool accumulate, cudaStream_t st) {
  if (a.nviews <= 0) return cudaSuccess;
  // par / fan: a column's z taps are the same in every view and stay in
  // registers across the view loop; 8 z voxels per thread keep that at ~100
  // registers without spills
  constexpr int ZC = 16, ZP = 8;
  using Q = QuadLayout<float>;
  const int Wp = sino_pad_pitch(a.det_w);
  const int zc = geom == 2 ? ZC : ZP;
  const int nz = (a.H + zc - 1) / zc;
  dim3 blk(32, 4), grd((a.W + 31) / 32, (a.W + 3) / 4, nz);
  const int acc = accumulate ? 1 : 0;
  const Q* sq = static_cast<const Q*>(sino_quad);
  switch (geom) {
    case 0:
      bp_pad_kernel<0, ZP, Q, float, 1><<<grd, blk, 0, st>>>(a, sq, Wp, vol, acc, nz, 1, nullptr, 0);
      break;
    case 1:
      bp_pad_kernel<1, ZP, Q, float, 1><<<grd, blk, 0, st>>>(a, sq, Wp, vol, acc, nz, 1, nullptr, 0);
      break;
    case 2:
      bp_pad_kernel<2, ZC, Q, float, 1><<<grd, blk, 0, st>>>(a, sq, Wp, vol, acc, nz, 1, nullptr, 0);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_bp_sub(int geom, const VoxArgs& a, const void* sino_quad, float* vol,
                          bool accumulate, cudaStream_t st) {
  if (a.nviews <= 0) return cudaSuccess;
  constexpr int ZC = 16;
  const int Wp = sino_pad_pitch(a.W);
  const int nz = (a.nzs + ZC - 1) / ZC;
  dim3 blk(32, 4), grd((a.W + 31) / 32, (a.W + 3) / 4, nz);
  const int acc = accumulate ? 1 : 0;
  using Q = QuadLayout<float>;
  const Q* sq = static_cast<const Q*>(sino_quad);
  switch (geom) {
    case 0:
      bp_pad_kernel<0, ZC, Q, float, 2><<<grd, blk, 0, st>>>(a, sq, Wp, vol, acc, nz, 1, nullptr, 0);
      break;
    case 1:
      bp_pad_kernel<1, ZC, Q, float, 2><<<grd, blk, 0, st>>>(a, sq, Wp, vol, acc, nz, 1, nullptr, 0);
      break;
    case 2:
      bp_pad_kernel<2, ZC, Q, float, 2><<<grd, blk, 0, st>>>(a, sq, Wp, vol, acc, nz, 1, nullptr, 0);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// dst = w * src (first) or dst + w * src: the sub-ray average of a
// super-sampled FP, one sub-ray sinogram at a time.
__global__ void __launch_bounds__(256) add_scaled_kernel(const float* __restrict__ src,
                                                         float* __restrict__ dst, long long n,
                                                         float w, int first) {
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (long long)gridDim.x * 256) {
    const float t = w * src[i];
    dst[i] = first ? t : dst[i] + t;
  }
}

cudaError_t launch_add_scaled(const float* src, float* dst, long long n, float w, bool first,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int ctas = (int)std::min<long long>((n + 255) / 256, 16ll * device_sms());
  add_scaled_kernel<<<ctas, 256, 0, st>>>(src, dst, n, w, first ? 1 : 0);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// general3D BP (CUDAmex_general3D_BP.cu:61-188): ray-driven, two-corner
// scatter with atomics.  Positions advance incrementally in binary32 and the
// voxel indices / weights / deposits are binary32 exactly as written, because
// floor()/ceil() of the position are discontinuous.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) g3d_bp_kernel(
    const __grid_constant__ RayArgs A, const float* __restrict__ sino,
    const float* __restrict__ pts, float* __restrict__ vol) {
  const int view = blockIdx.x;
  const int tiles_u = (A.det_w + 31) >> 5;
  const int ix = (blockIdx.y % tiles_u) * 32 + threadIdx.x;
  const int iy = (blockIdx.y / tiles_u) * blockDim.y + threadIdx.y;
  if (ix >= A.det_w || iy >= A.det_h) return;
  const float p = __ldg(sino + (size_t)(A.view0 + view * A.vstride) * A.P +
                        (size_t)iy * A.det_w + ix);
  if (p == 0.f) return;  // adds +0 only; the sum is unchanged
  const Ray r = make_ray<3>(A, view, ix, iy, pts);
  const int S = A.S, Z = A.Z;
  const size_t SS = (size_t)S * S;
  const float ps = fmul(p, A.step);
  float cx = r.cx, cy = r.cy, cz = r.cz;
  // Consecutive samples (step 0.5) mostly deposit into the same two voxels:
  // the deposits of a run of samples with the same targets are summed in
  // registers and reach memory in one atomic per voxel (the deposits
  // themselves are the reference's binary32 values; only their grouping
  // changes, as the order of the atomics already does).
  size_t qL = ~(size_t)0, qU = 0;
  float aL = 0.f, aU = 0.f;
  for (int k = 0; k < r.n; ++k) {
    const float fx = fsub(cx, A.bx), fy = fsub(cy, A.by), fz = fsub(cz, A.bz);
    const float flx = floorf(fx), fly = floorf(fy), flz = floorf(fz);
    const int iL = (int)flx, iU = (int)ceilf(fx);
    const int jL = (int)fly, jU = (int)ceilf(fy);
    const int kL = (int)flz, kU = (int)ceilf(fz);
    if (!(iL < 0 || jL < 0 || kL < 0 || iU >= S || jU >= S || kU >= Z)) {
      const float wxx = fadd(fsub(fx, (float)iL), 0.5f);
      const float wyy = fadd(fsub(fy, (float)jL), 0.5f);
      const float wz = fadd(fsub(fz, (float)kL), 0.5f);
      const float wzz = fsub(1.0f, wz);
      const float pxy = fmul(fmul(ps, wxx), wyy);
      const size_t base = (size_t)jL * S + (size_t)iL;
      const size_t tL = base + (size_t)kL * SS, tU = base + (size_t)kU * SS;
      const float dL = fmul(pxy, wzz), dU = fmul(pxy, wz);
      if (tL == qL && tU == qU) {
        aL = fadd(aL, dL);
        aU = fadd(aU, dU);
      } else {
        if (qL != ~(size_t)0) {
          atomicAdd(vol + qL, aL);
          atomicAdd(vol + qU, aU);
        }
        qL = tL;
        qU = tU;
        aL = dL;
        aU = dU;
      }
    }
    cx = fadd(cx, r.dx);
    cy = fadd(cy, r.dy);
    cz = fadd(cz, r.dz);
  }
  if (qL != ~(size_t)0) {
    atomicAdd(vol + qL, aL);
    atomicAdd(vol + qU, aU);
  }
}

// ---------------------------------------------------------------------------
// Matched-adjoint general3D BP (no counterpart in the reference, whose BP is a
// two-corner scatter that is not the transpose of its FP; the eight-corner form
// left commented out at CUDAmex_general3D_BP.cu:172-179 points this way).  The
// exact transpose of the general3D FP of this library (the slab kernel, border
// addressing, step 0.5): the same rays and the same FP32 sample positions
// fma(k, d, t0) in tap space, the eight trilinear taps of each sample, and
// p * step * w added to each tap voxel inside the volume (frame taps, which
// the FP reads as zeros, are dropped).  A run of samples in the same cell is
// summed in registers and lands in one atomic per corner.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void adj_flush(float* __restrict__ vol, int S, int Z, int ci, int cj,
                                          int ck, const float (&w)[8]) {
  // ci, cj, ck: lower tap in padded (voxel + 1) coordinates
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const int i = ci + (t & 1) - 1, j = cj + ((t >> 1) & 1) - 1, k = ck + (t >> 2) - 1;
    if (w[t] != 0.f && i >= 0 && i < S && j >= 0 && j < S && k >= 0 && k < Z)
      atomicAdd(vol + (size_t)i + (size_t)S * ((size_t)j + (size_t)S * k), w[t]);
  }
}

__global__ void __launch_bounds__(256) g3d_bp_adjoint_kernel(
    const __grid_constant__ RayArgs A, const float* __restrict__ sino,
    const float* __restrict__ pts, float* __restrict__ vol) {
  const int view = blockIdx.x;
  const int tiles_u = (A.det_w + 31) >> 5;
  const int ix = (blockIdx.y % tiles_u) * 32 + threadIdx.x;
  const int iy = (blockIdx.y / tiles_u) * blockDim.y + threadIdx.y;
  if (ix >= A.det_w || iy >= A.det_h) return;
  const float p = __ldg(sino + (size_t)(A.view0 + view * A.vstride) * A.P +
                        (size_t)iy * A.det_w + ix);
  if (p == 0.f) return;
  const Ray r = make_ray<3>(A, view, ix, iy, pts);
  const int S = A.S, Z = A.Z;
  // tap space: padded coordinate minus 0.5 = world - b + 0.5 (as the slab FP)
  const float tx0 = (r.cx - A.bx) + 0.5f, ty0 = (r.cy - A.by) + 0.5f, tz0 = (r.cz - A.bz) + 0.5f;
  // samples whose taps can touch the padded volume: t in [0, P - 1) per axis
  float klo = 0.f, khi = (float)r.n;
  auto clampk = [&](float t0, float d, float hi) {
    if (d == 0.f) {
      if (!(t0 >= 0.f && t0 < hi)) khi = -1.f;
    } else {
      const float k1 = (0.f - t0) / d, k2 = (hi - t0) / d;
      klo = fmaxf(klo, fminf(k1, k2));
      khi = fminf(khi, fmaxf(k1, k2));
    }
  };
  clampk(tx0, r.dx, (float)(S + 1));
  clampk(ty0, r.dy, (float)(S + 1));
  clampk(tz0, r.dz, (float)(Z + 1));
  if (!(khi >= klo)) return;
  const int k0 = max((int)floorf(klo) - 1, 0), k1 = min((int)ceilf(khi) + 1, r.n);
  const float ps = p * A.step;
  float w[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  int ci = -1000000, cj = 0, ck = 0;
  for (int k = k0; k < k1; ++k) {
    const float kf = (float)k;
    const float tx = fmaf(kf, r.dx, tx0), ty = fmaf(kf, r.dy, ty0), tz = fmaf(kf, r.dz, tz0);
    const float fx = floorf(tx), fy = floorf(ty), fz = floorf(tz);
    const int i = (int)fx, j = (int)fy, l = (int)fz;
    if (i < -1 || i > S || j < -1 || j > S || l < -1 || l > Z) continue;  // all taps outside
    if (i != ci || j != cj || l != ck) {
      if (ci != -1000000) adj_flush(vol, S, Z, ci, cj, ck, w);
#pragma unroll
      for (int t = 0; t < 8; ++t) w[t] = 0.f;
      ci = i;
      cj = j;
      ck = l;
    }
    const float ax = tx - fx, ay = ty - fy, az = tz - fz;
    const float bx = 1.f - ax, by = 1.f - ay, bz = 1.f - az;
    const float p00 = ps * by * bz, p10 = ps * ay * bz, p01 = ps * by * az, p11 = ps * ay * az;
    w[0] = fmaf(bx, p00, w[0]);
    w[1] = fmaf(ax, p00, w[1]);
    w[2] = fmaf(bx, p10, w[2]);
    w[3] = fmaf(ax, p10, w[3]);
    w[4] = fmaf(bx, p01, w[4]);
    w[5] = fmaf(ax, p01, w[5]);
    w[6] = fmaf(bx, p11, w[6]);
    w[7] = fmaf(ax, p11, w[7]);
  }
  if (ci != -1000000) adj_flush(vol, S, Z, ci, cj, ck, w);
}

cudaError_t launch_g3d_bp_adjoint(const RayArgs& a, const float* sino, const float* pts,
                                  float* vol, cudaStream_t st) {
  if (a.nviews <= 0) return cudaSuccess;
  const int tiles = ((a.det_w + 31) / 32) * ((a.det_h + 7) / 8);
  dim3 blk(32, 8), grd(a.nviews, tiles);
  g3d_bp_adjoint_kernel<<<grd, blk, 0, st>>>(a, sino, pts, vol);
  return cudaGetLastError();
}

cudaError_t launch_g3d_bp(const RayArgs& a, const float* sino,
                          const float* pts, float* vol, cudaStream_t st) {
  if (a.nviews <= 0) return cudaSuccess;
  const int tiles = ((a.det_w + 31) / 32) * ((a.det_h + 7) / 8);
  dim3 blk(32, 8), grd(a.nviews, tiles);
  g3d_bp_kernel<<<grd, blk, 0, st>>>(a, sino, pts, vol);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// OSC kernels.  The subset FP with the residual epilogue
// (CUDAmex_oscIter.cu:140-271) is the slab kernel of k_slab.cu with border
// addressing and step 0.5.
// ---------------------------------------------------------------------------
// Dual BP of the residuals with border addressing (CUDAmex_oscIter.cu:305-356)
// into register accumulators, then mu <- max(mu + mu*num/den, 0) inside the
// circle (:119-134).  num/den never touch memory.
// DET: a decoupled detector (A.det_w x A.det_h pixels of reciprocal pitch
// A.inv_du, A.inv_dv; no counterpart in the reference): every geometry
// interpolates its residuals in v, as the detector BP does.
template <int GEOM, int ZC, typename TM, bool DET = false, typename SD = float>
__global__ void __launch_bounds__(256) osc_bp_update_kernel(
    const __grid_constant__ VoxArgs A, const void* __restrict__ rpre,
    const void* __restrict__ rpost, TM* __restrict__ mu, TM* __restrict__ padx,
    TM* __restrict__ pady, int Pf) {
  using Q = typename QuadT<SD>::T;  // residual quads: float4, or four FP16 in a uint2
  // 8 x 4 column patch per warp, as in bp_pad_kernel (blocks of 32 x 8)
  const int w = threadIdx.y, lane = threadIdx.x;
  const int ix = blockIdx.x * 32 + 8 * (w & 3) + (lane & 7);
  const int iy = blockIdx.y * blockDim.y + 4 * (w >> 2) + (lane >> 3);
  // slices zl .. zl + ZC - 1 of the output (slices zoff .. zoff + nzs - 1 of
  // the volume: the whole volume, or a z-slab of it)
  const int zl = blockIdx.z * ZC;
  const int z0 = A.zoff + zl;
  if (ix >= A.W || iy >= A.W) return;
  if (!in_circle(ix, iy, A.hw)) return;
  float num[ZC], den[ZC];
#pragma unroll
  for (int j = 0; j < ZC; ++j) num[j] = den[j] = 0.f;
  const float x = (float)ix - ((float)A.hw + 0.5f);
  const float y = (float)iy - ((float)A.hw + 0.5f);
  const int Wp = sino_pad_pitch(DET ? A.det_w : A.W);
  const size_t vstride = (size_t)Wp * ((DET ? A.det_h : A.H) + 2 * kSinoPad);
  for (int v = 0; v < A.nviews; ++v) {
    const ColGeom<GEOM> g =
        DET ? col_geom<GEOM>(x, y, A.trig[v], A.SR, A.v0, A.hwd, A.v0d, A.inv_du, A.inv_dv)
            : col_geom<GEOM>(x, y, A.trig[v], A.SR, A.v0, (float)A.hw, A.v0, 1.f, 1.f);
    // zero frame = border addressing (CUDAmex_oscIter.cu:419-425); residuals
    // in the quad layout written by the FP epilogue
    const Q* qpre = static_cast<const Q*>(rpre) + (size_t)v * vstride;
    const Q* qpost = static_cast<const Q*>(rpost) + (size_t)v * vstride;
    if constexpr (DET) {
      bp_column_quad<ZC, SD, GEOM>(qpre, A.det_w, A.det_h, Wp, z0, g, num);
      bp_column_quad<ZC, SD, GEOM>(qpost, A.det_w, A.det_h, Wp, z0, g, den);
    } else if constexpr (GEOM == 2) {
      bp_column_quad<ZC, SD>(qpre, A.W, A.H, Wp, z0, g, num);
      bp_column_quad<ZC, SD>(qpost, A.W, A.H, Wp, z0, g, den);
    } else {
      bp_column_quadrows<GEOM, ZC, SD>(qpre, A.W, A.H, Wp, z0, g, num);
      bp_column_quadrows<GEOM, ZC, SD>(qpost, A.W, A.H, Wp, z0, g, den);
    }
  }
  const size_t base = (size_t)iy * A.W + ix;
  const size_t sz = (size_t)A.W * A.W;
  const size_t Ps = (size_t)A.W + 2;
#pragma unroll
  for (int j = 0; j < ZC; ++j) {
    const int z = zl + j;
    if (z < A.nzs) {
      TM* o = mu + base + (size_t)z * sz;
      const float f = ldp(o);
      const float m = fmaxf(f + (f * num[j] / den[j]), 0.f);
      stf(o, m);
      if (padx) {
        // the slab FP's padded layouts: x-fastest and y-fastest, frame of one
        const size_t zp = (size_t)(z + 1) * Ps;
        stf(padx + (size_t)(ix + 1) + (size_t)Pf * ((size_t)(iy + 1) + zp), m);
        stf(pady + (size_t)(iy + 1) + (size_t)Pf * ((size_t)(ix + 1) + zp), m);
      }
    }
  }
}

cudaError_t launch_osc_bp_update_det(int geom, const VoxArgs& a, const float* rpre,
                                     const float* rpost, void* mu, int mt, void* padx,
                                     void* pady, int Pf, cudaStream_t st) {
  constexpr int ZC = 4;
  if (mt != kF32) return cudaErrorInvalidValue;
  dim3 blk(32, 8), grd((a.W + 31) / 32, (a.W + 7) / 8, (a.nzs + ZC - 1) / ZC);
#define OSC_BP(G)                                                                      \
  osc_bp_update_kernel<G, ZC, float, true><<<grd, blk, 0, st>>>(a, rpre, rpost, (float*)mu, \
                                                                (float*)padx, (float*)pady, Pf)
  if (geom == 0) OSC_BP(0);
  else if (geom == 1) OSC_BP(1);
  else OSC_BP(2);
#undef OSC_BP
  return cudaGetLastError();
}

cudaError_t launch_osc_bp_update(int geom, const VoxArgs& a,
                                 const void* rpre, const void* rpost,
                                 void* mu, int mt, void* padx, void* pady, int Pf,
                                 cudaStream_t st, int dt) {
  constexpr int ZC = 4;
  if (a.zoff % ZC != 0 || a.zoff < 0 || a.nzs < 1 || a.zoff + a.nzs > a.H)
    return cudaErrorInvalidValue;
  dim3 blk(32, 8), grd((a.W + 31) / 32, (a.W + 7) / 8, (a.nzs + ZC - 1) / ZC);
  if (dt == kF16) {  // FP16 residual views (FP32 mu)
    if (mt != kF32) return cudaErrorInvalidValue;
#define OSC_BP16(G)                                                                      \
  osc_bp_update_kernel<G, ZC, float, false, __half><<<grd, blk, 0, st>>>(                \
      a, rpre, rpost, (float*)mu, (float*)padx, (float*)pady, Pf)
    if (geom == 0) OSC_BP16(0);
    else if (geom == 1) OSC_BP16(1);
    else OSC_BP16(2);
#undef OSC_BP16
    return cudaGetLastError();
  }
#define OSC_BP(G, T)                                                                 \
  osc_bp_update_kernel<G, ZC, T><<<grd, blk, 0, st>>>(a, rpre, rpost, (T*)mu, (T*)padx, \
                                                      (T*)pady, Pf)
  if (mt == kF32) {
    if (geom == 0) OSC_BP(0, float);
    else if (geom == 1) OSC_BP(1, float);
    else OSC_BP(2, float);
  } else if (mt == kF16) {
    if (geom == 0) OSC_BP(0, __half);
    else if (geom == 1) OSC_BP(1, __half);
    else OSC_BP(2, __half);
  } else {
    if (geom == 0) OSC_BP(0, __nv_bfloat16);
    else if (geom == 1) OSC_BP(1, __nv_bfloat16);
    else OSC_BP(2, __nv_bfloat16);
  }
#undef OSC_BP
  return cudaGetLastError();
}

// Residual views of one OSC subset from its line integrals l (W x H x n
// views, e.g. the sum of the z-slabs' forward passes): pre e^-l - post and
// pre e^-l l (CUDAmex_oscIter.cu:262-268), the values the slab FP's residual
// epilogue writes, into the same padded quad layout.
__global__ void __launch_bounds__(256) osc_residual_kernel(const float* __restrict__ l,
                                                           const float* __restrict__ pre,
                                                           const float* __restrict__ post, int W,
                                                           int H, long long n,
                                                           float* __restrict__ rpre,
                                                           float* __restrict__ rpost) {
  const long long P = (long long)W * H;
  const int Wp = sino_pad_pitch(W);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const long long v = i / P;
    const int pix = (int)(i - v * P);
    const int iy = pix / W, ix = pix - iy * W;
    const float lv = __ldg(l + i), pv = __ldg(pre + i), qv = __ldg(post + i);
    const float ehat = pv * expf(-lv);
    const float r0 = ehat - qv, r1 = ehat * lv;
    const size_t ri = ((size_t)v * (H + 2 * kSinoPad) + (iy + kSinoPad)) * Wp + (ix + kSinoPad);
    const size_t q[4] = {4 * ri, 4 * (ri - Wp) + 1, 4 * (ri - 1) + 2, 4 * (ri - Wp - 1) + 3};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      rpre[q[t]] = r0;
      rpost[q[t]] = r1;
    }
  }
}

cudaError_t launch_osc_residual(const float* l, const float* pre, const float* post, int W, int H,
                                int nviews, float* rpre, float* rpost, cudaStream_t st) {
  const long long n = (long long)W * H * nviews;
  if (n <= 0) return cudaSuccess;
  const long long blocks = std::min<long long>((n + 255) / 256, 16ll * device_sms());
  osc_residual_kernel<<<(unsigned)blocks, 256, 0, st>>>(l, pre, post, W, H, n, rpre, rpost);
  return cudaGetLastError();
}

}  // namespace mexct
