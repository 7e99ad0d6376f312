// k_iter.cu -- TV descent, FP64 reductions and the FDK/FBP pre-filter.
//
// TV (CUDAmex_TVmin_3D.cu:101-234).  The reference runs three full-volume
// passes per step (gradient kernel -> thrust norm -> thrust saxpy) and stores
// the gradient.  Here a step is two passes and no gradient volume:
//   tv_norm_kernel   gradient recomputed per voxel, ||g||^2 reduced (FP32 per
//                    thread, FP64 across threads: warp shuffles, per-CTA
//                    partials, last-CTA fixed-order sum: deterministic), step
//                    scale -c/||g|| written to HBM;
//   tv_update_kernel gradient recomputed, y = x + scale*g into the other
//                    buffer of a ping-pong pair.
// Algorithmic traffic is 12 bytes per voxel per step (read x twice, write y).
// FP32 volumes whose x extent is a multiple of 4 use tv4_kernel (four x-voxels
// per thread, 16-byte loads and stores, packed FP32x2 arithmetic): 512^3 step
// 0.92 -> 0.55 ms, 2.9 TB/s of algorithmic traffic; other volumes tv_sweep.
#include <atomic>
#include <cstdint>
#include <cstdio>

#include "kernels.h"

namespace mexct {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-level FP64 sum with a fixed tree (deterministic); blockDim.x*y*z
// threads, result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  v = warp_sum(v);
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (tid < 32) {
    r = (tid < (nt + 31) / 32) ? red[tid] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Last-CTA finalisation: every CTA stores its partial, the last one to arrive
// sums all partials in index order (deterministic).  Returns true in thread 0
// of the last CTA with *total set.
__device__ __forceinline__ bool finish_partials(double mine, double* partials,
                                                unsigned* counter,
                                                double* total) {
  __shared__ bool last;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
  const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (tid == 0) {
    partials[bid] = mine;
    __threadfence();
    last = (atomicAdd(counter, 1u) == nb - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc = 0.0;
  for (unsigned i = tid; i < nb; i += nt) acc += __ldcg(partials + i);
  acc = block_sum(acc);
  if (tid == 0) {
    *total = acc;
    *counter = 0u;  // ready for the next launch on this stream
  }
  return tid == 0;
}

// ---------------------------------------------------------------------------
// Tiled TV gradient.  With backward differences a_p = x_p - x_{p-1},
// b_p = x_p - x_{p-sy}, c_p = x_p - x_{p-sz} and r_p = 1/(eps + |(a,b,c)_p|),
// the four terms of the reference's gradient at voxel i are
//   g_i = (a+b+c)_i r_i - a_{i+1} r_{i+1} - b_{i+sy} r_{i+sy} - c_{i+sz} r_{i+sz}
// (CUDAmex_TVmin_3D.cu:121-152: the second to fourth terms are the first
// term's components at the +x, +y and +z neighbours), so each voxel's
// (a, b, c, r) is computed once (one reciprocal square root, one reciprocal)
// instead of four times.  A CTA of 32 x 16 threads sweeps a column tile along z:
// thread (tx, ty) computes q at its column in every plane, takes the +x
// neighbour's value by a shuffle, the +y neighbour's from shared memory (one
// barrier per plane) and the +z neighbour's from its next plane, and writes the
// voxel when tx < 31 and ty < 15 (tiles overlap by one column and one row).  The
// next plane's loads are issued before the current plane is computed.
// ---------------------------------------------------------------------------
// 32 x 16 threads (31 x 15 outputs: 91 % of the threads own a voxel, 85 % with
// 32 x 8; 512^3 step 0.978 -> 0.926 ms), 32 planes per CTA
constexpr int kTvBx = 32, kTvBy = 16, kTvZ = 32;
constexpr int kTvOx = kTvBx - 1, kTvOy = kTvBy - 1;  // output voxels per tile row / column

// Sweep of one tile: calls visit(z, x_z, g, out) for every plane z of the
// tile, with x_z the voxel value, g the gradient (0 on the volume border) and
// out whether this thread owns the voxel.
template <typename T, typename F>
__device__ __forceinline__ void tv_sweep(const T* __restrict__ v, int Nx, int Ny, int Nz,
                                         F&& visit) {
  __shared__ float sqb[2][kTvBy][kTvBx];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int gx = blockIdx.x * kTvOx + tx, gy = blockIdx.y * kTvOy + ty;
  const int z0 = blockIdx.z * kTvZ;
  const int zend = min(z0 + kTvZ, Nz);
  const size_t sy = (size_t)Nx, sz = (size_t)Nx * Ny;
  const bool incol = gx < Nx && gy < Ny;
  const bool qcol = incol && gx >= 1 && gy >= 1;  // columns where q exists
  const bool own = incol && tx < kTvOx && ty < kTvOy;
  const size_t ci = (size_t)gx + (size_t)gy * sy;
  // column-invariant parts of the interior test and of the loads
  const bool col_int = gx >= 1 && gy >= 1 && gx < Nx - 1 && gy < Ny - 1;
  const bool ld_y = gy >= 1, ld_m = tx == 0 && gx >= 1;
  const int srow = ty + (ty < kTvOy);  // row of the +y neighbour in sqb
  // value of the plane below the first one, and the first plane's loads
  float xprev = (qcol && z0 >= 1) ? ldf(v + ci + (size_t)(z0 - 1) * sz) : 0.f;
  float xcur = 0.f, xym = 0.f, xxm = 0.f;
  const T* pl = v + ci + (size_t)z0 * sz;  // column at the plane being loaded
  auto load = [&](int p, float& xo, float& yo, float& mo) {
    if (incol && p < Nz) {
      xo = ldf(pl);
      yo = ld_y ? ldf(pl - sy) : 0.f;
      mo = ld_m ? ldf(pl - 1) : 0.f;
    }
    pl += sz;
  };
  load(z0, xcur, xym, xxm);
  float q0p = 0.f, qanp = 0.f, xz = 0.f;  // plane p-1: own q0, +x neighbour's qa, x
  for (int p = z0; p <= zend; ++p) {
    float xn = 0.f, yn = 0.f, mn = 0.f;
    if (p + 1 <= zend) load(p + 1, xn, yn, mn);  // prefetch the next plane
    // x_{p-1} of lane tx is lane tx-1's x_p; lane 0 loaded it
    const float xl = __shfl_up_sync(0xffffffffu, xcur, 1);
    const float xm = tx == 0 ? xxm : xl;
    float q0 = 0.f, qa = 0.f, qb = 0.f, qc = 0.f;
    if (qcol && p >= 1 && p < Nz) {
      const float a = xcur - xm, b = xcur - xym, c = xcur - xprev;
      // |(a,b,c)| from the hardware reciprocal square root and 1/(eps + |.|)
      // from the hardware reciprocal (a few ulp each, far inside the 1e-5
      // bound; the IEEE-rounded forms cost ~4x the instructions of the whole
      // stencil).  s = 0 (flat region) gives |.| = 0 as it must.
      const float s2 = fmaf(c, c, fmaf(b, b, a * a));
      const float nrm = s2 > 0.f ? s2 * rsqrtf(s2) : 0.f;
      const float r = __fdividef(1.0f, 1.0e-6f + nrm);
      q0 = ((a + b) + c) * r;
      qa = a * r;
      qb = b * r;
      qc = c * r;
    }
    if (p > z0) {
      const int z = p - 1;
      const bool interior = col_int && z >= 1 && z < Nz - 1;
      const float g = interior ? ((q0p - qanp) - sqb[(p - 1) & 1][srow][tx]) - qc : 0.f;
      visit(z, xz, g, own && interior, own);
    }
    sqb[p & 1][ty][tx] = qb;
    qanp = __shfl_down_sync(0xffffffffu, qa, 1);
    q0p = q0;
    xz = xcur;
    xprev = xcur;
    xcur = xn;
    xym = yn;
    xxm = mn;
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(kTvBx * kTvBy) tv_norm_kernel(
    const T* __restrict__ x, int Nx, int Ny, int Nz, float c,
    const double* __restrict__ cmul, double* __restrict__ partials,
    unsigned* __restrict__ counter, float* __restrict__ scale,
    double* __restrict__ norm) {
  // ||g||^2: squares and the 32-voxel sum of a thread in FP32, every level
  // above in FP64 (fixed order, deterministic).
  float ss = 0.f;
  tv_sweep(x, Nx, Ny, Nz, [&](int, float, float g, bool interior, bool) {
    if (interior) ss = fmaf(g, g, ss);
  });
  const double blk = block_sum((double)ss);
  double total;
  if (finish_partials(blk, partials, counter, &total)) {
    const double m = sqrt(total);
    // c_eff = c * (*cmul): the OSC-TV driver passes TV_constant * d_a with d_a
    // computed on the device (OSC_TV_recon.m:68).
    const double ce = cmul ? (double)c * __ldcg(cmul) : (double)c;
    *norm = m;
    *scale = (float)(-ce / m);
  }
}

template <typename T>
__global__ void __launch_bounds__(kTvBx * kTvBy) tv_update_kernel(
    const T* __restrict__ x, T* __restrict__ y, int Nx, int Ny, int Nz,
    const float* __restrict__ scale) {
  const float a = __ldg(scale);
  const size_t sy = (size_t)Nx, sz = (size_t)Nx * Ny;
  const size_t ci = (size_t)(blockIdx.x * kTvOx + threadIdx.x) +
                    (size_t)(blockIdx.y * kTvOy + threadIdx.y) * sy;
  tv_sweep(x, Nx, Ny, Nz, [&](int z, float xv, float g, bool, bool own) {
    // x <- a*g + x (thrust saxpy, CUDAmex_TVmin_3D.cu:232); border g = 0.
    if (own) stf(y + ci + (size_t)z * sz, fmaf(a, g, xv));
  });
}

// ---------------------------------------------------------------------------
// TV sweep, four x-voxels per thread (FP32 volumes with Nx % 4 == 0 and
// 16-byte aligned pointers).  Same per-voxel arithmetic as tv_sweep, in the
// same order, with every elementwise step done as two packed FP32x2
// operations and each thread's row segment moved by one 16-byte load or
// store: a thread's per-plane cost (loop, barrier, addresses, predicates) is
// shared by four voxels.  A CTA of 32 x 16 threads covers 128 x 16 columns
// and owns 124 x 15 of them: the last lane's four columns and the last row
// give the +x / +y neighbours' terms (the stride of 124 keeps every segment
// 16-byte aligned).  The norm's per-thread FP32 partial covers its 4 x 32
// voxels; everything above is FP64 as in tv_norm_kernel.
// ---------------------------------------------------------------------------
constexpr int kT4Bx = 32, kT4By = 16, kT4Z = 32;
constexpr int kT4Ox = kT4Bx * 4 - 4, kT4Oy = kT4By - 1;  // 124 x 15 outputs

// a - b as one packed fma with -1 (the product is exact, so the result is the
// correctly rounded difference, as a subtraction gives).
__device__ __forceinline__ float2 tv_sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}

// Four voxels as two pairs.
struct V4 {
  float2 lo, hi;
};
__device__ __forceinline__ V4 v4(float4 f) { return V4{make_float2(f.x, f.y), make_float2(f.z, f.w)}; }
__device__ __forceinline__ V4 sub4(V4 a, V4 b) { return V4{tv_sub2(a.lo, b.lo), tv_sub2(a.hi, b.hi)}; }
__device__ __forceinline__ V4 add4(V4 a, V4 b) { return V4{__fadd2_rn(a.lo, b.lo), __fadd2_rn(a.hi, b.hi)}; }
__device__ __forceinline__ V4 mul4(V4 a, V4 b) { return V4{__fmul2_rn(a.lo, b.lo), __fmul2_rn(a.hi, b.hi)}; }
__device__ __forceinline__ V4 fma4(V4 a, V4 b, V4 c) {
  return V4{__ffma2_rn(a.lo, b.lo, c.lo), __ffma2_rn(a.hi, b.hi, c.hi)};
}

// mode 0: ||g||^2 reduction (scale / norm written by the last CTA);
// mode 1: y = x + scale*g for the owned voxels.
template <int MODE>
__global__ void __launch_bounds__(kT4Bx * kT4By, 2) tv4_kernel(
    const float* __restrict__ v, float* __restrict__ yout, int Nx, int Ny, int Nz, float c,
    const double* __restrict__ cmul, double* __restrict__ partials,
    unsigned* __restrict__ counter, float* __restrict__ scale, double* __restrict__ norm,
    const float* __restrict__ scale_in) {
  __shared__ float4 qbs[2][kT4By][kT4Bx];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int gx0 = blockIdx.x * kT4Ox + tx * 4, gy = blockIdx.y * kT4Oy + ty;
  const int z0 = blockIdx.z * kT4Z;
  const int zend = min(z0 + kT4Z, Nz);
  // 32-bit element offsets (the volume holds fewer than 2^31 voxels)
  const int sy = Nx, sz = Nx * Ny;
  const bool incol = gx0 < Nx && gy < Ny;  // Nx % 4 == 0: the whole segment is in range
  const bool own = incol && tx < kT4Bx - 1 && ty < kT4Oy;
  const bool ld_y = incol && gy >= 1, ld_l = incol && tx == 0 && gx0 >= 1;
  const bool row_int = gy >= 1 && gy < Ny - 1;
  // interior columns of the segment as 0/1 masks (g is 0 on the volume border)
  float xin[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) xin[e] = (gx0 + e >= 1 && gx0 + e < Nx - 1 && row_int) ? 1.f : 0.f;
  const V4 xmask{make_float2(xin[0], xin[1]), make_float2(xin[2], xin[3])};
  const float a_upd = MODE == 1 ? __ldg(scale_in) : 0.f;
  const float2 a2 = make_float2(a_upd, a_upd);
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  // offset of the column at plane z0 (the row above and the left neighbour are
  // read only where they exist)
  int oc = gx0 + gy * sy + z0 * sz;
  auto ld4 = [&](int o, bool ok) {
    return ok ? __ldg(reinterpret_cast<const float4*>(v + o)) : z4;
  };
  V4 xprev = v4(ld4(oc - sz, incol && z0 >= 1));
  float4 xc4 = ld4(oc, incol && z0 < Nz);
  float4 xy4 = ld4(oc - sy, ld_y && z0 < Nz);
  float xl = (ld_l && z0 < Nz) ? __ldg(v + oc - 1) : 0.f;
  V4 q0p{}, qap{}, xz{};
  float qa_next = 0.f;  // +x neighbour's qa of the previous plane (lane + 1, element 0)
  float ss = 0.f;
#pragma unroll 1
  for (int p = z0; p <= zend; ++p) {
    // prefetch the next plane
    const int on = oc + sz;
    const bool nxt = p + 1 <= zend && p + 1 < Nz;
    const float4 xn4 = ld4(on, incol && nxt), yn4 = ld4(on - sy, ld_y && nxt);
    const float ln = (ld_l && nxt) ? __ldg(v + on - 1) : 0.f;
    const V4 xc = v4(xc4), xy = v4(xy4);
    // x - 1 of element 0: lane tx-1's element 3 (lane 0 loaded it)
    const float left = __shfl_up_sync(0xffffffffu, xc4.w, 1);
    const V4 xm{make_float2(tx == 0 ? xl : left, xc4.x), make_float2(xc4.y, xc4.z)};
    const V4 a = sub4(xc, xm), b = sub4(xc, xy), cc = sub4(xc, xprev);
    const V4 s2 = fma4(cc, cc, fma4(b, b, mul4(a, a)));
    // |(a,b,c)| = s2 * rsqrt(s2) (0 for s2 = 0: the argument is kept >= FLT_MIN,
    // where eps dominates anyway), r = 1/(eps + |.|), 0 where q does not exist
    const V4 rs{make_float2(rsqrtf(fmaxf(s2.lo.x, 1.17549435e-38f)), rsqrtf(fmaxf(s2.lo.y, 1.17549435e-38f))),
                make_float2(rsqrtf(fmaxf(s2.hi.x, 1.17549435e-38f)), rsqrtf(fmaxf(s2.hi.y, 1.17549435e-38f)))};
    const float2 eps2 = make_float2(1.0e-6f, 1.0e-6f);
    const V4 den{__fadd2_rn(eps2, __fmul2_rn(s2.lo, rs.lo)), __fadd2_rn(eps2, __fmul2_rn(s2.hi, rs.hi))};
    const float qm = (incol && gy >= 1 && p >= 1 && p < Nz) ? 1.f : 0.f;
    const float2 qm2 = make_float2(qm, qm);
    const V4 r{__fmul2_rn(qm2, make_float2(__fdividef(1.0f, den.lo.x), __fdividef(1.0f, den.lo.y))),
               __fmul2_rn(qm2, make_float2(__fdividef(1.0f, den.hi.x), __fdividef(1.0f, den.hi.y)))};
    const V4 q0 = mul4(add4(add4(a, b), cc), r);
    const V4 qa = mul4(a, r), qb = mul4(b, r), qc = mul4(cc, r);
    if (p > z0) {
      // g of plane p - 1 = q0 - qa(x+1) - qb(y+1) - qc(z+1), 0 on the border
      const int z = p - 1;
      const float zm = (z >= 1 && z < Nz - 1) ? 1.f : 0.f;
      const float4 qbb = qbs[(p - 1) & 1][ty + (ty < kT4By - 1)][tx];
      const V4 qan{make_float2(qap.lo.y, qap.hi.x), make_float2(qap.hi.y, qa_next)};
      V4 g = sub4(sub4(sub4(q0p, qan), v4(qbb)), qc);
      const float2 zm2 = make_float2(zm, zm);
      g = V4{__fmul2_rn(__fmul2_rn(g.lo, xmask.lo), zm2), __fmul2_rn(__fmul2_rn(g.hi, xmask.hi), zm2)};
      if (MODE == 0) {
        if (own) {
          ss = fmaf(g.lo.x, g.lo.x, ss);
          ss = fmaf(g.lo.y, g.lo.y, ss);
          ss = fmaf(g.hi.x, g.hi.x, ss);
          ss = fmaf(g.hi.y, g.hi.y, ss);
        }
      } else if (own) {
        const float2 lo = __ffma2_rn(a2, g.lo, xz.lo), hi = __ffma2_rn(a2, g.hi, xz.hi);
        *reinterpret_cast<float4*>(yout + (oc - sz)) = make_float4(lo.x, lo.y, hi.x, hi.y);
      }
    }
    oc = on;
    qbs[p & 1][ty][tx] = make_float4(qb.lo.x, qb.lo.y, qb.hi.x, qb.hi.y);
    qa_next = __shfl_down_sync(0xffffffffu, qa.lo.x, 1);
    q0p = q0;
    qap = qa;
    xz = xc;
    xprev = xc;
    xc4 = xn4;
    xy4 = yn4;
    xl = ln;
    __syncthreads();
  }
  if (MODE == 0) {
    const double blk = block_sum((double)ss);
    double total;
    if (finish_partials(blk, partials, counter, &total)) {
      const double m = sqrt(total);
      const double ce = cmul ? (double)c * __ldg(cmul) : (double)c;
      *norm = m;
      *scale = (float)(-ce / m);
    }
  }
}

static bool tv4_ok(const void* x, const void* y, int xt, int Nx, int Ny, int Nz) {
  return xt == kF32 && Nx % 4 == 0 && ((uintptr_t)x & 15) == 0 && ((uintptr_t)y & 15) == 0 &&
         (long long)Nx * Ny * (Nz + 1) < (1LL << 31);
}

static dim3 tv4_grid(int Nx, int Ny, int Nz) {
  return dim3((Nx + kT4Ox - 1) / kT4Ox, (Ny + kT4Oy - 1) / kT4Oy, (Nz + kT4Z - 1) / kT4Z);
}

static dim3 tv_grid(int Nx, int Ny, int Nz) {
  return dim3((Nx + kTvOx - 1) / kTvOx, (Ny + kTvOy - 1) / kTvOy, (Nz + kTvZ - 1) / kTvZ);
}

size_t tv_partials_needed(int Nx, int Ny, int Nz) {
  // the four-voxel grid never has more CTAs than this one
  const dim3 g = tv_grid(Nx, Ny, Nz);
  return (size_t)g.x * g.y * g.z;
}

bool tv_shape_launchable(int Nx, int Ny, int Nz) {
  const long long gx = ((long long)Nx + kTvOx - 1) / kTvOx;
  const long long gy = ((long long)Ny + kTvOy - 1) / kTvOy, gz = ((long long)Nz + kTvZ - 1) / kTvZ;
  return gx <= 0x7fffffffLL && gy <= 65535 && gz <= 65535;
}

static cudaError_t tv_norm_go(const void* x, int xt, int Nx, int Ny, int Nz, float c,
                              const double* cmul, double* partials, unsigned* counter,
                              float* scale, double* norm, cudaStream_t st) {
  if (tv4_ok(x, x, xt, Nx, Ny, Nz)) {
    tv4_kernel<0><<<tv4_grid(Nx, Ny, Nz), dim3(kT4Bx, kT4By), 0, st>>>(
        (const float*)x, nullptr, Nx, Ny, Nz, c, cmul, partials, counter, scale, norm, nullptr);
    return cudaGetLastError();
  }
  dim3 blk(kTvBx, kTvBy), grd = tv_grid(Nx, Ny, Nz);
  if (xt == kF32)
    tv_norm_kernel<float><<<grd, blk, 0, st>>>((const float*)x, Nx, Ny, Nz, c, cmul,
                                               partials, counter, scale, norm);
  else if (xt == kF16)
    tv_norm_kernel<__half><<<grd, blk, 0, st>>>((const __half*)x, Nx, Ny, Nz, c, cmul,
                                                partials, counter, scale, norm);
  else
    tv_norm_kernel<__nv_bfloat16><<<grd, blk, 0, st>>>(
        (const __nv_bfloat16*)x, Nx, Ny, Nz, c, cmul, partials, counter, scale, norm);
  return cudaGetLastError();
}

cudaError_t launch_tv_norm(const void* x, int xt, int Nx, int Ny, int Nz,
                           float c, double* partials, unsigned* counter,
                           float* scale, double* norm, cudaStream_t st) {
  return tv_norm_go(x, xt, Nx, Ny, Nz, c, nullptr, partials, counter, scale, norm, st);
}

cudaError_t launch_tv_norm_scaled(const void* x, int xt, int Nx, int Ny, int Nz,
                                  float c, const double* cmul, double* partials,
                                  unsigned* counter, float* scale, double* norm,
                                  cudaStream_t st) {
  return tv_norm_go(x, xt, Nx, Ny, Nz, c, cmul, partials, counter, scale, norm, st);
}

cudaError_t launch_tv_update(const void* x, void* y, int xt, int Nx, int Ny,
                             int Nz, const float* scale, cudaStream_t st) {
  if (tv4_ok(x, y, xt, Nx, Ny, Nz)) {
    tv4_kernel<1><<<tv4_grid(Nx, Ny, Nz), dim3(kT4Bx, kT4By), 0, st>>>(
        (const float*)x, (float*)y, Nx, Ny, Nz, 0.f, nullptr, nullptr, nullptr, nullptr, nullptr,
        scale);
    return cudaGetLastError();
  }
  dim3 blk(kTvBx, kTvBy), grd = tv_grid(Nx, Ny, Nz);
  if (xt == kF32)
    tv_update_kernel<float><<<grd, blk, 0, st>>>((const float*)x, (float*)y,
                                                 Nx, Ny, Nz, scale);
  else if (xt == kF16)
    tv_update_kernel<__half><<<grd, blk, 0, st>>>((const __half*)x,
                                                  (__half*)y, Nx, Ny, Nz, scale);
  else
    tv_update_kernel<__nv_bfloat16><<<grd, blk, 0, st>>>(
        (const __nv_bfloat16*)x, (__nv_bfloat16*)y, Nx, Ny, Nz, scale);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ||a - b||^2 in FP64 with NaN differences dropped and, optionally, a[0]
// taken as 0 (OSC_TV_recon.m:45,65-67: mu_old(1) = 0, mu_old(isnan) = 0).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) ssd_kernel(
    const T* __restrict__ a, const T* __restrict__ b, long long n,
    int zero_first, double* partials, unsigned* counter, double* out) {
  double ss = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    const float av = (zero_first && i == 0) ? 0.f : ldf(a + i);
    const float d = av - ldf(b + i);
    if (!isnan(d)) ss += (double)d * (double)d;
  }
  const double blk = block_sum(ss);
  double total;
  if (finish_partials(blk, partials, counter, &total)) *out = sqrt(total);
}

__global__ void __launch_bounds__(1024) sum_partials_kernel(const double* __restrict__ p,
                                                           long long n, double* __restrict__ out) {
  double acc = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) acc += p[i];
  acc = block_sum(acc);
  if (threadIdx.x == 0) *out = acc;
}

cudaError_t launch_sum_partials(const double* partials, long long n, double* out,
                                cudaStream_t st) {
  sum_partials_kernel<<<1, 1024, 0, st>>>(partials, n, out);
  return cudaGetLastError();
}

// Norms of the parts of a volume (z-slabs) combined in index order:
// out = sqrt(sum parts[i]^2); with scale non-null also the TV step scale
// -c * (*cmul) / out, as the last CTA of the norm kernel writes it.
__global__ void combine_norms_kernel(const double* __restrict__ parts, int n,
                                     double* __restrict__ out, float c,
                                     const double* __restrict__ cmul, float* __restrict__ scale) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += parts[i] * parts[i];
  const double m = sqrt(s);
  *out = m;
  if (scale) {
    const double ce = cmul ? (double)c * *cmul : (double)c;
    *scale = (float)(-ce / m);
  }
}

cudaError_t launch_combine_norms(const double* parts, int n, double* out, float c,
                                 const double* cmul, float* scale, cudaStream_t st) {
  combine_norms_kernel<<<1, 1, 0, st>>>(parts, n, out, c, cmul, scale);
  return cudaGetLastError();
}

int device_sms() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    dev = 0;
  }
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n > 0) return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    n = 1;
  }
  cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

size_t ssd_partials_needed() { return (size_t)device_sms() * 4; }

cudaError_t launch_ssd(const void* a, const void* b, int dt, long long n,
                       int zero_first, double* partials, unsigned* counter,
                       double* out, cudaStream_t st) {
  const int blocks = (int)ssd_partials_needed();
  if (dt == kF32)
    ssd_kernel<float><<<blocks, 256, 0, st>>>((const float*)a, (const float*)b,
                                              n, zero_first, partials, counter, out);
  else if (dt == kF16)
    ssd_kernel<__half><<<blocks, 256, 0, st>>>((const __half*)a,
                                               (const __half*)b, n, zero_first,
                                               partials, counter, out);
  else
    ssd_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(
        (const __nv_bfloat16*)a, (const __nv_bfloat16*)b, n, zero_first,
        partials, counter, out);
  return cudaGetLastError();
}

template <typename T>
__global__ void finite_kernel(T* x, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    const float v = ldp(x + i);
    if (!isfinite(v)) stf(x + i, 0.f);
  }
}

cudaError_t launch_finite(void* x, int dt, long long n, cudaStream_t st) {
  const int blocks = device_sms() * 8;
  if (dt == kF32) finite_kernel<float><<<blocks, 256, 0, st>>>((float*)x, n);
  else if (dt == kF16) finite_kernel<__half><<<blocks, 256, 0, st>>>((__half*)x, n);
  else finite_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>((__nv_bfloat16*)x, n);
  return cudaGetLastError();
}

template <typename T>
__global__ void fill_kernel(T* x, long long n, float v) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride)
    stf(x + i, v);
}

cudaError_t launch_fill(void* x, int dt, long long n, float v,
                        cudaStream_t st) {
  const int blocks = device_sms() * 8;
  if (dt == kF32) fill_kernel<float><<<blocks, 256, 0, st>>>((float*)x, n, v);
  else if (dt == kF16) fill_kernel<__half><<<blocks, 256, 0, st>>>((__half*)x, n, v);
  else fill_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>((__nv_bfloat16*)x, n, v);
  return cudaGetLastError();
}

// OSC_TV_recon.m:35-37: x(x < eps) = eps (NaN stays NaN, as in MATLAB).
__global__ void clamp_copy_kernel(const float* __restrict__ s, float* __restrict__ d,
                                  long long n, float eps) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float v = s[i];
    d[i] = (v < eps) ? eps : v;
  }
}

cudaError_t launch_clamp_copy(const float* src, float* dst, long long n, float eps,
                              cudaStream_t st) {
  clamp_copy_kernel<<<device_sms() * 8, 256, 0, st>>>(src, dst, n, eps);
  return cudaGetLastError();
}

// Largest finite value of n FP32 values as an order-preserving integer key
// (atomicMax on the bits of a non-negative float orders like the float; a
// negative or NaN value counts as 0).  *out must start at 0.
__global__ void max_nonneg_kernel(const float* __restrict__ x, long long n,
                                  unsigned* __restrict__ out) {
  unsigned m = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float v = x[i];
    if (v > 0.f && v <= 3.4028235e38f) m = max(m, __float_as_uint(v));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

cudaError_t launch_max_nonneg(const float* x, long long n, unsigned* out, cudaStream_t st) {
  max_nonneg_kernel<<<device_sms() * 8, 256, 0, st>>>(x, n, out);
  return cudaGetLastError();
}

template <typename S, typename D>
__global__ void convert_kernel(const S* __restrict__ s, D* __restrict__ d,
                               long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride)
    stf(d + i, ldp(s + i));
}

cudaError_t launch_convert(const void* src, int st_, void* dst, int dt,
                           long long n, cudaStream_t st) {
  const int blocks = device_sms() * 8;
#define CV(SA, DA) convert_kernel<SA, DA><<<blocks, 256, 0, st>>>((const SA*)src, (DA*)dst, n)
  if (st_ == kF32 && dt == kF16) CV(float, __half);
  else if (st_ == kF32 && dt == kBF16) CV(float, __nv_bfloat16);
  else if (st_ == kF16 && dt == kF32) CV(__half, float);
  else if (st_ == kBF16 && dt == kF32) CV(__nv_bfloat16, float);
  else if (st_ == kF32 && dt == kF32) CV(float, float);
  else return cudaErrorInvalidValue;
#undef CV
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FDK/FBP pre-filter: per detector row, the cosine weight
// (preFilterSinogram.m:38-57, 1-based U/V as written), the Parker window of
// the row element (parker_weight.m:216-226, a host-built [nP, W] table), the
// zero-padded ramp x window filter as a direct linear convolution with the
// spatial kernel real(ifft(H)) (preFilterSinogram.m:72-78: padding to
// order >= 2W makes the circular convolution linear), and the dbeta/2 factor
// (:80-84).  Optional FBP_recon.m:26-28 log transform on load.
// ---------------------------------------------------------------------------
constexpr int kFiltRows = 4;

__global__ void __launch_bounds__(256) prefilter_kernel(
    const FiltArgs A, const float* __restrict__ sino,
    const float* __restrict__ pre, const float* __restrict__ parker,
    const float* __restrict__ dbeta, const float* __restrict__ kern,
    float* __restrict__ out) {
  extern __shared__ float sm[];
  float* ks = sm;                       // order
  float* xs = sm + A.order;             // kFiltRows * W
  const int view = blockIdx.y;
  const int v0 = blockIdx.x * kFiltRows;
  const int W = A.W, H = A.H;
  for (int i = threadIdx.x; i < A.order; i += blockDim.x) ks[i] = __ldg(kern + i);
  const size_t vbase = (size_t)view * W * H;
  const float db = __ldg(dbeta + view);
  for (int r = 0; r < kFiltRows; ++r) {
    const int v = v0 + r;
    for (int u = threadIdx.x; u < W; u += blockDim.x) {
      float w = 0.f;
      if (v < H) {
        const size_t gi = vbase + (size_t)v * W + u;
        float s = __ldg(sino + gi);
        if (A.log_input) {
          s = -logf(s / __ldg(pre + gi));
          if (!isfinite(s)) s = 0.f;
        }
        const float U = (float)(u + 1) - (float)(W - 1) * 0.5f;
        const float V = (float)(v + 1) - (float)(H - 1) * 0.5f;
        if (A.geom == 1) s *= A.sad / sqrtf(A.sad * A.sad + U * U);
        if (A.geom == 2) s *= A.sad / sqrtf(A.sad * A.sad + U * U + V * V);
        w = s * __ldg(parker + (size_t)view * W + u);
      }
      xs[r * W + u] = w;
    }
  }
  __syncthreads();
  const int mask = A.order - 1;
  for (int u = threadIdx.x; u < W; u += blockDim.x) {
    float acc[kFiltRows];
#pragma unroll
    for (int r = 0; r < kFiltRows; ++r) acc[r] = 0.f;
    for (int j = 0; j < W; ++j) {
      const float k = ks[(u - j) & mask];
#pragma unroll
      for (int r = 0; r < kFiltRows; ++r) acc[r] = fmaf(xs[r * W + j], k, acc[r]);
    }
#pragma unroll
    for (int r = 0; r < kFiltRows; ++r) {
      const int v = v0 + r;
      if (v < H) out[vbase + (size_t)v * W + u] = acc[r] * db;
    }
  }
}

// Weighted input sample of the pre-filter (log transform, cosine weight,
// Parker weight), as prefilter_kernel stages it.
__device__ __forceinline__ float prefilter_input(const FiltArgs& A, const float* __restrict__ sino,
                                                 const float* __restrict__ pre,
                                                 const float* __restrict__ parker, int view,
                                                 int v, int u) {
  const size_t gi = ((size_t)view * A.H + v) * A.W + u;
  float s = __ldg(sino + gi);
  if (A.log_input) {
    s = -logf(s / __ldg(pre + gi));
    if (!isfinite(s)) s = 0.f;
  }
  const float U = (float)(u + 1) - (float)(A.W - 1) * 0.5f;
  const float V = (float)(v + 1) - (float)(A.H - 1) * 0.5f;
  if (A.geom == 1) s *= A.sad / sqrtf(A.sad * A.sad + U * U);
  if (A.geom == 2) s *= A.sad / sqrtf(A.sad * A.sad + U * U + V * V);
  return s * __ldg(parker + (size_t)view * A.W + u);
}

// Register-blocked form of prefilter_kernel: a block filters 8*RG detector
// rows of one view, each thread 8 rows x 8 consecutive columns.  The rows are
// staged in shared memory (zero-padded to a multiple of 8 columns); the
// thread keeps the 15 kernel taps k[(u0 - j0 - 7 + m) & mask] its 8 columns
// need for 8 consecutive j in registers, so 64 FMAs take 8 row loads
// (broadcasts) and 15/8 tap loads.  Each output is the same FMA chain over
// j = 0 .. W-1 as in prefilter_kernel: the results are bit-identical.
template <int RG>
__global__ void __launch_bounds__(256) prefilter_tiled_kernel(
    const FiltArgs A, const float* __restrict__ sino, const float* __restrict__ pre,
    const float* __restrict__ parker, const float* __restrict__ dbeta,
    const float* __restrict__ kern, float* __restrict__ out) {
  constexpr int ROWS = 8 * RG, UG = 256 / RG;  // rows per block, column groups
  extern __shared__ float sm[];
  const int W = A.W, H = A.H, Wj = (W + 7) & ~7;
  float* ks = sm;            // order (circular kernel)
  float* xs = sm + A.order;  // ROWS x Wj, row-major
  const int view = blockIdx.y;
  const int v0 = blockIdx.x * ROWS;
  for (int i = threadIdx.x; i < A.order; i += 256) ks[i] = __ldg(kern + i);
  for (int i = threadIdx.x; i < ROWS * Wj; i += 256) {
    const int r = i / Wj, j = i - r * Wj, v = v0 + r;
    xs[i] = (v < H && j < W) ? prefilter_input(A, sino, pre, parker, view, v, j) : 0.f;
  }
  __syncthreads();
  const int mask = A.order - 1;
  const int ug = threadIdx.x % UG, rg = threadIdx.x / UG;
  const float* xr = xs + (size_t)rg * 8 * Wj;
  const float db = __ldg(dbeta + view);
  for (int u0 = 8 * ug; u0 < W; u0 += 8 * UG) {
    float acc[8][8];
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
      for (int i = 0; i < 8; ++i) acc[r][i] = 0.f;
    for (int j0 = 0; j0 < Wj; j0 += 8) {
      float kw[15];
#pragma unroll
      for (int m = 0; m < 15; ++m) kw[m] = ks[(u0 - j0 - 7 + m) & mask];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        float x[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) x[r] = xr[r * Wj + j0 + jj];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float k = kw[i - jj + 7];  // k[(u0 + i - j) & mask]
#pragma unroll
          for (int r = 0; r < 8; ++r) acc[r][i] = fmaf(x[r], k, acc[r][i]);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int v = v0 + rg * 8 + r;
      if (v >= H) continue;
      float* o = out + ((size_t)view * H + v) * W;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (u0 + i < W) o[u0 + i] = acc[r][i] * db;
    }
  }
}

template <int RG>
static cudaError_t prefilter_tiled_go(const FiltArgs& a, size_t smem, const float* sino,
                                      const float* pre, const float* parker, const float* dbeta,
                                      const float* kern, float* out, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(prefilter_tiled_kernel<RG>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grd((a.H + 8 * RG - 1) / (8 * RG), a.nP);
  prefilter_tiled_kernel<RG><<<grd, 256, smem, st>>>(a, sino, pre, parker, dbeta, kern, out);
  return cudaGetLastError();
}

cudaError_t launch_prefilter(const FiltArgs& a, const float* sino,
                             const float* pre, const float* parker,
                             const float* dbeta, const float* kern, float* out,
                             cudaStream_t st) {
  // register-blocked form with the most rows per block whose rows and kernel
  // fit 200 KB of shared memory
  const size_t Wj = (size_t)((a.W + 7) & ~7);
  for (int rg : {4, 2, 1}) {
    const size_t smem = sizeof(float) * ((size_t)a.order + (size_t)8 * rg * Wj);
    if (smem > 200 * 1024) continue;
    if (rg == 4) return prefilter_tiled_go<4>(a, smem, sino, pre, parker, dbeta, kern, out, st);
    if (rg == 2) return prefilter_tiled_go<2>(a, smem, sino, pre, parker, dbeta, kern, out, st);
    return prefilter_tiled_go<1>(a, smem, sino, pre, parker, dbeta, kern, out, st);
  }
  dim3 grd((a.H + kFiltRows - 1) / kFiltRows, a.nP);
  const size_t smem = sizeof(float) * ((size_t)a.order + (size_t)kFiltRows * a.W);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(
        prefilter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  prefilter_kernel<<<grd, 256, smem, st>>>(a, sino, pre, parker, dbeta, kern, out);
  return cudaGetLastError();
}

}  // namespace mexct
