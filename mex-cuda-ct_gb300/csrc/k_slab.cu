// k_slab.cu -- slab-staged forward projection with TMA for the standard
// geometries (CUDAmex_FP.cu:56-346) and the OSC forward pass
// (CUDAmex_oscIter.cu:140-271).
//
// Why: a ray-per-thread march that fetches its 8 trilinear taps through L1
// issues ~28 L1 wavefronts per warp-sample, because the 32 rays of a warp
// enter the volume through different faces and are spread along the ray
// direction.  Here a CTA (32 x 8 detector pixels of one view) sweeps the
// volume along the view's dominant axis a (x or y) in slabs of SlabCfg::T tap
// planes.  Before the sweep the whole CTA plans every slab at once: the
// bounding box of the tile's ray bundle in the slab, from the 4 corner rays
// (the coordinates across a plane are monotone in the detector coordinates).
// During the sweep one thread starts the TMA copy of the next slab's box from
// a padded volume into shared memory ([z][a][f] with f fastest) and every
// lane takes its samples whose a-tap lies in the slab from shared memory with
// constant-offset loads.  Two buffers and two mbarriers overlap the copy of
// slab j+1 with the sampling of slab j.  Shapes (measured on cone 512^3 x
// 720): 4 taps per slab, boxes of 64 (f) x 5 (a) x <=20 (z) elements that
// hold 99.9% of the bundles, copied as one 20-row box per slab (2-, 4-, 5-
// and 10-row boxes for the rows the bundle needs were 1-5% slower: the
// issuing thread stalls its warp), 4 CTAs of 256 threads per SM (<=64
// registers, 50 KB of buffers each); 3 taps (4 or 5 CTAs/SM) and 2 taps
// (5 CTAs/SM) were 12-32% slower.  Planning all slabs up front instead of one
// slab ahead in warp 0 took 15% off the sweep.
//
// The padded volume has a one-voxel border (replicated edge for clamp
// addressing, zeros for border addressing) and a fast-axis pitch rounded up
// to 8 elements, so taps never need clamping and every TMA box starts on a
// 16-byte boundary.  A slab whose bundle does not fit the box falls back to
// loads from the padded volume in global memory.
//
// Samples are the reference's: p_k = entry + k*step*dir for k < n with the
// binary32 ray set-up of geom.cuh; only the order in which a thread visits
// its samples is unchanged (increasing k), the accumulation is FP32.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "kernels.h"

namespace mexct {

// ---------------------------------------------------------------------------
// Padded volumes.
// ---------------------------------------------------------------------------
template <typename T>
// border: bit 0 zero frame everywhere (border addressing), bit 1 / bit 2 zero
// frame below / above the z range only (inner faces of a sub-volume slab).
__global__ void __launch_bounds__(256) pad_x_kernel(const T* __restrict__ src,
                                                    T* __restrict__ dst, int W,
                                                    int H, int Pf, int border) {
  const int xp = blockIdx.x * 32 + threadIdx.x;
  const int yp = blockIdx.y * 8 + threadIdx.y;
  const int zp = blockIdx.z;
  const int Ps = W + 2;
  if (xp >= Pf || yp >= Ps) return;
  float v = 0.f;
  if (xp < Ps) {
    int x = xp - 1, y = yp - 1, z = zp - 1;
    const bool out = x < 0 || x >= W || y < 0 || y >= W || z < 0 || z >= H;
    const bool zero = ((border & 1) && out) || ((border & 2) && z < 0) || ((border & 4) && z >= H);
    if (!zero) {
      x = min(max(x, 0), W - 1);
      y = min(max(y, 0), W - 1);
      z = min(max(z, 0), H - 1);
      v = ldf(src + (size_t)x + (size_t)W * ((size_t)y + (size_t)W * z));
    }
  }
  stf(dst + (size_t)xp + (size_t)Pf * ((size_t)yp + (size_t)Ps * zp), v);
}

template <typename T>
__global__ void __launch_bounds__(256) pad_transpose_kernel(
    const T* __restrict__ px, T* __restrict__ py, int Ps, int Pf) {
  __shared__ float tile[32][33];
  const size_t zoff = (size_t)blockIdx.z * Pf * Ps;
  const int a0 = blockIdx.x * 32, b0 = blockIdx.y * 32;  // a: x, b: y
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int x = a0 + threadIdx.x, y = b0 + j;
    tile[j][threadIdx.x] = (x < Pf && y < Ps) ? ldp(px + zoff + (size_t)y * Pf + x) : 0.f;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int y = b0 + threadIdx.x, x = a0 + j;
    if (y < Pf && x < Ps) stf(py + zoff + (size_t)x * Pf + y, (y < Ps) ? tile[threadIdx.x][j] : 0.f);
  }
}

// Batched padding: one CTA per (problem, padded z slice, 32 x 32 tile) writes
// both padded layouts of the tile (clamp addressing).
__global__ void __launch_bounds__(256) pad_batch_kernel(const BatchFp* __restrict__ probs,
                                                        int nprob, long long total) {
  __shared__ float tile[32][33];
  const long long item = blockIdx.x;
  if (item >= total) return;
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].pad_item0 <= item) lo = mid;
    else hi = mid - 1;
  }
  const BatchFp& B = probs[lo];
  const int W = B.W, H = B.H, Pf = B.Pf, Ps = W + 2;
  const int nt = (Pf + 31) / 32;
  const long long r = item - B.pad_item0;
  const int zp = (int)(r / ((long long)nt * nt));
  const int t = (int)(r % ((long long)nt * nt));
  const int x0 = (t % nt) * 32, y0 = (t / nt) * 32;
  const float* src = static_cast<const float*>(B.vol);
  float* px = static_cast<float*>(const_cast<void*>(B.px));
  float* py = static_cast<float*>(const_cast<void*>(B.py));
  const size_t zoff = (size_t)zp * Pf * Ps;
  const int z = min(max(zp - 1, 0), H - 1);
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int xp = x0 + threadIdx.x, yp = y0 + j;
    float v = 0.f;
    if (xp < Ps && yp < Ps) {
      const int x = min(max(xp - 1, 0), W - 1), y = min(max(yp - 1, 0), W - 1);
      v = __ldg(src + (size_t)x + (size_t)W * ((size_t)y + (size_t)W * z));
    }
    tile[j][threadIdx.x] = v;
    if (xp < Pf && yp < Ps) px[zoff + (size_t)yp * Pf + xp] = v;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int yp = y0 + threadIdx.x, xp = x0 + j;
    if (yp < Pf && xp < Ps) py[zoff + (size_t)xp * Pf + yp] = tile[threadIdx.x][j];
  }
}

cudaError_t launch_pad_batch(const BatchFp* d_probs, int nprob, long long total,
                             cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  if (total > 0x7fffffffLL) return cudaErrorInvalidValue;
  pad_batch_kernel<<<(unsigned)total, dim3(32, 8), 0, st>>>(d_probs, nprob, total);
  return cudaGetLastError();
}

cudaError_t launch_pad_volume(const void* src, int dtype, int W, int H, int Pf,
                              bool border, void* px, void* py, cudaStream_t st) {
  const int Ps = W + 2, Pz = H + 2;
  dim3 blk(32, 8), g1((Pf + 31) / 32, (Ps + 7) / 8, Pz);
  dim3 g2((Pf + 31) / 32, (Pf + 31) / 32, Pz);
#define PAD(T)                                                                        \
  pad_x_kernel<T><<<g1, blk, 0, st>>>((const T*)src, (T*)px, W, H, Pf, border ? 1 : 0); \
  pad_transpose_kernel<T><<<g2, blk, 0, st>>>((const T*)px, (T*)py, Ps, Pf)
  if (dtype == kF32) {
    PAD(float);
  } else if (dtype == kF16) {
    PAD(__half);
  } else {
    PAD(__nv_bfloat16);
  }
#undef PAD
  return cudaGetLastError();
}

cudaError_t launch_pad_volume_sub(const float* src, int W, int nz, int Pf, bool zero_lo,
                                  bool zero_hi, float* px, float* py, cudaStream_t st,
                                  bool border) {
  const int Ps = W + 2, Pz = nz + 2;
  dim3 blk(32, 8), g1((Pf + 31) / 32, (Ps + 7) / 8, Pz);
  dim3 g2((Pf + 31) / 32, (Pf + 31) / 32, Pz);
  const int mode = border ? 1 : ((zero_lo ? 2 : 0) | (zero_hi ? 4 : 0));
  pad_x_kernel<float><<<g1, blk, 0, st>>>(src, px, W, nz, Pf, mode);
  pad_transpose_kernel<float><<<g2, blk, 0, st>>>(px, py, Ps, Pf);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// TMA / mbarrier helpers (inline PTX).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1,
                                            int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Non-blocking test of a phase (try_wait may suspend the thread for a while).
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// After a CTA gave up waiting: copies issued before still land in its
// buffers, so wait (at most 2 s each) until the last copy issued into each
// buffer has completed.  Copies into one buffer complete in order, so the
// last one's phase parity is (count - 1) & 1.  issued: 16-bit counts per
// buffer.  Kept out of line: it only runs after a failure.
__device__ __noinline__ void slab_drain(uint64_t* bar, uint32_t issued, unsigned* err) {
  for (int b = 0; b < 2; ++b) {
    const uint32_t n = (issued >> (16 * b)) & 0xffffu;
    if (n == 0) continue;
    const uint64_t t0 = global_ns();
    bool done = false;
    do {
      done = mbar_try_wait(&bar[b], (n - 1u) & 1u);
    } while (!done && global_ns() - t0 < 2000000000ull);
    if (!done && err) atomicOr(err, 2u);
  }
}

// Bounded wait: after one attempt, keeps trying for at most wait_us
// microseconds of wall time (default 2 s; < 0: one non-blocking test only), then records the
// failure in err and in the CTA's abort flag and reports it to the caller,
// which samples the slab from global memory instead (the result is the same).
// Once a CTA has given up, its later waits return at once and no further
// copies are issued, so a broken pipeline costs one time-out per CTA.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned* err,
                                                  volatile int* abort, int wait_us) {
  if (*abort) return false;
  if (wait_us < 0) {
    if (mbar_test_wait(bar, parity)) return true;
  } else {
    // the usual short waits end here, without reading the clock
    for (int i = 0; i < 64; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    const uint64_t limit = wait_us > 0 ? (uint64_t)wait_us * 1000ull : 2000000000ull;
    const uint64_t t0 = global_ns();
    while (global_ns() - t0 < limit)
      if (mbar_try_wait(bar, parity)) return true;
  }
  *abort = 1;
  if (err) atomicOr(err, 1u);
  return false;
}

// ---------------------------------------------------------------------------
// Slab kernel.
// ---------------------------------------------------------------------------
constexpr int kSlabCtas = 4;                  // resident CTAs per SM (launch bounds)
// Slab shape per projection geometry: F x A x Z boxes (f extent, a-planes =
// taps + 1, z rows).  Cone rays spread in z along a slab, so cone slabs are 5
// taps thick in 18-row boxes; par / fan rays keep their z (an 8-row tile spans
// 8 rows), so their slabs are 8 taps thick in 12-row boxes: fewer slabs per
// ray, less per-slab work.  Measured at 512^3 x 720: cone 187.0 -> 180.8 ms,
// par 202.6 -> 173.9 ms against 4 taps in 20 rows for both.  One box fills a
// buffer; the buffers are sized for the larger shape, so the batched kernel
// has one shared-memory size for every geometry.
constexpr int kConeF = 64, kConeT = 5, kConeZ = 18;
constexpr int kParF = 64, kParT = 8, kParZ = 12;
template <int GEOM>
struct SlabCfg {
  static constexpr int F = GEOM >= 2 ? kConeF : kParF;   // box extent along f
  static constexpr int T = GEOM >= 2 ? kConeT : kParT;   // a-taps per slab
  static constexpr int A = T + 1;                        // a-planes in a box
  static constexpr int Z = GEOM >= 2 ? kConeZ : kParZ;   // z rows per box (and buffer)
  static constexpr int Plane = A * F;                    // elements per z row of a buffer
  static constexpr int BufElems = Z * Plane;             // elements of a box
  static constexpr int MaxIdx = BufElems - 1 - (Plane + F + 1);
  static constexpr int MaxPlans = 2048 / T;              // planned slabs per tile
  // A TMA box row must be whole 16-byte units and a TMA destination in shared
  // memory 128-byte aligned (both buffers start on a multiple of 128 bytes for
  // 2- and 4-byte types); nzr is packed in 5 bits.
  static_assert((F * 2) % 16 == 0, "box rows must be whole 16-byte units");
  static_assert(Z < 32, "nzr must fit 5 bits");
};
constexpr int cmax(int a, int b) { return a > b ? a : b; }
// elements per buffer: the larger box, rounded to 64 elements (128 bytes)
constexpr int kBufElems = (cmax(SlabCfg<2>::BufElems, SlabCfg<0>::BufElems) + 63) / 64 * 64;
constexpr int kMaxPlans = cmax(SlabCfg<2>::MaxPlans, SlabCfg<0>::MaxPlans);

struct SlabPlan {
  int alo, ahi;  // a-taps sampled in this slab
  int a0;        // first a-plane in the buffer (= alo)
  int f0, z0;    // first f column / z row in the buffer
  int fb;        // 1: sample from global memory
};

int slab_ctas_per_sm() { return kSlabCtas; }

size_t slab_smem_bytes(int dtype) {
  return 2 * (size_t)kBufElems * (dtype == kF32 ? 4 : 2) + 256;
}

template <typename T>
__device__ __forceinline__ float ld_any(const T* p) {
  return ldp(p);
}

// One trilinear (or, with Z2 = false, bilinear in the a/f plane) sample at
// tap-space coordinates ta/tf/tz from a [z][a][f] array with strides.
template <bool Z2, typename T>
__device__ __forceinline__ float sample_at(const T* base, int sa, int sz, float wa,
                                           float wf, float wz) {
  const float v00 = ld_any(base), v01 = ld_any(base + 1);
  const float v10 = ld_any(base + sa), v11 = ld_any(base + sa + 1);
  const float r0 = fmaf(wf, v01 - v00, v00);
  const float r1 = fmaf(wf, v11 - v10, v10);
  const float s0 = fmaf(wa, r1 - r0, r0);
  if (!Z2) return s0;
  const T* b = base + sz;
  const float u00 = ld_any(b), u01 = ld_any(b + 1);
  const float u10 = ld_any(b + sa), u11 = ld_any(b + sa + 1);
  const float q0 = fmaf(wf, u01 - u00, u00);
  const float q1 = fmaf(wf, u11 - u10, u10);
  const float s1 = fmaf(wa, q1 - q0, q0);
  return fmaf(wz, s1 - s0, s0);
}

// sample_at for a sub-volume slab from global memory: z rows r and r + 1 of
// a tensor of zrows rows, a row outside it reading as zeros (what a TMA copy
// fills there), with sample_at's operations.
template <bool Z2, typename T>
__device__ __forceinline__ float sample_rows(const T* col, int r, int zrows, int sa, int sz,
                                             float wa, float wf, float wz) {
  float s0 = 0.f, s1 = 0.f;
  if (r >= 0 && r < zrows) {
    const T* b = col + (size_t)r * sz;
    const float v00 = ld_any(b), v01 = ld_any(b + 1);
    const float v10 = ld_any(b + sa), v11 = ld_any(b + sa + 1);
    const float r0 = fmaf(wf, v01 - v00, v00);
    const float r1 = fmaf(wf, v11 - v10, v10);
    s0 = fmaf(wa, r1 - r0, r0);
  }
  if (!Z2) return s0;
  if (r + 1 >= 0 && r + 1 < zrows) {
    const T* b = col + (size_t)(r + 1) * sz;
    const float u00 = ld_any(b), u01 = ld_any(b + 1);
    const float u10 = ld_any(b + sa), u11 = ld_any(b + sa + 1);
    const float q0 = fmaf(wf, u01 - u00, u00);
    const float q1 = fmaf(wf, u11 - u10, u10);
    s1 = fmaf(wa, q1 - q0, q0);
  }
  return fmaf(wz, s1 - s0, s0);
}

// a - b on both lanes of a packed FP32x2 pair (one sub.rn.f32x2).
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  float2 d;
  asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
      " sub.rn.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

// Two samples at once (x: sample k, y: sample k+1) with every lerp a packed
// FP32x2 subtract + fma: per sample the same IEEE operations in the same
// order as sample_at, so each lane's result is bit-identical to it.
template <bool Z2, typename T>
__device__ __forceinline__ float2 sample_pair(const T* p0, const T* p1, int sa, int sz,
                                              float2 wa, float2 wf, float2 wz) {
  const float2 A = make_float2(ld_any(p0), ld_any(p1));
  const float2 B = make_float2(ld_any(p0 + 1), ld_any(p1 + 1));
  const float2 C = make_float2(ld_any(p0 + sa), ld_any(p1 + sa));
  const float2 D = make_float2(ld_any(p0 + sa + 1), ld_any(p1 + sa + 1));
  const float2 r0 = __ffma2_rn(wf, sub2(B, A), A);
  const float2 r1 = __ffma2_rn(wf, sub2(D, C), C);
  const float2 s0 = __ffma2_rn(wa, sub2(r1, r0), r0);
  if (!Z2) return s0;
  const T* q0 = p0 + sz;
  const T* q1 = p1 + sz;
  const float2 E = make_float2(ld_any(q0), ld_any(q1));
  const float2 F = make_float2(ld_any(q0 + 1), ld_any(q1 + 1));
  const float2 G = make_float2(ld_any(q0 + sa), ld_any(q1 + sa));
  const float2 H = make_float2(ld_any(q0 + sa + 1), ld_any(q1 + sa + 1));
  const float2 u0 = __ffma2_rn(wf, sub2(F, E), E);
  const float2 u1 = __ffma2_rn(wf, sub2(H, G), G);
  const float2 s1 = __ffma2_rn(wa, sub2(u1, u0), u0);
  return __ffma2_rn(wz, sub2(s1, s0), s0);
}

// Geometry of one slab job: a 32 x 8 detector tile of one view.
struct SlabJob {
  int det_w, det_h, S, Z, Pf;
  float u0, v0, bx, by, bz, SR, RD, step;
  float du, dv, ou, ov;  // detector pitch and sub-pixel ray offset
  int zoff, zrows, accum;  // sub-volume slab (RayArgs)
  float zlo, zhi;
  const float* pts;        // general3D: ray end points of this view (6 planes of P)
  Trig tr[2];       // the job's views (nv of them; general3D: one)
  int nv;
  long long P;         // detector pixels per view
  long long gview[2];  // sinogram / pre / post slot of each view
  long long lview[2];  // residual slot of each view (OSC epilogue)
  int tu0, tv0;     // tile origin on the detector
  const CUtensorMap* tmx;
  const CUtensorMap* tmy;
  const void* px;
  const void* py;
  void* out;
};

// Packed slab plan: f0/4 (bits 0-13), z0 (bits 14-26) and the box's z rows
// nzr (bits 27-31) in the padded volume; nzr = 0 means "sample the slab from
// global memory".  Plans are computed for the first kMaxPlans slabs of a tile
// (an a-extent of 2048 taps, W <= ~2040); later slabs of larger volumes, and
// boxes beyond f0 = 65532 or z0 = 8191, read global memory.
constexpr uint32_t kPlanFallback = 0u;

__device__ __forceinline__ uint32_t pack_plan(int f0, int z0, int nzr) {
  return ((uint32_t)f0 >> 2) | ((uint32_t)z0 << 14) | ((uint32_t)nzr << 27);
}
__device__ __forceinline__ int plan_f0(uint32_t p) { return (int)(p & 0x3fffu) << 2; }
__device__ __forceinline__ int plan_z0(uint32_t p) { return (int)((p >> 14) & 0x1fffu); }
__device__ __forceinline__ int plan_nzr(uint32_t p) { return (int)(p >> 27); }

struct SlabShared {
  uint64_t bar[2];
  uint32_t plans[kMaxPlans];
  float corner[8][6];  // corner rays of a tile: four per view
  int gbi[8];         // general3D: ray bounds over the tile, order-preserving int keys
  int amin, amax, pos, neg;
  int abort;          // set by a timed-out wait
  long long item;
};

__device__ __forceinline__ void slab_init_barriers(SlabShared& S) {
  if (threadIdx.x + 32 * threadIdx.y == 0) {
    mbar_init(&S.bar[0], 1);
    mbar_init(&S.bar[1], 1);
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// Per-ray state of a tile's sweep: tap-space entry point and step, par / fan
// z row and weight, next sample, end, accumulator.
struct RayLane {
  float ta0, tf0, tz0, da, df, dz;
  float fzc, wzc;  // par / fan: the ray's z tap row and its weight
  int k, n;
  float acc;
  bool valid;
};

// Ray of detector pixel (ix, iy) in tap space (padded texture coordinate
// minus 0.5, i.e. world - b + 0.5) with its first sample and sample count.
// ZL (decoupled detector): a ray that misses the volume samples nothing.
// SUB: only the k whose z taps can reach the slab's rows.  GEOM 3: the k whose
// taps can touch the padded volume.
template <int GEOM, bool ZL, bool SUB>
__device__ __forceinline__ void ray_setup(const SlabJob& J, const Trig tr, bool view_ok, int ix,
                                          int iy, bool xdom, int Ps, int Pz, RayLane& L,
                                          float s[3], float e[3]) {
  L.valid = view_ok && ix < J.det_w && iy < J.det_h;
  if constexpr (GEOM == 3) {
    const long long pix = (long long)min(iy, J.det_h - 1) * J.det_w + min(ix, J.det_w - 1);
    g3d_ray(J.pts, pix, J.P, tr.s, tr.c, s, e);
  } else {
    std_ray<GEOM>(min(ix, J.det_w - 1), min(iy, J.det_h - 1), J.u0, J.v0, tr.s, tr.c, J.SR,
                  J.RD, s, e, J.du, J.dv, J.ou, J.ov);
  }
  const Ray r = clip_ray(s[0], s[1], s[2], e[0], e[1], e[2], J.bx, J.by, J.bz, J.step);
  const float ca = xdom ? r.cx - J.bx : r.cy - J.by;
  const float cf = xdom ? r.cy - J.by : r.cx - J.bx;
  const float ta0 = ca + 0.5f, tf0 = cf + 0.5f, tz0 = (r.cz - J.bz) + 0.5f;
  const float da = xdom ? r.dx : r.dy, df = xdom ? r.dy : r.dx, dz = r.dz;
  const bool miss = ZL && !hits_box(s, e, J.bx, J.by, J.bz);
  int n = (L.valid && !miss) ? r.n : 0;
  int k0 = 0;  // first sample
  if (SUB && n > 0) {
    // Samples with tz in [zlo, zhi) can touch the slab's rows; the others
    // read zeros only.  The range is widened by one sample each way, so
    // rounding can only add samples that contribute exact zeros.
    if (dz == 0.f) {
      if (!(tz0 >= J.zlo && tz0 < J.zhi)) n = 0;
    } else {
      const float ka = (J.zlo - tz0) / dz, kb = (J.zhi - tz0) / dz;
      const float lim = (float)n + 2.0f;
      const float kmin = fminf(fmaxf(fminf(ka, kb), -2.0f), lim);
      const float kmax = fminf(fmaxf(fmaxf(ka, kb), -2.0f), lim);
      k0 = max((int)floorf(kmin) - 1, 0);
      n = min((int)ceilf(kmax) + 2, n);
      if (k0 >= n) {
        k0 = 0;
        n = 0;
      }
    }
  }
  if (GEOM == 3 && n > 0) {
    // general3D rays are not clipped when they miss the volume (the
    // reference marches them between two points outside it): keep the
    // samples whose taps can touch the padded volume, floor(t) in [0, P-2]
    // on every axis.  With border addressing (zero frame) every other sample
    // reads only zeros, so the sum is unchanged.  The samples kept are an
    // interval of k; the estimates are settled with the loop's own positions.
    const float Pa = (float)(Ps - 1), Pff = (float)(Ps - 1), Pzz = (float)(Pz - 1);
    auto inside = [&](int k) {
      const float kf = (float)k;
      const float ta = fmaf(kf, da, ta0), tf = fmaf(kf, df, tf0), tz = fmaf(kf, dz, tz0);
      return ta >= 0.f && ta < Pa && tf >= 0.f && tf < Pff && tz >= 0.f && tz < Pzz;
    };
    float klo = 0.f, khi = (float)n;
    auto clampk = [&](float t0, float d, float hi) {
      if (d == 0.f) {
        if (!(t0 >= 0.f && t0 < hi)) khi = -1.f;
      } else {
        const float k1 = (0.f - t0) / d, k2 = (hi - t0) / d;
        klo = fmaxf(klo, fminf(k1, k2));
        khi = fminf(khi, fmaxf(k1, k2));
      }
    };
    clampk(ta0, da, Pa);
    clampk(tf0, df, Pff);
    clampk(tz0, dz, Pzz);
    // estimate [a0, a1), then settle both ends on the exact test (an empty
    // estimate starts from one point next to where the interval would be)
    const bool some = khi >= klo;
    int a0 = (int)fminf(fmaxf(ceilf(some ? klo : fminf(klo, khi)), 0.f), (float)n);
    int a1 = some ? (int)fminf(fmaxf(ceilf(khi), 0.f), (float)n) : a0;
    while (a0 > 0 && inside(a0 - 1)) --a0;
    while (a0 < a1 && !inside(a0)) ++a0;
    while (a1 < n && inside(a1)) ++a1;
    while (a1 > a0 && !inside(a1 - 1)) --a1;
    k0 = a0;
    n = a1;
    if (k0 >= n) {
      k0 = 0;
      n = 0;
    }
  }
  L.ta0 = ta0; L.tf0 = tf0; L.tz0 = tz0;
  L.da = da; L.df = df; L.dz = dz;
  // par / fan rays keep one z tap row for the whole ray
  L.fzc = floorf(tz0);
  L.wzc = tz0 - L.fzc;
  L.k = k0;
  L.n = n;
  L.acc = 0.f;
}

// Samples of one ray whose a-tap lies in the slab [alo, ahi] (sweep direction
// D), from the slab's buffer b, two per iteration where possible: positions
// fma(k, d, t0) on both lanes of a pair.  Tap indices are kept as floats
// (exact below 2^24) so a sample costs one float->int conversion for its
// shared-memory index.
template <int GEOM, bool ZW, int D, typename TV>
__device__ __forceinline__ void smem_ray(RayLane& L, const TV* b, float2 off2, float alo_f,
                                         float ahi_f) {
  using C = SlabCfg<GEOM>;
  constexpr bool Z2 = (GEOM >= 2);
  const float2 da2 = make_float2(L.da, L.da), df2 = make_float2(L.df, L.df);
  const float2 dz2 = make_float2(L.dz, L.dz);
  const float2 ta02 = make_float2(L.ta0, L.ta0), tf02 = make_float2(L.tf0, L.tf0);
  const float2 tz02 = make_float2(L.tz0, L.tz0);
  const float2 fz02 = make_float2(L.fzc, L.fzc), wz02 = make_float2(L.wzc, L.wzc);
  int k = L.k;
  const int n = L.n;
  float acc = L.acc;
  while (k < n) {
    const float k0 = (float)k;
    const float2 kk = make_float2(k0, k0 + 1.0f);
    const float2 ta2 = __ffma2_rn(kk, da2, ta02);
    const float fa0 = floorf(ta2.x);
    if (D > 0 ? fa0 > ahi_f : fa0 < alo_f) break;
    const float fa1 = floorf(ta2.y);
    const bool two = (k + 1 < n) && (D > 0 ? fa1 <= ahi_f : fa1 >= alo_f);
    const float2 tf2 = __ffma2_rn(kk, df2, tf02);
    const float2 fa2 = make_float2(fa0, fa1);
    const float2 ff2 = make_float2(floorf(tf2.x), floorf(tf2.y));
    float2 fz2 = fz02, wz2 = wz02;
    if (Z2) {
      const float2 tz2 = __ffma2_rn(kk, dz2, tz02);
      fz2 = make_float2(floorf(tz2.x), floorf(tz2.y));
      wz2 = sub2(tz2, fz2);
    }
    const float2 wa2 = sub2(ta2, fa2), wf2 = sub2(tf2, ff2);
    const float2 x2 = __ffma2_rn(fz2, make_float2((float)C::Plane, (float)C::Plane),
                                 __ffma2_rn(fa2, make_float2((float)C::F, (float)C::F),
                                            __fadd2_rn(ff2, off2)));
    // Tap indices are exact in FP32 (< 2^24); a negative one wraps to a
    // large unsigned value and is clamped like one past the end.
    const unsigned i0 = min((unsigned)__float2int_rn(x2.x), (unsigned)C::MaxIdx);
    if (two) {
      const unsigned i1 = min((unsigned)__float2int_rn(x2.y), (unsigned)C::MaxIdx);
      const float2 v = sample_pair<ZW>(b + i0, b + i1, C::F, C::Plane, wa2, wf2, wz2);
      acc += v.x;
      acc += v.y;
      k += 2;
    } else {
      acc += sample_at<ZW>(b + i0, C::F, C::Plane, wa2.x, wf2.x, wz2.x);
      k += 1;
      break;
    }
  }
  L.k = k;
  L.acc = acc;
}

// The rays of one thread in two views through the slab in step: sample k_A of
// ray A and k_B of ray B on the two lanes of each FP32x2 operation (per ray the
// same operations as smem_ray), while both have a sample in the slab; the ray
// left over finishes with smem_ray.
template <int GEOM, bool ZW, int D, typename TV>
__device__ __forceinline__ void smem_ray_pair(RayLane& A, RayLane& B, const TV* b, float2 off2,
                                              float alo_f, float ahi_f) {
  using C = SlabCfg<GEOM>;
  constexpr bool Z2 = (GEOM >= 2);
  const float2 da2 = make_float2(A.da, B.da), df2 = make_float2(A.df, B.df);
  const float2 dz2 = make_float2(A.dz, B.dz);
  const float2 ta02 = make_float2(A.ta0, B.ta0), tf02 = make_float2(A.tf0, B.tf0);
  const float2 tz02 = make_float2(A.tz0, B.tz0);
  const float2 fz02 = make_float2(A.fzc, B.fzc), wz02 = make_float2(A.wzc, B.wzc);
  int ka = A.k, kb = B.k;
  float acca = A.acc, accb = B.acc;
  while (ka < A.n && kb < B.n) {
    const float2 kk = make_float2((float)ka, (float)kb);
    const float2 ta2 = __ffma2_rn(kk, da2, ta02);
    const float2 fa2 = make_float2(floorf(ta2.x), floorf(ta2.y));
    if (D > 0 ? fmaxf(fa2.x, fa2.y) > ahi_f : fminf(fa2.x, fa2.y) < alo_f) break;
    const float2 tf2 = __ffma2_rn(kk, df2, tf02);
    const float2 ff2 = make_float2(floorf(tf2.x), floorf(tf2.y));
    float2 fz2 = fz02, wz2 = wz02;
    if (Z2) {
      const float2 tz2 = __ffma2_rn(kk, dz2, tz02);
      fz2 = make_float2(floorf(tz2.x), floorf(tz2.y));
      wz2 = sub2(tz2, fz2);
    }
    const float2 wa2 = sub2(ta2, fa2), wf2 = sub2(tf2, ff2);
    const float2 x2 = __ffma2_rn(fz2, make_float2((float)C::Plane, (float)C::Plane),
                                 __ffma2_rn(fa2, make_float2((float)C::F, (float)C::F),
                                            __fadd2_rn(ff2, off2)));
    const unsigned i0 = min((unsigned)__float2int_rn(x2.x), (unsigned)C::MaxIdx);
    const unsigned i1 = min((unsigned)__float2int_rn(x2.y), (unsigned)C::MaxIdx);
    const float2 v = sample_pair<ZW>(b + i0, b + i1, C::F, C::Plane, wa2, wf2, wz2);
    acca += v.x;
    accb += v.y;
    ++ka;
    ++kb;
  }
  A.k = ka;
  A.acc = acca;
  B.k = kb;
  B.acc = accb;
  smem_ray<GEOM, ZW, D>(A, b, off2, alo_f, ahi_f);
  smem_ray<GEOM, ZW, D>(B, b, off2, alo_f, ahi_f);
}

// The same samples of one ray from the padded volume in global memory (a
// slab whose bundle did not fit the box, or after a wait gave up).
template <int GEOM, bool ZW, bool SUB, typename TV>
__device__ __forceinline__ void global_ray(RayLane& L, const TV* gv, const SlabJob& J, int dir,
                                           float alo_f, float ahi_f, int Ps, int Pz, int Pf) {
  constexpr bool Z2 = (GEOM >= 2);
  int k = L.k;
  float acc = L.acc;
  while (k < L.n) {
    const float kq = (float)k;
    const float tq = fmaf(kq, L.da, L.ta0);
    const float fq = floorf(tq);
    if (dir > 0 ? fq > ahi_f : fq < alo_f) break;
    const float tfq = fmaf(kq, L.df, L.tf0);
    const float tzq = Z2 ? fmaf(kq, L.dz, L.tz0) : L.tz0;
    const float ffq = floorf(tfq), fzq = floorf(tzq);
    const int ga = min(max((int)fq, 0), Ps - 2), gf = min(max((int)ffq, 0), Pf - 2);
    const int gz = min(max((int)fzq, 0), Pz - 2);
    if (SUB)
      acc += sample_rows<ZW>(gv + (size_t)gf + (size_t)Pf * (size_t)ga, gz - J.zoff, J.zrows, Pf,
                             Pf * Ps, tq - fq, tfq - ffq, tzq - fzq);
    else
      acc += sample_at<ZW>(gv + (size_t)gf + (size_t)Pf * ((size_t)ga + (size_t)Ps * gz), Pf,
                           Pf * Ps, tq - fq, tfq - ffq, tzq - fzq);
    ++k;
  }
  L.k = k;
  L.acc = acc;
}

// One tile: sweep the volume along the views' dominant axis slab by slab.
// Ends with a CTA barrier, so the shared state can be reused by the next job.
// V views per CTA (the tile's pixels in J.nv <= V consecutive views with the
// same dominant axis): every slab's box covers the bundles of all of them, and
// each thread samples its pixel's ray in every view.
// ZL (decoupled detector): par / fan rays whose constant z falls between
// texel rows interpolate in z as well, and rays that miss the volume sample
// nothing.
// SUB: a z-slab of the volume (launch_fp_slab_sub); each ray samples only
// the k whose z taps can reach the slab's rows.
template <int GEOM, int EPI, typename TV, typename TO, bool ZL = false, bool SUB = false,
          int V = 1>
__device__ __forceinline__ void slab_tile(const SlabJob& J, TV* buf0, TV* buf1, SlabShared& S,
                                          uint32_t& phase, uint32_t& issued,
                                          const SlabEpi& E, int vb = 0, int nvj = -1) {
  static_assert(V == 1 || V == 2, "one or two views per CTA");
  // this call's views: J's views vb .. vb + nvj - 1 (nvj < 0: all of J's)
  if (nvj < 0) nvj = J.nv;
  const Trig trv[2] = {vb ? J.tr[1] : J.tr[0], J.tr[1]};
  const long long gvv[2] = {vb ? J.gview[1] : J.gview[0], J.gview[1]};
  const long long lvv[2] = {vb ? J.lview[1] : J.lview[0], J.lview[1]};
  using C = SlabCfg<GEOM>;
  constexpr bool Z2 = (GEOM >= 2);  // z changes along the ray
  // trilinear samples; otherwise par/fan rays sample exact z texel rows
  constexpr bool ZW = Z2 || ZL;
  constexpr int NC = 4 * V;  // corner rays: four per view
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int u0 = J.tu0, v0 = J.tv0;
  const int ix = u0 + threadIdx.x, iy = v0 + threadIdx.y;
  const bool xdom = fabsf(trv[0].c) >= fabsf(trv[0].s);  // rays run mostly along x
  const int Ps = J.S + 2, Pz = J.Z + 2, Pf = J.Pf;

  // An absent second view (J.nv = 1) repeats the first one's geometry with no
  // samples, so its corner rays change no box.
  RayLane L[V];
  float se[V][6];
#pragma unroll
  for (int r = 0; r < V; ++r)
    ray_setup<GEOM, ZL, SUB>(J, r < nvj ? trv[r] : trv[0], r < nvj, ix, iy, xdom, Ps, Pz, L[r],
                             &se[r][0], &se[r][3]);

  if (tid == 0) {
    S.amin = 0x7fffffff;
    S.amax = -0x7fffffff;
    S.pos = 0;
    S.neg = 0;
    if (GEOM == 3)
#pragma unroll
      for (int i = 0; i < 8; ++i) S.gbi[i] = (i & 1) ? (int)0x80000000 : 0x7fffffff;
  }
  // Corner rays of the valid part of the tile bound the bundle (slot 4r + c:
  // c bit 0 right column, bit 1 bottom row).
  const int lx = min(31, J.det_w - 1 - u0), ly = min(7, J.det_h - 1 - v0);
  __syncthreads();
  {
    const bool top = threadIdx.y == 0, bot = (int)threadIdx.y == ly;
    const bool lft = threadIdx.x == 0, rgt = (int)threadIdx.x == lx;
#pragma unroll
    for (int r = 0; r < V; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (((c & 2) ? bot : top) && ((c & 1) ? rgt : lft))
#pragma unroll
          for (int i = 0; i < 6; ++i) S.corner[4 * r + c][i] = se[r][i];
  }
  {
    int lo = 0x7fffffff, hi = -0x7fffffff, np = 0, nn = 0;
#pragma unroll
    for (int r = 0; r < V; ++r) {
      if (L[r].n > 0) {
        const int t_first =
            __float2int_rd((SUB || GEOM == 3) ? fmaf((float)L[r].k, L[r].da, L[r].ta0) : L[r].ta0);
        const int t_last = __float2int_rd(fmaf((float)(L[r].n - 1), L[r].da, L[r].ta0));
        lo = min(lo, min(t_first, t_last));
        hi = max(hi, max(t_first, t_last));
        if (L[r].da > 0.f) ++np;
        else ++nn;
      }
    }
    if (np + nn > 0) {
      atomicMin(&S.amin, lo);
      atomicMax(&S.amax, hi);
      if (np) atomicAdd(&S.pos, np);
      if (nn) atomicAdd(&S.neg, nn);
    }
  }
  __syncthreads();
  const int s_amin = S.amin, s_amax = S.amax;
  const bool any = s_amax >= s_amin;
  const int dir = S.neg == 0 ? 1 : -1;
  const bool mixed = S.pos > 0 && S.neg > 0;
  const int nslab = any ? (s_amax - s_amin) / C::T + 1 : 0;
  // general3D: a tile's rays need not lie in the hull of its corner rays, so
  // the slab boxes come from bounds over all its rays.  Along the sweep axis
  // a ray's f and z are linear in a: f = F + mf (a - aref) with F its f at
  // aref, so over the tile f >= Fmin + (a >= aref ? mfmin : mfmax)(a - aref),
  // f <= Fmax + (a >= aref ? mfmax : mfmin)(a - aref), and the same for z.
  float gb[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // Fmin Fmax mfmin mfmax, z: same
  bool gunb = false;  // a ray nearly parallel to the a-planes: no box
  const float aref = 0.5f * (float)(s_amin + s_amax + 1);
  if constexpr (GEOM == 3) {
    float v[8];
    bool bad = false;
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = (i & 1) ? -3.0e38f : 3.0e38f;
#pragma unroll
    for (int r = 0; r < V; ++r) {
      if (L[r].n > 0) {
        if (!(fabsf(L[r].da) >= 1e-3f)) {
          bad = true;
        } else {
          const float mf = L[r].df / L[r].da, mz = L[r].dz / L[r].da;
          const float Fr = fmaf(aref - L[r].ta0, mf, L[r].tf0);
          const float Zr = fmaf(aref - L[r].ta0, mz, L[r].tz0);
          v[0] = fminf(v[0], Fr); v[1] = fmaxf(v[1], Fr);
          v[2] = fminf(v[2], mf); v[3] = fmaxf(v[3], mf);
          v[4] = fminf(v[4], Zr); v[5] = fmaxf(v[5], Zr);
          v[6] = fminf(v[6], mz); v[7] = fmaxf(v[7], mz);
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float t = __shfl_xor_sync(0xffffffffu, v[i], o);
        v[i] = (i & 1) ? fmaxf(v[i], t) : fminf(v[i], t);
      }
    // floats as order-preserving ints for the shared-memory atomics
    auto key = [](float f) {
      const int i = __float_as_int(f);
      return i >= 0 ? i : i ^ 0x7fffffff;
    };
    if ((tid & 31) == 0)
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (i & 1) atomicMax(&S.gbi[i], key(v[i]));
        else atomicMin(&S.gbi[i], key(v[i]));
      }
    gunb = __syncthreads_or(bad) != 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int k = S.gbi[i];
      gb[i] = __int_as_float(k >= 0 ? k : k ^ 0x7fffffff);
    }
  }
  const TV* gv = static_cast<const TV*>(xdom ? J.py : J.px);  // f-fastest padded layout
  const CUtensorMap* tm = xdom ? J.tmy : J.tmx;
  uint64_t* bar = S.bar;
  // Tap range [alo, ahi] of slab j.
  auto slab_range = [&](int j, int& alo, int& ahi) {
    if (dir > 0) {
      alo = s_amin + j * C::T;
      ahi = alo + C::T - 1;
    } else {
      ahi = s_amax - j * C::T;
      alo = ahi - C::T + 1;
    }
  };

  // Plan every slab of the tile up front, 256 / (2 NC) slabs per pass of the
  // CTA: the 2 NC lanes of a group evaluate the NC corner rays at the 2
  // a-ends of their slab in FP32 (error ~1e-4 voxel, covered by the 1-voxel
  // margin), reduce the f/z extent by shuffles, and the group's first lane
  // stores the box.
  {
    const float bfw = xdom ? J.by : J.bx;  // world offset of the f axis
    const float baw = xdom ? J.bx : J.by;  // world offset of the a axis
    const int np = min(nslab, C::MaxPlans);
    const int c = tid % NC, w = (tid / NC) & 1;
    const float sa = xdom ? S.corner[c][0] : S.corner[c][1];
    const float sf = xdom ? S.corner[c][1] : S.corner[c][0];
    const float ea = xdom ? S.corner[c][3] : S.corner[c][4];
    const float ef = xdom ? S.corner[c][4] : S.corner[c][3];
    const float sz = S.corner[c][2], ez = S.corner[c][5];
    const float den = ea - sa;
    for (int base = 0; base < np; base += 256 / (2 * NC)) {
      const int j = base + tid / (2 * NC);
      const bool act = j < np;
      int alo, ahi;
      slab_range(j, alo, ahi);
      float fmn, fmx, zmn, zmx;  // world f / z extent at this lane's slab end
      if constexpr (GEOM == 3) {
        // bounds over the tile's rays at tap-space a = alo or ahi + 1
        const float dT = (w ? (float)ahi + 1.0f : (float)alo) - aref;
        const bool up = dT >= 0.f;
        fmn = fmaf(dT, up ? gb[2] : gb[3], gb[0]) + bfw - 0.5f;
        fmx = fmaf(dT, up ? gb[3] : gb[2], gb[1]) + bfw - 0.5f;
        zmn = fmaf(dT, up ? gb[6] : gb[7], gb[4]) + J.bz - 0.5f;
        zmx = fmaf(dT, up ? gb[7] : gb[6], gb[5]) + J.bz - 0.5f;
        if (!act || gunb) {
          fmn = zmn = 3.0e38f;
          fmx = zmx = -3.0e38f;
        }
      } else {
        const float aw = w ? (float)ahi + 0.5f + baw : (float)alo - 0.5f + baw;
        const float t = den != 0.f ? (aw - sa) / den : 0.f;
        const float fv = fmaf(t, ef - sf, sf), zv = fmaf(t, ez - sz, sz);
        fmn = act ? fv : 3.0e38f;
        fmx = act ? fv : -3.0e38f;
        zmn = act ? zv : 3.0e38f;
        zmx = act ? zv : -3.0e38f;
      }
#pragma unroll
      for (int o = NC; o > 0; o >>= 1) {
        fmn = fminf(fmn, __shfl_xor_sync(0xffffffffu, fmn, o));
        fmx = fmaxf(fmx, __shfl_xor_sync(0xffffffffu, fmx, o));
        zmn = fminf(zmn, __shfl_xor_sync(0xffffffffu, zmn, o));
        zmx = fmaxf(zmx, __shfl_xor_sync(0xffffffffu, zmx, o));
      }
      if (act && (tid % (2 * NC)) == 0) {
        const int align = sizeof(TV) == 4 ? 4 : 8;
        const float flo = floorf(fmn - bfw + 0.5f) - 1.0f;
        const float fhi = floorf(fmx - bfw + 0.5f) + 2.0f;
        const float zlo = floorf(zmn - J.bz + 0.5f) - 1.0f;
        const float zhi = floorf(zmx - J.bz + 0.5f) + 2.0f;
        bool fits = isfinite(flo) && isfinite(fhi) && isfinite(zlo) && isfinite(zhi) &&
                    !mixed && !gunb && fhi >= 0.f && zhi >= 0.f && flo <= (float)(Pf - 1) &&
                    zlo <= (float)(Pz - 1);
        int f0 = 0, z0 = 0;
        if (fits) {
          const int fl = (int)fmaxf(flo, 0.f), zl = (int)fmaxf(zlo, 0.f);
          const int fh = (int)fminf(fhi, (float)(Pf - 1));
          const int zh = (int)fminf(zhi, (float)(Pz - 1));
          f0 = (fl / align) * align;
          z0 = zl;
          const int nzr = zh - z0 + 1;
          fits = (fh - f0 + 1 <= C::F) && (nzr <= C::Z) && nzr > 0 && f0 <= 65532 &&
                 z0 <= 8191;
          if (fits) S.plans[j] = pack_plan(f0, z0, nzr);
        }
        if (!fits) S.plans[j] = kPlanFallback;
      }
    }
  }
  __syncthreads();

  // Start the copy of slab j into buffer j&1 (thread 0 only).
  auto issue = [&](int j) {
    const uint32_t pk = j < C::MaxPlans ? S.plans[j] : kPlanFallback;
    const int nzr = plan_nzr(pk);
    if (nzr == 0 || S.abort) return;
    int alo, ahi;
    slab_range(j, alo, ahi);
    const int nbox = (nzr + C::Z - 1) / C::Z;
    const int f0 = plan_f0(pk), z0 = plan_z0(pk);
    TV* dst = (j & 1) ? buf1 : buf0;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar[j & 1], (uint32_t)(nbox * C::Z * C::Plane * sizeof(TV)));
    for (int bx = 0; bx < nbox; ++bx)
      tma_load_3d(dst + (size_t)bx * C::Z * C::Plane, tm, f0, alo,
                  z0 + bx * C::Z - (SUB ? J.zoff : 0), &bar[j & 1]);
    // thread 0 counts the copies issued into each buffer (16 bits each)
    issued += 1u << (16 * (j & 1));
  };
  if (tid == 0 && nslab > 0) issue(0);

  // One accumulator per ray, samples added in ray order: the sum does not
  // depend on how the samples fall into slabs or on which path (shared /
  // global) took them.
  for (int j = 0; j < nslab; ++j) {
    // Buffer (j+1)&1 was released by the barrier that ended slab j-1.
    if (tid == 0 && j + 1 < nslab) issue(j + 1);
    const uint32_t pk = j < C::MaxPlans ? S.plans[j] : kPlanFallback;
    int alo, ahi;
    slab_range(j, alo, ahi);
    const TV* b = (j & 1) ? buf1 : buf0;
    // A copy was issued exactly when the plan has a box and no wait of this
    // CTA had timed out; after a time-out every wait returns false at once.
    bool from_smem = plan_nzr(pk) != 0;
    if (from_smem) {
      // bit b of phase: parity of buffer b's next completion
      from_smem = mbar_wait_bounded(&bar[j & 1], (phase >> (j & 1)) & 1u, E.err, &S.abort,
                                    E.wait_us);
      phase ^= 1u << (j & 1);
    }
    const float alo_f = (float)alo, ahi_f = (float)ahi;
    // The sweep direction and the sample source are uniform over a slab, so
    // each gets its own loop: the shared-memory loops compare against one
    // bound with no per-sample selects or source branch.
    if (from_smem) {
      const float off = -(float)(plan_z0(pk) * C::Plane + alo * C::F + plan_f0(pk));
      const float2 off2 = make_float2(off, off);
      if constexpr (V == 2) {
        if (dir > 0) smem_ray_pair<GEOM, ZW, 1>(L[0], L[1], b, off2, alo_f, ahi_f);
        else smem_ray_pair<GEOM, ZW, -1>(L[0], L[1], b, off2, alo_f, ahi_f);
      } else {
        if (dir > 0) smem_ray<GEOM, ZW, 1>(L[0], b, off2, alo_f, ahi_f);
        else smem_ray<GEOM, ZW, -1>(L[0], b, off2, alo_f, ahi_f);
      }
    } else {
#pragma unroll
      for (int r = 0; r < V; ++r)
        global_ray<GEOM, ZW, SUB>(L[r], gv, J, dir, alo_f, ahi_f, Ps, Pz, Pf);
    }
    __syncthreads();
  }
  if (tid == 0 && S.abort) {
    // Copies issued before a wait gave up still land in this CTA's buffers:
    // wait for them (bounded) before the buffers are reused or the CTA exits.
    slab_drain(bar, issued, E.err);
  }
  if (EPI == 2) {
    // Objective epilogue: sum of pre*e^-l + post*l over the tile in FP64
    // (fixed order: the thread's views, warp shuffles, then the 8 warps in
    // order), added to the CTA's partial (zeroed by the caller).
    __shared__ double wsum[8];
    double t = 0.0;
#pragma unroll
    for (int r = 0; r < V; ++r) {
      if (L[r].valid) {
        const float l = L[r].acc * J.step;
        const size_t gi = (size_t)gvv[r] * J.P + (size_t)iy * J.det_w + ix;
        const float pv = __ldg(E.pre + gi), qv = __ldg(E.post + gi);
        t += (double)(pv * expf(-l)) + (double)qv * (double)l;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((tid & 31) == 0) wsum[tid >> 5] = t;
    __syncthreads();
    if (tid == 0) {
      double bs = 0.0;
#pragma unroll
      for (int w = 0; w < 8; ++w) bs += wsum[w];
      E.obj[(size_t)blockIdx.x * gridDim.y + blockIdx.y] += bs;
    }
  }
#pragma unroll
  for (int r = 0; r < V; ++r) {
    if (EPI != 2 && L[r].valid) {
      const float l = L[r].acc * J.step;
      const size_t pix = (size_t)iy * J.det_w + ix;
      const size_t gi = (size_t)gvv[r] * J.P + pix;
      if (EPI == 0) {
        TO* o = static_cast<TO*>(J.out) + gi;
        stf(o, (SUB && J.accum) ? ldp(o) + l : l);
      } else {
        // CUDAmex_oscIter.cu:262-268: pre' = pre e^-l - post, post' = pre e^-l l.
        const float pv = __ldg(E.pre + gi), qv = __ldg(E.post + gi);
        const float ehat = pv * expf(-l);
        // padded residual view [H+4][W+4] (zero frame kept by the caller)
        const int Wp = sino_pad_pitch(J.det_w);
        const size_t ri = ((size_t)lvv[r] * (J.det_h + 2 * kSinoPad) + (iy + kSinoPad)) * Wp +
                          (ix + kSinoPad);
        const float r0 = ehat - qv, r1 = ehat * l;
        // quad layout (the dual BP's one 16-byte load per voxel, cone, or per z
        // pair, par / fan): the padded texel P(r, c) is component x of quad
        // (r, c), y of (r-1, c), z of (r, c-1) and w of (r-1, c-1)
        const size_t q[4] = {4 * ri, 4 * (ri - Wp) + 1, 4 * (ri - 1) + 2, 4 * (ri - Wp - 1) + 3};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if constexpr (std::is_same<TO, float>::value) {
            static_cast<float*>(E.rpre)[q[t]] = r0;
            static_cast<float*>(E.rpost)[q[t]] = r1;
          } else {
            // 16-bit residual views hold the residuals times a power of two
            stf(static_cast<TO*>(E.rpre) + q[t], r0 * E.rscale);
            stf(static_cast<TO*>(E.rpost) + q[t], r1 * E.rscale);
          }
        }
      }
    }
  }
  __syncthreads();
}

// V views per CTA: 2 where the launch pairs adjacent views (their bundles
// overlap: slab_pair_views), else 1.
template <int GEOM, bool BORDER, int EPI, typename TV, typename TO, bool ZL = false,
          bool SUB = false, int V = 1>
__global__ void __launch_bounds__(256, kSlabCtas) fp_slab_kernel(
    const __grid_constant__ RayArgs A, const __grid_constant__ CUtensorMap tmx,
    const __grid_constant__ CUtensorMap tmy, const TV* __restrict__ px,
    const TV* __restrict__ py, int Pf, TO* __restrict__ out, const SlabEpi E) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ SlabShared S;
  TV* buf0 = reinterpret_cast<TV*>(smem_raw);
  TV* buf1 = buf0 + kBufElems;
  slab_init_barriers(S);
  uint32_t phase = 0u, issued = 0u;  // issued: copies per buffer (thread 0)
  const int per = V;
  const int view0 = blockIdx.x * per;
  const int tiles_u = (A.det_w + 31) >> 5;
  SlabJob J;
  J.det_w = A.det_w; J.det_h = A.det_h; J.S = A.S; J.Z = A.Z; J.Pf = Pf;
  J.u0 = A.u0; J.v0 = A.v0; J.bx = A.bx; J.by = A.by; J.bz = A.bz;
  J.SR = A.SR; J.RD = A.RD; J.step = A.step;
  J.du = A.du; J.dv = A.dv; J.ou = A.ou; J.ov = A.ov;
  J.zoff = A.zoff; J.zrows = A.zrows; J.accum = A.accum; J.zlo = A.zlo; J.zhi = A.zhi;
  J.nv = min(per, A.nviews - view0);
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int vr = view0 + min(r, J.nv - 1);
    J.tr[r] = A.trig[vr];
    J.gview[r] = A.view0 + (long long)vr * A.vstride;
    J.lview[r] = vr;
  }
  J.P = A.P;
  J.pts = GEOM == 3 ? A.pts + (A.pts_per_view ? (size_t)6 * A.P * J.gview[0] : 0) : nullptr;
  J.tu0 = (blockIdx.y % tiles_u) * 32;
  J.tv0 = (blockIdx.y / tiles_u) * 8;
  J.tmx = &tmx; J.tmy = &tmy; J.px = px; J.py = py; J.out = out;
  const bool split = V == 2 && J.nv == 2 &&
                     (fabsf(J.tr[0].c) >= fabsf(J.tr[0].s)) != (fabsf(J.tr[1].c) >= fabsf(J.tr[1].s));
  if (!split) {
    slab_tile<GEOM, EPI, TV, TO, ZL, SUB, V>(J, buf0, buf1, S, phase, issued, E);
  } else {
    // the two views sweep different axes: one view at a time
    slab_tile<GEOM, EPI, TV, TO, ZL, SUB, V>(J, buf0, buf1, S, phase, issued, E, 0, 1);
    slab_tile<GEOM, EPI, TV, TO, ZL, SUB, V>(J, buf0, buf1, S, phase, issued, E, 1, 1);
  }
}

// ---------------------------------------------------------------------------
// Batched FP over many problems of different sizes and geometries in one
// persistent launch: CTAs take (problem, view, tile) items from a global
// counter (work stealing) and run the same tile code as above.
// ---------------------------------------------------------------------------
template <typename TV>
__global__ void __launch_bounds__(256, kSlabCtas) fp_batch_kernel(
    const BatchFp* __restrict__ probs, int nprob, long long total,
    unsigned long long* __restrict__ counter, unsigned* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ SlabShared S;
  TV* buf0 = reinterpret_cast<TV*>(smem_raw);
  TV* buf1 = buf0 + kBufElems;
  slab_init_barriers(S);
  uint32_t phase = 0u, issued = 0u;  // issued: copies per buffer (thread 0)
  const SlabEpi E{nullptr, nullptr, nullptr, nullptr, err};
  for (;;) {
    if (threadIdx.x + 32 * threadIdx.y == 0) S.item = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const long long item = S.item;
    if (item >= total) break;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (probs[mid].item0 <= item) lo = mid;
      else hi = mid - 1;
    }
    const BatchFp& B = probs[lo];
    const long long rr = item - B.item0;
    const int view = (int)(rr % B.nviews);
    const int tile = (int)(rr / B.nviews);
    SlabJob J;
    J.det_w = B.W; J.det_h = B.H; J.S = B.W; J.Z = B.H; J.Pf = B.Pf;
    J.u0 = B.u0; J.v0 = B.v0; J.bx = B.bx; J.by = B.by; J.bz = B.bz;
    J.SR = B.sad; J.RD = B.sad; J.step = B.step;
    J.du = 1.0f; J.dv = 1.0f; J.ou = 0.0f; J.ov = 0.0f;
    J.zoff = 0; J.zrows = B.H + 2; J.accum = 0; J.zlo = 0.f; J.zhi = 0.f; J.pts = nullptr;
    J.tr[0] = J.tr[1] = B.trig[view];
    J.nv = 1;
    J.P = (long long)B.W * B.H;
    J.gview[0] = J.gview[1] = view;
    J.lview[0] = J.lview[1] = view;
    J.tu0 = (tile % B.tiles_u) * 32;
    J.tv0 = (tile / B.tiles_u) * 8;
    J.tmx = &B.tmx; J.tmy = &B.tmy; J.px = B.px; J.py = B.py; J.out = B.out;
    if (B.geom == 0) slab_tile<0, 0, TV, TV>(J, buf0, buf1, S, phase, issued, E);
    else if (B.geom == 1) slab_tile<1, 0, TV, TV>(J, buf0, buf1, S, phase, issued, E);
    else slab_tile<2, 0, TV, TV>(J, buf0, buf1, S, phase, issued, E);
  }
}

// ---------------------------------------------------------------------------
// Host side: tensor maps and launch.
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

cudaError_t make_slab_tmap(CUtensorMap* map, const void* base, int dtype, int Pf, int Ps,
                           int Pz, int geom) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  const size_t es = dtype == kF32 ? 4 : 2;
  cuuint64_t dims[3] = {(cuuint64_t)Pf, (cuuint64_t)Ps, (cuuint64_t)Pz};
  cuuint64_t strides[2] = {(cuuint64_t)Pf * es, (cuuint64_t)Pf * Ps * es};
  const int F = geom >= 2 ? SlabCfg<2>::F : SlabCfg<0>::F;
  const int A = geom >= 2 ? SlabCfg<2>::A : SlabCfg<0>::A;
  const int Z = geom >= 2 ? SlabCfg<2>::Z : SlabCfg<0>::Z;
  cuuint32_t box[3] = {(cuuint32_t)F, (cuuint32_t)A, (cuuint32_t)Z};
  cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = dtype == kF32   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                 : dtype == kF16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  CUresult r = fn(map, dt, 3, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int slab_pitch(int W) { return ((W + 2 + 7) / 8) * 8; }

// Whether views 2i and 2i+1 of a launch share their slab boxes: the box
// covers a tile's bundle with ~18 voxels to spare along f, and two views
// delta apart shift the bundle by up to delta times the volume's half
// diagonal W/sqrt(2), so pairs are taken while that shift stays within
// ~6 voxels (0.95 degrees at W = 512: 720 views over 2 pi pair, 360 do not).
bool slab_pair_views(const RayArgs& a) {
  if (a.nviews < 2) return false;
  const double lim = 8.5 / (double)std::max(a.S, 1);
  const double cmin = std::cos(lim);
  for (int i = 0; i + 1 < a.nviews; i += 2) {
    const Trig p = a.trig[i], q = a.trig[i + 1];
    if ((double)p.c * q.c + (double)p.s * q.s < cmin) return false;
  }
  return true;
}

// Dynamic shared memory of the slab kernels and the largest shared-memory
// carveout: kSlabCtas CTAs of 57 KB each need nearly all of an SM's 228 KB.
template <typename K>
static cudaError_t set_slab_attrs(K k, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                              cudaSharedmemCarveoutMaxShared);
}

// Resident CTAs per SM of the cone FP32 slab kernel (occupancy calculator).
int slab_resident_ctas() {
  auto k = fp_slab_kernel<2, false, 0, float, float>;
  const size_t smem = 2 * (size_t)kBufElems * sizeof(float) + 128;
  if (set_slab_attrs(k, smem) != cudaSuccess) return -1;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 256, smem) != cudaSuccess) return -1;
  return n;
}

cudaError_t launch_fp_batch(const BatchFp* d_probs, int nprob, long long total,
                            unsigned long long* counter, unsigned* err, int ctas,
                            cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  auto k = fp_batch_kernel<float>;
  const size_t smem = 2 * (size_t)kBufElems * sizeof(float) + 128;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = set_slab_attrs(k, smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  k<<<ctas, dim3(32, 8), smem, st>>>(d_probs, nprob, total, counter, err);
  return cudaGetLastError();
}

template <int GEOM, bool BORDER, int EPI, typename TV, typename TO, bool ZL = false,
          bool SUB = false>
static cudaError_t slab_go(const RayArgs& a, const CUtensorMap& mx, const CUtensorMap& my,
                           const void* px, const void* py, int Pf, void* out,
                           const SlabEpi& e, cudaStream_t st) {
  auto k1 = fp_slab_kernel<GEOM, BORDER, EPI, TV, TO, ZL, SUB, 1>;
  auto k2 = fp_slab_kernel<GEOM, BORDER, EPI, TV, TO, ZL, SUB, GEOM == 3 ? 1 : 2>;
  const size_t smem = 2 * (size_t)kBufElems * sizeof(TV) + 128;
  static bool attr_set = false;  // once per instantiation (before any capture)
  if (!attr_set) {
    cudaError_t err = set_slab_attrs(k1, smem);
    if (err == cudaSuccess) err = set_slab_attrs(k2, smem);
    if (err != cudaSuccess) return err;
    attr_set = true;
  }
  if (a.nviews <= 0) return cudaSuccess;
  const int tiles = ((a.det_w + 31) / 32) * ((a.det_h + 7) / 8);
  const bool pair = GEOM != 3 && slab_pair_views(a);
  dim3 blk(32, 8), grd(pair ? (a.nviews + 1) / 2 : a.nviews, tiles);
  if (pair)
    k2<<<grd, blk, smem, st>>>(a, mx, my, (const TV*)px, (const TV*)py, Pf, (TO*)out, e);
  else
    k1<<<grd, blk, smem, st>>>(a, mx, my, (const TV*)px, (const TV*)py, Pf, (TO*)out, e);
  return cudaGetLastError();
}

cudaError_t launch_fp_slab_det(int geom, const RayArgs& a, const CUtensorMap& mx,
                               const CUtensorMap& my, const void* px, const void* py, int Pf,
                               float* out, const SlabEpi& e, cudaStream_t st) {
  if (geom == 0) return slab_go<0, false, 0, float, float, true>(a, mx, my, px, py, Pf, out, e, st);
  if (geom == 1) return slab_go<1, false, 0, float, float, true>(a, mx, my, px, py, Pf, out, e, st);
  if (geom == 2) return slab_go<2, false, 0, float, float, true>(a, mx, my, px, py, Pf, out, e, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_fp_slab_osc_det(int geom, const RayArgs& a, const CUtensorMap& mx,
                                   const CUtensorMap& my, const void* px, const void* py, int Pf,
                                   const SlabEpi& e, cudaStream_t st) {
  if (geom == 0) return slab_go<0, true, 1, float, float, true>(a, mx, my, px, py, Pf, nullptr, e, st);
  if (geom == 1) return slab_go<1, true, 1, float, float, true>(a, mx, my, px, py, Pf, nullptr, e, st);
  if (geom == 2) return slab_go<2, true, 1, float, float, true>(a, mx, my, px, py, Pf, nullptr, e, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_fp_slab_g3d(const RayArgs& a, const CUtensorMap& mx, const CUtensorMap& my,
                               const void* px, const void* py, int Pf, float* out,
                               const SlabEpi& e, cudaStream_t st) {
  return slab_go<3, true, 0, float, float>(a, mx, my, px, py, Pf, out, e, st);
}

cudaError_t launch_fp_slab_sub(int geom, const RayArgs& a, const CUtensorMap& mx,
                               const CUtensorMap& my, const void* px, const void* py, int Pf,
                               float* out, const SlabEpi& e, cudaStream_t st) {
  if (geom == 0)
    return slab_go<0, false, 0, float, float, false, true>(a, mx, my, px, py, Pf, out, e, st);
  if (geom == 1)
    return slab_go<1, false, 0, float, float, false, true>(a, mx, my, px, py, Pf, out, e, st);
  if (geom == 2)
    return slab_go<2, false, 0, float, float, false, true>(a, mx, my, px, py, Pf, out, e, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_fp_slab_objective(int geom, const RayArgs& a, const CUtensorMap& mx,
                                     const CUtensorMap& my, const void* px, const void* py,
                                     int Pf, int vt, const SlabEpi& e, cudaStream_t st) {
  if (!e.obj || !e.pre || !e.post) return cudaErrorInvalidValue;
#define GO(G, TV) return slab_go<G, true, 2, TV, float>(a, mx, my, px, py, Pf, nullptr, e, st)
  if (vt == kF32) {
    if (geom == 0) GO(0, float);
    if (geom == 1) GO(1, float);
    GO(2, float);
  }
  if (vt == kF16) {
    if (geom == 0) GO(0, __half);
    if (geom == 1) GO(1, __half);
    GO(2, __half);
  }
  if (geom == 0) GO(0, __nv_bfloat16);
  if (geom == 1) GO(1, __nv_bfloat16);
  GO(2, __nv_bfloat16);
#undef GO
}

cudaError_t launch_fp_slab(int geom, bool border, bool osc, const RayArgs& a,
                           const CUtensorMap& mx, const CUtensorMap& my, const void* px,
                           const void* py, int Pf, int vt, void* out, int ot,
                           const SlabEpi& e, cudaStream_t st) {
#define GO(G, B, EP, TV, TO) return slab_go<G, B, EP, TV, TO>(a, mx, my, px, py, Pf, out, e, st)
  if (osc) {
    // ot: storage of the residual views (FP16 with FP32 mu only)
    if (ot == kF16) {
      if (vt != kF32) return cudaErrorInvalidValue;
      if (geom == 0) GO(0, true, 1, float, __half);
      if (geom == 1) GO(1, true, 1, float, __half);
      GO(2, true, 1, float, __half);
    }
    if (vt == kF32) {
      if (geom == 0) GO(0, true, 1, float, float);
      if (geom == 1) GO(1, true, 1, float, float);
      GO(2, true, 1, float, float);
    }
    if (vt == kF16) {
      if (geom == 0) GO(0, true, 1, __half, float);
      if (geom == 1) GO(1, true, 1, __half, float);
      GO(2, true, 1, __half, float);
    }
    if (geom == 0) GO(0, true, 1, __nv_bfloat16, float);
    if (geom == 1) GO(1, true, 1, __nv_bfloat16, float);
    GO(2, true, 1, __nv_bfloat16, float);
  }
  (void)border;
  if (vt == kF32 && ot == kF32) {
    if (geom == 0) GO(0, false, 0, float, float);
    if (geom == 1) GO(1, false, 0, float, float);
    GO(2, false, 0, float, float);
  }
  if (vt == kF16 && ot == kF16) {
    if (geom == 0) GO(0, false, 0, __half, __half);
    if (geom == 1) GO(1, false, 0, __half, __half);
    GO(2, false, 0, __half, __half);
  }
  if (vt == kF16 && ot == kF32) {
    if (geom == 0) GO(0, false, 0, __half, float);
    if (geom == 1) GO(1, false, 0, __half, float);
    GO(2, false, 0, __half, float);
  }
  if (vt == kBF16 && ot == kBF16) {
    if (geom == 0) GO(0, false, 0, __nv_bfloat16, __nv_bfloat16);
    if (geom == 1) GO(1, false, 0, __nv_bfloat16, __nv_bfloat16);
    GO(2, false, 0, __nv_bfloat16, __nv_bfloat16);
  }
  if (vt == kBF16 && ot == kF32) {
    if (geom == 0) GO(0, false, 0, __nv_bfloat16, float);
    if (geom == 1) GO(1, false, 0, __nv_bfloat16, float);
    GO(2, false, 0, __nv_bfloat16, float);
  }
#undef GO
  return cudaErrorInvalidValue;
}

}  // namespace mexct
