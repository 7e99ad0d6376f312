// oracle.cpp -- FP64 C++17/OpenMP restatement of the mex-cuda-CT operators.
//
// TEST INFRASTRUCTURE ONLY (the correctness checker and the timed CPU
// baseline).  The product library never links or calls this file.
//
// Every function cites the reference file:line it restates.  The reference
// files are kurtishdekker/mex-cuda-CT:
//   projection_kernels/CUDAmex_FP.cu, CUDAmex_BP.cu, CUDAmex_general3D_FP.cu,
//   CUDAmex_general3D_BP.cu, iterative_reconstruction/CUDAmex_oscIter.cu,
//   CUDAmex_TVmin_3D.cu, OSC_TV_recon.m, fbp_reconstruction/preFilterSinogram.m,
//   parker_weight.m.
//
// Build with -ffp-contract=off (oracle/Makefile): the binary32 ray set-up
// below must round every operation separately, as the reference source
// writes it, on x86-64 and on aarch64 alike.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

int g_threads = 0;
// Interpolation weights of the texture fetches: 0 = exact, 1 = rounded to the
// nearest 1/256, 2 = truncated to 1/256, 3 = the texture unit's own rule
// (tex_hw below).  CUDA's linear texture filter keeps
// the fractional weight in 9-bit fixed point with 8 fractional bits (CUDA C
// Programming Guide, "Linear Filtering"); modes 1/2 emulate that so the
// difference between exact trilinear output and the reference's
// texture-filtered output can be stated.
int g_tex_weights = 0;

// Sample positions: 0 = FP64 p0 + k*d (default); 1 = the reference's own
// binary32 arithmetic: FP positions advanced by `currentpoint += stepsize`
// and turned into texture coordinates by a binary32 `currentpoint - b`
// (CUDAmex_FP.cu:141-148,240-246,337-343; CUDAmex_general3D_FP.cu:141-147;
// CUDAmex_oscIter.cu:253-259), BP columns set up in binary32 (s, t, U,
// proj_y, proj_z) and advanced by `proj_z += U` (CUDAmex_BP.cu:86-101,
// :144-159, :201-219; CUDAmex_oscIter.cu:307-355).  Sums stay FP64 in both
// modes, so mode 1 against mode 0 isolates the stepping difference.
int g_ref_steps = 0;

inline double qw(double a) {
  if (g_tex_weights == 1) return std::floor(a * 256.0 + 0.5) / 256.0;
  if (g_tex_weights == 2) return std::floor(a * 256.0) / 256.0;
  return a;
}

inline int nthreads() {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

const float kNaNf = std::numeric_limits<float>::quiet_NaN();

// ---------------------------------------------------------------------------
// Ray set-up in binary32 as the reference computes it: CUDAmex_FP.cu:82-137
// (the same block appears in CUDAmex_general3D_FP.cu:81-136,
// CUDAmex_general3D_BP.cu:81-143 and CUDAmex_oscIter.cu:193-248), with the
// multiply-adds its nvcc build fuses written as explicit fmas.
// ---------------------------------------------------------------------------
struct Ray {
  float cx, cy, cz;  // clipped entry point ("currentpoint")
  float dx, dy, dz;  // per-step displacement ("stepsizeX/Y/Z")
  int n;             // number of samples of while(travelled < distance)
};

Ray clip_ray(float sx, float sy, float sz, float ex, float ey, float ez,
             float bx, float by, float bz, float step) {
  float ax1, ax2, ay1, ay2, az1, az2;
  // `fabsf(d) >= 1e-5` compares in double (1e-5 is a double literal).
  if ((double)std::fabs(ex - sx) >= 1e-5) {
    ax1 = (bx - sx) / (ex - sx);
    ax2 = (-bx - sx) / (ex - sx);
  } else {
    ax1 = ax2 = kNaNf;
  }
  if ((double)std::fabs(ey - sy) >= 1e-5) {
    ay1 = (by - sy) / (ey - sy);
    ay2 = (-by - sy) / (ey - sy);
  } else {
    ay1 = ay2 = kNaNf;
  }
  if ((double)std::fabs(ez - sz) >= 1e-5) {
    az1 = (bz - sz) / (ez - sz);
    az2 = (-bz - sz) / (ez - sz);
  } else {
    az1 = az2 = kNaNf;
  }
  const float axmin = std::fmin(ax1, ax2), axmax = std::fmax(ax1, ax2);
  const float aymin = std::fmin(ay1, ay2), aymax = std::fmax(ay1, ay2);
  const float azmin = std::fmin(az1, az2), azmax = std::fmax(az1, az2);
  float tmp = std::fmax(axmin, std::fmax(aymin, azmin));
  const float amin = std::fmax(0.f, tmp);
  tmp = std::fmin(axmax, std::fmin(aymax, azmax));
  const float amax = std::fmin(1.f, tmp);

  // The reference's build (nvcc -O3, fused multiply-add on by default) fuses
  // `s + a*(e - s)` into one fma, and the squared length into
  // fma(qz, qz, fma(qx, qx, qy*qy)); the reference-output fixtures pin this
  // (general3D BP indices and weights reproduce only with these fmas, and a
  // texture FP with them reproduces the reference's FP bit for bit).
  Ray r;
  r.cx = std::fma(amin, ex - sx, sx);
  r.cy = std::fma(amin, ey - sy, sy);
  r.cz = std::fma(amin, ez - sz, sz);
  const float px = std::fma(amax, ex - sx, sx);
  const float py = std::fma(amax, ey - sy, sy);
  const float pz = std::fma(amax, ez - sz, sz);
  const float qx = px - r.cx, qy = py - r.cy, qz = pz - r.cz;
  const float dist = std::sqrt(std::fma(qz, qz, std::fma(qx, qx, qy * qy)));
  r.dx = (px - r.cx) / dist * step;
  r.dy = (py - r.cy) / dist * step;
  r.dz = (pz - r.cz) / dist * step;
  // while(travelled < distance) with travelled = k*step exact in binary32:
  // the number of k >= 0 with k*step < dist is ceil(dist/step) (dist/step is
  // exact for step 0.5 and 1).  NaN / non-positive distance: no sample.  An
  // infinite distance would never terminate in the reference; it yields no
  // sample here.
  if (!(dist > 0.f) || !std::isfinite(dist)) {
    r.n = 0;
  } else {
    r.n = (int)std::ceil(dist / step);
  }
  return r;
}

// Whether the segment s -> e meets the volume box [b, -b] per axis, with the
// clip's own per-axis alphas.  The reference's rays always do (each crosses
// the isocentre plane at least 0.5 voxel inside the box); on a decoupled
// detector a ray can miss, and then adds nothing (the clip above would march
// it between two points outside the box, an axis it runs parallel to open).
bool hits_box(const float* s, const float* e, float bx, float by, float bz) {
  const float b[3] = {bx, by, bz};
  float amin = 0.f, amax = 1.f;
  for (int i = 0; i < 3; ++i) {
    const float d = e[i] - s[i];
    if ((double)std::fabs(d) >= 1e-5) {
      const float a1 = (b[i] - s[i]) / d, a2 = (-b[i] - s[i]) / d;
      amin = std::fmax(amin, std::fmin(a1, a2));
      amax = std::fmin(amax, std::fmax(a1, a2));
    } else if (std::fabs(s[i]) > -b[i]) {
      return false;
    }
  }
  return amin <= amax;
}

// ---------------------------------------------------------------------------
// Texture fetch semantics (unnormalised coordinates, texel centre at i+0.5,
// linear filter), with exact FP64 weights.  Clamp = clamp index to the edge,
// border = 0 outside.  Address modes: CUDAmex_FP.cu:407-409 (clamp),
// CUDAmex_BP.cu:272-273 (clamp), CUDAmex_general3D_FP.cu:219-221 (border),
// CUDAmex_oscIter.cu:419-425,460-462 (border).
// ---------------------------------------------------------------------------
inline double safe_coord(double c, int n) {
  // Keep the coordinate where floor() fits an int; the fetched value does not
  // change (clamp: edge texel; border: zero).
  if (c < -4.0) return -4.0;
  if (c > (double)n + 4.0) return (double)n + 4.0;
  return c;
}

// Mode 3 (g_tex_weights == 3): the GPU texture unit's linear filter as
// measured on a GB300 (the CUDA Programming Guide states only that the
// weights are 9-bit fixed point with 8 fractional bits).  Per axis, clamp
// addressing first clamps the coordinate c - 0.5 to [0, n - 1]; the result is
// rounded to the nearest 1/256 (ties up) and split into the index i and the
// fraction f in [0, 255] (a fraction that rounds up to 256 carries into i).
// With fractions a (x), b (y), c (z) the eight integer weights, which sum to
// 256, are built per z plane k (z weight fz = c or 256 - c):
//   X1 = rnd(a*fz/256), X0 = fz - X1                       (x = 1 / x = 0),
//   W(1,1,k) = rnd(X1*b/256),       W(1,0,k) = X1 - W(1,1,k),
//   W(0,0,k) = rnd(X0*(256-b)/256), W(0,1,k) = X0 - W(0,0,k),
// with rnd = round to nearest, ties up; 2-D fetches are the same rule with
// c = 0.  The value is sum(W * texel) / 256.  Against 65,536 random fetches
// of each kind this reproduces the hardware to 6e-8 absolute (the hardware
// rounds its sum to binary32; that last ulp is the only difference).
struct HwAxis {
  int i;     // lower texel index
  double f;  // fraction in units of 1/256, 0..255
};

inline HwAxis hw_axis(double c, int n, bool border) {
  double cb = c - 0.5;
  if (!border) cb = std::min(std::max(cb, 0.0), (double)(n - 1));
  const double q = std::floor(cb * 256.0 + 0.5);
  const double i = std::floor(q / 256.0);
  return HwAxis{(int)i, q - 256.0 * i};
}

inline double rnd_hu(double x) { return std::floor(x + 0.5); }

template <typename T>
inline double hw_tap(const T* v, int n0, int n1, int n2, int i, int j, int k,
                     bool border) {
  if (border) {
    if (i < 0 || i >= n0 || j < 0 || j >= n1 || k < 0 || k >= n2) return 0.0;
  } else {
    i = std::min(std::max(i, 0), n0 - 1);
    j = std::min(std::max(j, 0), n1 - 1);
    k = std::min(std::max(k, 0), n2 - 1);
  }
  return (double)v[(size_t)i + (size_t)n0 * ((size_t)j + (size_t)n1 * k)];
}

template <typename T>
inline double tex_hw(const T* v, int n0, int n1, int n2, double c0, double c1,
                     double c2, bool border, bool three_d) {
  const HwAxis x = hw_axis(c0, n0, border), y = hw_axis(c1, n1, border);
  const HwAxis z = three_d ? hw_axis(c2, n2, border) : HwAxis{0, 0.0};
  const double a = x.f, b = y.f, c = z.f;
  double acc = 0.0;
  for (int k = 0; k < (three_d ? 2 : 1); ++k) {
    const double fz = k ? c : 256.0 - c;
    const double X1 = rnd_hu(a * fz / 256.0), X0 = fz - X1;
    const double w11 = rnd_hu(X1 * b / 256.0), w10 = X1 - w11;
    const double w00 = rnd_hu(X0 * (256.0 - b) / 256.0), w01 = X0 - w00;
    const int kk = z.i + k;
    acc += w00 * hw_tap(v, n0, n1, n2, x.i, y.i, kk, border) +
           w10 * hw_tap(v, n0, n1, n2, x.i + 1, y.i, kk, border) +
           w01 * hw_tap(v, n0, n1, n2, x.i, y.i + 1, kk, border) +
           w11 * hw_tap(v, n0, n1, n2, x.i + 1, y.i + 1, kk, border);
  }
  return acc / 256.0;
}

template <typename T>
inline double tex3(const T* v, int n0, int n1, int n2, double c0, double c1,
                   double c2, bool border) {
  if (g_tex_weights == 3)
    return tex_hw(v, n0, n1, n2, safe_coord(c0, n0), safe_coord(c1, n1),
                  safe_coord(c2, n2), border, true);
  c0 = safe_coord(c0, n0) - 0.5;
  c1 = safe_coord(c1, n1) - 0.5;
  c2 = safe_coord(c2, n2) - 0.5;
  const double f0 = std::floor(c0), f1 = std::floor(c1), f2 = std::floor(c2);
  const double a = qw(c0 - f0), b = qw(c1 - f1), g = qw(c2 - f2);
  const int i0 = (int)f0, j0 = (int)f1, k0 = (int)f2;
  double acc = 0.0;
  for (int dk = 0; dk < 2; ++dk) {
    int k = k0 + dk;
    const double wk = dk ? g : 1.0 - g;
    if (border) {
      if (k < 0 || k >= n2) continue;
    } else {
      k = std::min(std::max(k, 0), n2 - 1);
    }
    for (int dj = 0; dj < 2; ++dj) {
      int j = j0 + dj;
      const double wj = dj ? b : 1.0 - b;
      if (border) {
        if (j < 0 || j >= n1) continue;
      } else {
        j = std::min(std::max(j, 0), n1 - 1);
      }
      for (int di = 0; di < 2; ++di) {
        int i = i0 + di;
        const double wi = di ? a : 1.0 - a;
        if (border) {
          if (i < 0 || i >= n0) continue;
        } else {
          i = std::min(std::max(i, 0), n0 - 1);
        }
        acc += wk * wj * wi *
               (double)v[(size_t)i + (size_t)n0 * ((size_t)j + (size_t)n1 * k)];
      }
    }
  }
  return acc;
}

template <typename T>
inline double tex2(const T* p, int n0, int n1, double c0, double c1,
                   bool border) {
  if (g_tex_weights == 3)
    return tex_hw(p, n0, n1, 1, safe_coord(c0, n0), safe_coord(c1, n1), 0.0,
                  border, false);
  c0 = safe_coord(c0, n0) - 0.5;
  c1 = safe_coord(c1, n1) - 0.5;
  const double f0 = std::floor(c0), f1 = std::floor(c1);
  const double a = qw(c0 - f0), b = qw(c1 - f1);
  const int i0 = (int)f0, j0 = (int)f1;
  double acc = 0.0;
  for (int dj = 0; dj < 2; ++dj) {
    int j = j0 + dj;
    const double wj = dj ? b : 1.0 - b;
    if (border) {
      if (j < 0 || j >= n1) continue;
    } else {
      j = std::min(std::max(j, 0), n1 - 1);
    }
    for (int di = 0; di < 2; ++di) {
      int i = i0 + di;
      const double wi = di ? a : 1.0 - a;
      if (border) {
        if (i < 0 || i >= n0) continue;
      } else {
        i = std::min(std::max(i, 0), n0 - 1);
      }
      acc += wj * wi * (double)p[(size_t)i + (size_t)n0 * j];
    }
  }
  return acc;
}

// Host trig of the projection angle.  The reference calls sincosf(beta) on
// the host (CUDAmex_FP.cu:449); the correctly rounded binary32 value of the
// FP64 sine/cosine is used here and in the CUDA library alike.
inline void trig(float beta, float* s, float* c) {
  *s = (float)std::sin((double)beta);
  *c = (float)std::cos((double)beta);
}

// Ray end points of the standard geometries in binary32.
// par: CUDAmex_FP.cu:64-77; cone: :162-175; fan: :259-272 (and the switch in
// CUDAmex_oscIter.cu:152-187).
// Detector generalisation (no counterpart in the reference, whose detector is
// the volume's W x H with one voxel per pixel at the isocentre): pixel pitch
// du, dv at the isocentre and a sub-pixel offset ou, ov.  du = dv = 1,
// ou = ov = 0 give the reference's binary32 operations exactly.
inline void std_ray(int geom, int ix, int iy, float u0, float v0, float sb,
                    float cb, float SR, float RD, float* s, float* e,
                    float du = 1.0f, float dv = 1.0f, float ou = 0.0f,
                    float ov = 0.0f) {
  float u, v;
  // Fused as the reference's build fuses them (pinned by the reference-output
  // fixtures).  A product used twice is rounded once and shared: in the
  // parallel geometry u*sinB and u*cosB appear in both end points, so the
  // other product of each sum is the fused one; in fan and cone u appears
  // only in the detector end point, fused as fma(-RD, cosB, -(u*sinB)) and
  // fma(u, cosB, -RD*sinB) (the general3D rotation has the same form).
  switch (geom) {
    case 0:
      u = (((float)ix + ou) - u0) * du;
      v = (((float)iy + ov) - v0) * dv;
      s[0] = std::fma(SR, cb, -(u * sb));
      s[1] = std::fma(SR, sb, u * cb);
      s[2] = v;
      e[0] = std::fma(-RD, cb, -(u * sb));
      e[1] = std::fma(-RD, sb, u * cb);
      e[2] = v;
      return;
    case 1:
      u = ((((float)ix + ou) - u0) * du) * (SR + RD) / SR;
      v = (((float)iy + ov) - v0) * dv;
      s[0] = (SR * cb);
      s[1] = (SR * sb);
      s[2] = v;
      break;
    default:
      u = ((((float)ix + ou) - u0) * du) * (SR + RD) / SR;
      v = ((((float)iy + ov) - v0) * dv) * (SR + RD) / SR;
      s[0] = (SR * cb);
      s[1] = (SR * sb);
      s[2] = 0.0f;
      break;
  }
  e[0] = std::fma(-RD, cb, -(u * sb));
  e[1] = std::fma(u, cb, -RD * sb);
  e[2] = v;
}

// general3D end points rotated by the view angle (CUDAmex_general3D_FP.cu:71-77,
// CUDAmex_general3D_BP.cu:73-79), fused as the reference's build fuses them.
inline void g3d_rotate(float x, float y, float sb, float cb, float* rx, float* ry) {
  *rx = std::fma(x, cb, -(y * sb));
  *ry = std::fma(y, cb, x * sb);
}

// March one clipped ray over a volume with FP64 positions p0 + k*d.
template <typename T>
inline double march(const Ray& r, float step, const T* vol, int n0, int n1,
                    int n2, float bx, float by, float bz, bool border) {
  double acc = 0.0;
  if (g_ref_steps) {
    float cx = r.cx, cy = r.cy, cz = r.cz;
    for (int k = 0; k < r.n; ++k) {
      const float tx = cx - bx, ty = cy - by, tz = cz - bz;
      acc += tex3(vol, n0, n1, n2, (double)tx, (double)ty, (double)tz, border) *
             (double)step;
      cx += r.dx;
      cy += r.dy;
      cz += r.dz;
    }
    return acc;
  }
  for (int k = 0; k < r.n; ++k) {
    const double px = (double)r.cx + (double)k * (double)r.dx;
    const double py = (double)r.cy + (double)k * (double)r.dy;
    const double pz = (double)r.cz + (double)k * (double)r.dz;
    acc += tex3(vol, n0, n1, n2, px - (double)bx, py - (double)by,
                pz - (double)bz, border) *
           (double)step;
  }
  return acc;
}

// Circle of reconstruction with the reference's unsigned arithmetic
// (CUDAmex_BP.cu:73-77, CUDAmex_oscIter.cu:100-101,119-120,301-305).
inline bool in_circle(int ix, int iy, uint32_t hw) {
  const uint32_t dx = (uint32_t)ix - hw, dy = (uint32_t)iy - hw;
  return (uint32_t)(dx * dx + dy * dy) < (uint32_t)(hw * hw);
}

// Standard-geometry BP sample position of one voxel column
// (CUDAmex_BP.cu:79-101, :137-159, :199-219; CUDAmex_oscIter.cu:307-354).
struct BpCol {
  double wgt;   // U*U (UU*UU in the OSC kernel)
  double py;    // projection u coordinate
  double pz0;   // projection v coordinate at iz = 0
  double dpz;   // increment per iz
};

// Projection coordinates of voxel column (ix, iy) for one view.  The
// detector generalisation: the u centre is Wd/2 (integer division, the
// reference's hw + 1), the v centre (Hd - 1)/2 + 0.5, pixel pitches du, dv at
// the isocentre; Wd = W, Hd = H, du = dv = 1 are the reference's formulas.
inline BpCol bp_column(int geom, int ix, int iy, uint32_t hw, float v0,
                       float sb, float cb, float SR, int Wd = -1, int Hd = -1,
                       double du = 1.0, double dv = 1.0) {
  const float x = ix - (hw + 0.5f);
  const float y = iy - (hw + 0.5f);
  const double s = (double)x * cb + (double)y * sb;
  const double t = -(double)x * sb + (double)y * cb;
  const double uc = Wd < 0 ? (double)hw + 1.0 : (double)((uint32_t)Wd / 2u);
  const double v0d = Hd < 0 ? (double)v0 : (double)(Hd - 1) / 2.0;
  BpCol c;
  if (geom == 0) {
    c.wgt = 1.0;
    c.py = t / du + uc;
    c.pz0 = -(double)v0 / dv + v0d + 0.5;
    c.dpz = 1.0 / dv;
  } else {
    const double U = (double)SR / ((double)SR - s);
    c.wgt = U * U;
    c.py = t * U / du + uc;
    if (geom == 1) {
      c.pz0 = -(double)v0 / dv + v0d + 0.5;
      c.dpz = 1.0 / dv;
    } else {
      c.pz0 = -(double)v0 * U / dv + v0d + 0.5;
      c.dpz = U / dv;
    }
  }
  return c;
}

// The same column in the reference's binary32 arithmetic (g_ref_steps = 1),
// with the multiply-adds its build fuses written as fmas.
// The plain BP (CUDAmex_BP.cu:79-101 par, :137-159 fan, :197-219 cone) and the
// OSC dual BP (CUDAmex_oscIter.cu:307-355: weight UU*UU, fan with U = 1 and
// proj_z from 0.5) compute the same values term by term.  proj_z advances by
// dpz in binary32.
struct BpColF {
  float wgt, py, pz0, dpz;
};

inline BpColF bp_column_ref(int geom, int ix, int iy, uint32_t hw,
                            float v0, float sb, float cb, float SR) {
  const float x = ix - (hw + 0.5f);
  const float y = iy - (hw + 0.5f);
  const float s = std::fma(y, sb, x * cb);
  const float t = std::fma(y, cb, -x * sb);
  BpColF c;
  if (geom == 0) {
    const float U = 1.f;
    c.wgt = U * U;
    c.py = std::fma(t, U, (float)hw) + 1.f;
    c.pz0 = std::fma(-v0, U, v0) + 0.5f;
    c.dpz = U;
  } else if (geom == 1) {
    const float UU = SR / (SR - s);
    c.wgt = UU * UU;
    c.py = std::fma(t, UU, (float)hw) + 1.f;
    c.pz0 = 0.5f;
    c.dpz = 1.f;
  } else {
    const float U = SR / (SR - s);
    c.wgt = U * U;
    c.py = std::fma(t, U, (float)hw) + 1.f;
    c.pz0 = std::fma(-v0, U, v0) + 0.5f;
    c.dpz = U;
  }
  return c;
}

}  // namespace

extern "C" {

void orc_set_ref_steps(int mode) { g_ref_steps = mode ? 1 : 0; }
int orc_get_ref_steps(void) { return g_ref_steps; }

void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) { return nthreads(); }
void orc_set_tex_weights(int mode) { g_tex_weights = (mode >= 0 && mode <= 3) ? mode : 0; }
int orc_get_tex_weights(void) { return g_tex_weights; }

// CUDAmex_FP.cu:350-477 (gateway) and :56-346 (kernels), with the detector
// generalisation: Wd x Hd pixels of pitch du, dv at the isocentre, ss x ss
// rays per pixel at sub-pixel offsets (k + 0.5)/ss - 0.5, averaged.
int orc_fp_det(const float* vol, int W, int H, float sad, const float* angles,
               int nP, int geom, int Wd, int Hd, float du, float dv, int ss,
               double* out) {
  if (!vol || !angles || !out || W <= 0 || H <= 0 || nP < 0) return 1;
  if (geom < 0 || geom > 2 || Wd <= 0 || Hd <= 0 || ss < 1 || !(du > 0.f) || !(dv > 0.f))
    return 1;
  const float u0 = float(Wd - 1) / 2;
  const float v0 = float(Hd - 1) / 2;
  const float bx = -(float)W / 2.0f, by = -(float)W / 2.0f,
              bz = -(float)H / 2.0f;
  const float step = (geom == 2) ? 1.0f : 0.5f;  // :231 vs :133,:328
  const float SR = sad, RD = sad;
  const long long P = (long long)Wd * Hd;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
  for (long long r = 0; r < P * nP; ++r) {
    const int view = (int)(r / P);
    const int pix = (int)(r % P);
    const int ix = pix % Wd, iy = pix / Wd;
    float sb, cb;
    trig(angles[view], &sb, &cb);
    double acc = 0.0;
    for (int a = 0; a < ss; ++a)
      for (int b = 0; b < ss; ++b) {
        const float ou = ss == 1 ? 0.0f : ((float)b + 0.5f) / (float)ss - 0.5f;
        const float ov = ss == 1 ? 0.0f : ((float)a + 0.5f) / (float)ss - 0.5f;
        float s[3], e[3];
        std_ray(geom, ix, iy, u0, v0, sb, cb, SR, RD, s, e, du, dv, ou, ov);
        if (!hits_box(s, e, bx, by, bz)) continue;  // misses the volume: adds nothing
        const Ray ray = clip_ray(s[0], s[1], s[2], e[0], e[1], e[2], bx, by, bz,
                                 step);
        acc += march(ray, step, vol, W, W, H, bx, by, bz, /*border=*/false);
      }
    out[r] = acc / ((double)ss * ss);
  }
  return 0;
}

int orc_fp(const float* vol, int W, int H, float sad, const float* angles,
           int nP, int geom, double* out) {
  return orc_fp_det(vol, W, H, sad, angles, nP, geom, W, H, 1.0f, 1.0f, 1, out);
}

// CUDAmex_BP.cu:223-324 (gateway) and :44-221 (kernels), with the detector
// generalisation (sinogram Wd x Hd x nP, pitch du, dv; volume W x W x H).
int orc_bp_det(const float* sino, int Wd, int Hd, int nP, float sad,
               const float* angles, int geom, int W, int H, float du, float dv,
               double* vol) {
  if (!sino || !angles || !vol || W <= 0 || H <= 0 || Wd <= 0 || Hd <= 0 || nP < 0) return 1;
  if (geom < 0 || geom > 2 || !(du > 0.f) || !(dv > 0.f)) return 1;
  const float v0 = float(H - 1) / 2;
  const uint32_t hw = (uint32_t)W / 2u - 1u;
  const size_t N = (size_t)W * W * H;
  std::memset(vol, 0, N * sizeof(double));
  std::vector<float> sbv(nP), cbv(nP);
  for (int j = 0; j < nP; ++j) trig(angles[j], &sbv[j], &cbv[j]);
  const size_t P = (size_t)Wd * Hd;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads())
  for (long long col = 0; col < (long long)W * W; ++col) {
    const int ix = (int)(col % W), iy = (int)(col / W);
    if (!in_circle(ix, iy, hw)) continue;
    std::vector<double> acc(H, 0.0);
    const bool ref_cols = g_ref_steps && Wd == W && Hd == H && du == 1.f && dv == 1.f;
    for (int j = 0; j < nP; ++j) {
      const float* proj = sino + P * j;
      if (ref_cols) {
        const BpColF c = bp_column_ref(geom, ix, iy, hw, v0, sbv[j], cbv[j], sad);
        float pz = c.pz0;
        for (int iz = 0; iz < H; ++iz) {
          acc[iz] += (double)c.wgt * tex2(proj, Wd, Hd, (double)c.py, (double)pz, false);
          pz += c.dpz;
        }
        continue;
      }
      const BpCol c = bp_column(geom, ix, iy, hw, v0, sbv[j], cbv[j], sad, Wd, Hd, du, dv);
      for (int iz = 0; iz < H; ++iz) {
        const double pz = c.pz0 + c.dpz * iz;
        acc[iz] += c.wgt * tex2(proj, Wd, Hd, c.py, pz, /*border=*/false);
      }
    }
    for (int iz = 0; iz < H; ++iz)
      vol[(size_t)ix + (size_t)W * iy + (size_t)W * W * iz] = acc[iz];
  }
  return 0;
}

int orc_bp(const float* sino, int W, int H, int nP, float sad,
           const float* angles, int geom, double* vol) {
  return orc_bp_det(sino, W, H, nP, sad, angles, geom, W, H, 1.0f, 1.0f, vol);
}

// CUDAmex_general3D_FP.cu:154-252 (gateway) and :59-150 (kernel).
int orc_g3d_fp(const float* vol, int S, int Z, const float* angles,
               const float* pts, int W, int H, int nP, int pts_per_view,
               double* out) {
  if (!vol || !angles || !pts || !out || S <= 0 || Z <= 0 || W <= 0 ||
      H <= 0 || nP < 0)
    return 1;
  const float bx = -(float)S / 2.0f, by = bx, bz = -(float)Z / 2.0f;
  const float step = 0.5f;
  const long long P = (long long)W * H;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
  for (long long r = 0; r < P * nP; ++r) {
    const int view = (int)(r / P);
    const long long pix = r % P;
    const float* pt = pts + (pts_per_view ? (size_t)6 * P * view : 0);
    float sb, cb;
    trig(angles[view], &sb, &cb);
    // :71-77
    const float x1 = pt[pix], y1 = pt[pix + P], z1 = pt[pix + 2 * P];
    const float x2 = pt[pix + 3 * P], y2 = pt[pix + 4 * P],
                z2 = pt[pix + 5 * P];
    float sx, sy, ex, ey;
    g3d_rotate(x1, y1, sb, cb, &sx, &sy);
    g3d_rotate(x2, y2, sb, cb, &ex, &ey);
    const Ray ray = clip_ray(sx, sy, z1, ex, ey, z2, bx, by, bz, step);
    out[r] = march(ray, step, vol, S, S, Z, bx, by, bz, /*border=*/true);
  }
  return 0;
}

// The exact transpose of orc_g3d_fp (no counterpart in the reference): the
// same rays and FP64 sample positions, each sample's eight trilinear weights
// (border addressing: taps outside the volume dropped) times p * step added
// to the tap voxels.  Per-thread FP64 volumes, reduced in thread order.
int orc_g3d_bp_matched(const float* sino, int W, int H, int nP, const float* angles,
                       const float* pts, int pts_per_view, int S, int Z, double* vol) {
  if (!sino || !angles || !pts || !vol || S <= 0 || Z <= 0 || W <= 0 || H <= 0 || nP < 0)
    return 1;
  const float bx = -(float)S / 2.0f, by = bx, bz = -(float)Z / 2.0f;
  const float step = 0.5f;
  const size_t N = (size_t)S * S * Z;
  const long long P = (long long)W * H;
  const int nt = nthreads();
  std::vector<std::vector<double>> part(nt);
#pragma omp parallel num_threads(nt)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<double>& acc = part[tid];
    acc.assign(N, 0.0);
#pragma omp for schedule(dynamic, 16)
    for (long long r = 0; r < P * nP; ++r) {
      const int view = (int)(r / P);
      const long long pix = r % P;
      const double p = sino[(size_t)P * view + pix];
      if (p == 0.0) continue;
      const float* pt = pts + (pts_per_view ? (size_t)6 * P * view : 0);
      float sb, cb;
      trig(angles[view], &sb, &cb);
      float sx, sy, ex, ey;
      g3d_rotate(pt[pix], pt[pix + P], sb, cb, &sx, &sy);
      g3d_rotate(pt[pix + 3 * P], pt[pix + 4 * P], sb, cb, &ex, &ey);
      const Ray ray = clip_ray(sx, sy, pt[pix + 2 * P], ex, ey, pt[pix + 5 * P], bx, by, bz, step);
      for (int k = 0; k < ray.n; ++k) {
        const double c0 = (double)ray.cx + (double)k * (double)ray.dx - (double)bx - 0.5;
        const double c1 = (double)ray.cy + (double)k * (double)ray.dy - (double)by - 0.5;
        const double c2 = (double)ray.cz + (double)k * (double)ray.dz - (double)bz - 0.5;
        const double f0 = std::floor(c0), f1 = std::floor(c1), f2 = std::floor(c2);
        if (f0 < -2 || f0 > S || f1 < -2 || f1 > S || f2 < -2 || f2 > Z) continue;
        const double a = c0 - f0, b = c1 - f1, g = c2 - f2;
        const int i0 = (int)f0, j0 = (int)f1, k0 = (int)f2;
        for (int t = 0; t < 8; ++t) {
          const int i = i0 + (t & 1), j = j0 + ((t >> 1) & 1), kk = k0 + (t >> 2);
          if (i < 0 || i >= S || j < 0 || j >= S || kk < 0 || kk >= Z) continue;
          const double w = ((t & 1) ? a : 1.0 - a) * (((t >> 1) & 1) ? b : 1.0 - b) *
                           ((t >> 2) ? g : 1.0 - g);
          acc[(size_t)i + (size_t)S * ((size_t)j + (size_t)S * kk)] += p * (double)step * w;
        }
      }
    }
  }
  std::memset(vol, 0, N * sizeof(double));
  for (int t = 0; t < nt; ++t) {
    if (part[t].empty()) continue;
#pragma omp parallel for num_threads(nt)
    for (long long i = 0; i < (long long)N; ++i) vol[i] += part[t][i];
  }
  return 0;
}

// CUDAmex_general3D_BP.cu:194-282 (gateway) and :61-188 (kernel).  The
// positions advance incrementally in binary32 and the voxel indices and
// weights are binary32, exactly as in the reference (they are discontinuous
// in the position); each deposit is accumulated in FP64.
int orc_g3d_bp(const float* sino, int W, int H, int nP, const float* angles,
               const float* pts, int pts_per_view, int S, int Z,
               double* vol) {
  if (!sino || !angles || !pts || !vol || S <= 0 || Z <= 0 || W <= 0 ||
      H <= 0 || nP < 0)
    return 1;
  const float bx = -(float)S / 2.0f, by = bx, bz = -(float)Z / 2.0f;
  const float step = 0.5f;
  const size_t N = (size_t)S * S * Z;
  const long long P = (long long)W * H;
  const int nt = nthreads();
  // Per-thread accumulation volumes keep the sum order of each thread fixed;
  // they are reduced at the end in thread order.
  std::vector<std::vector<double>> part(nt);
#pragma omp parallel num_threads(nt)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<double>& acc = part[tid];
    acc.assign(N, 0.0);
#pragma omp for schedule(dynamic, 16)
    for (long long r = 0; r < P * nP; ++r) {
      const int view = (int)(r / P);
      const long long pix = r % P;
      const float* pt = pts + (pts_per_view ? (size_t)6 * P * view : 0);
      float sb, cb;
      trig(angles[view], &sb, &cb);
      const float x1 = pt[pix], y1 = pt[pix + P], z1 = pt[pix + 2 * P];
      const float x2 = pt[pix + 3 * P], y2 = pt[pix + 4 * P],
                  z2 = pt[pix + 5 * P];
      float sx, sy, ex, ey;
      g3d_rotate(x1, y1, sb, cb, &sx, &sy);
      g3d_rotate(x2, y2, sb, cb, &ex, &ey);
      Ray ray = clip_ray(sx, sy, z1, ex, ey, z2, bx, by, bz, step);
      const float p = sino[(size_t)P * view + pix];
      float cx = ray.cx, cy = ray.cy, cz = ray.cz;
      for (int k = 0; k < ray.n; ++k) {
        // :151-158
        const int iL = (int)std::floor(cx - (bx));
        const int iU = (int)std::ceil(cx - (bx));
        const int jL = (int)std::floor(cy - (by));
        const int jU = (int)std::ceil(cy - (by));
        const int kL = (int)std::floor(cz - (bz));
        const int kU = (int)std::ceil(cz - (bz));
        const bool add = !(iL < 0 || jL < 0 || kL < 0 || iU >= S || jU >= S ||
                           kU >= Z);
        if (add) {
          // :161-170
          const float wxx = cx - bx - iL + 0.5f;
          const float wyy = cy - by - jL + 0.5f;
          const float wz = cz - bz - kL + 0.5f;
          const float wzz = 1 - wz;
          const float d0 = p * step * wxx * wyy * wzz;
          const float d1 = p * step * wxx * wyy * wz;
          const size_t base = (size_t)jL * S + (size_t)iL;
          acc[base + (size_t)kL * S * S] += (double)d0;
          acc[base + (size_t)kU * S * S] += (double)d1;
        }
        cx += ray.dx;
        cy += ray.dy;
        cz += ray.dz;
      }
    }
  }
  std::memset(vol, 0, N * sizeof(double));
  for (int t = 0; t < nt; ++t) {
    if (part[t].empty()) continue;
#pragma omp parallel for num_threads(nt)
    for (long long i = 0; i < (long long)N; ++i) vol[i] += part[t][i];
  }
  return 0;
}

// CUDAmex_oscIter.cu:362-584 (gateway), :94-136 (zero / update),
// :140-271 (FP + residual), :272-358 (dual BP).  FP64 state.
// With a decoupled detector (Wd >= 1; no counterpart in the reference):
// pre/post are Wd x Hd x nP counts of pitch du x dv, one ray per pixel centre
// (a ray that misses the volume gives l = 0), and the dual BP samples the
// residual views of the detector (border addressing).  Wd < 0: the volume's
// own detector, the reference's operations.
int osc_iter_impl(double* mu, const float* pre, const float* post, int W,
                  int H, int nP, int nSub, const int32_t* picks,
                  const float* angles, float sad, int geom, int Wd, int Hd,
                  float du, float dv) {
  if (!mu || !pre || !post || !angles || W <= 0 || H <= 0 || nP < 0 ||
      nSub <= 0 || !picks)
    return 1;
  if (geom < 0 || geom > 2) return 1;
  const bool det = Wd > 0;
  if (det && (Hd <= 0 || !(du > 0.f) || !(dv > 0.f))) return 1;
  const int DW = det ? Wd : W, DH = det ? Hd : H;
  const float u0 = float(DW - 1) / 2, v0r = float(DH - 1) / 2;
  const float v0 = float(H - 1) / 2;
  const float bx = -(float)W / 2.0f, by = bx, bz = -(float)H / 2.0f;
  const float step = 0.5f;  // :244, every geometry
  const uint32_t hw = (uint32_t)W / 2u - 1u;
  const size_t P = (size_t)DW * DH;
  const size_t N = (size_t)W * W * H;
  std::vector<double> num(N), den(N);
  for (int si = 0; si < nSub; ++si) {
    const int sel = picks[si];
    std::vector<int> views;
    for (long long j = sel; j < nP; j += nSub)
      if (j >= 0) views.push_back((int)j);
    const int nv = (int)views.size();
    std::vector<double> rpre(P * nv), rpost(P * nv);
    // FP + residual (:252-268): pre' = pre e^-l - post, post' = pre e^-l l.
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
    for (long long r = 0; r < (long long)P * nv; ++r) {
      const int vi = (int)(r / P);
      const int pix = (int)(r % P);
      const int view = views[vi];
      const int ix = pix % DW, iy = pix / DW;
      float sb, cb;
      trig(angles[view], &sb, &cb);
      float s[3], e[3];
      if (det)
        std_ray(geom, ix, iy, u0, v0r, sb, cb, sad, sad, s, e, du, dv);
      else
        std_ray(geom, ix, iy, u0, v0r, sb, cb, sad, sad, s, e);
      double l = 0.0;
      if (!det || hits_box(s, e, bx, by, bz)) {
        const Ray ray =
            clip_ray(s[0], s[1], s[2], e[0], e[1], e[2], bx, by, bz, step);
        l = march(ray, step, mu, W, W, H, bx, by, bz, true);
      }
      const double pv = pre[P * view + pix], qv = post[P * view + pix];
      const double ehat = pv * std::exp(-l);
      rpre[r] = ehat - qv;
      rpost[r] = ehat * l;
    }
    // dual BP (:305-356) + update (:119-134), border addressing.
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads())
    for (long long col = 0; col < (long long)W * W; ++col) {
      const int ix = (int)(col % W), iy = (int)(col / W);
      if (!in_circle(ix, iy, hw)) continue;
      for (int iz = 0; iz < H; ++iz) {
        num[(size_t)col + (size_t)W * W * iz] = 0.0;
        den[(size_t)col + (size_t)W * W * iz] = 0.0;
      }
      for (int vi = 0; vi < nv; ++vi) {
        float sb, cb;
        trig(angles[views[vi]], &sb, &cb);
        const double* a = rpre.data() + P * vi;
        const double* b = rpost.data() + P * vi;
        if (g_ref_steps && !det) {
          const BpColF c = bp_column_ref(geom, ix, iy, hw, v0, sb, cb, sad);
          float pz = c.pz0;
          for (int iz = 0; iz < H; ++iz) {
            const size_t idx = (size_t)col + (size_t)W * W * iz;
            num[idx] += (double)c.wgt * tex2(a, W, H, (double)c.py, (double)pz, true);
            den[idx] += (double)c.wgt * tex2(b, W, H, (double)c.py, (double)pz, true);
            pz += c.dpz;
          }
          continue;
        }
        const BpCol c = det ? bp_column(geom, ix, iy, hw, v0, sb, cb, sad, DW, DH, du, dv)
                            : bp_column(geom, ix, iy, hw, v0, sb, cb, sad);
        for (int iz = 0; iz < H; ++iz) {
          const double pz = c.pz0 + c.dpz * iz;
          const size_t idx = (size_t)col + (size_t)W * W * iz;
          num[idx] += c.wgt * tex2(a, DW, DH, c.py, pz, true);
          den[idx] += c.wgt * tex2(b, DW, DH, c.py, pz, true);
        }
      }
      for (int iz = 0; iz < H; ++iz) {
        const size_t idx = (size_t)col + (size_t)W * W * iz;
        const double f = mu[idx];
        mu[idx] = std::fmax(f + (f * num[idx] / den[idx]), 0.0);
      }
    }
  }
  return 0;
}

int orc_osc_iter(double* mu, const float* pre, const float* post, int W,
                 int H, int nP, int nSub, const int32_t* picks,
                 const float* angles, float sad, int geom) {
  return osc_iter_impl(mu, pre, post, W, H, nP, nSub, picks, angles, sad, geom, -1, -1, 1.0f,
                       1.0f);
}

int orc_osc_iter_det(double* mu, const float* pre, const float* post, int W,
                     int H, int nP, int nSub, const int32_t* picks,
                     const float* angles, float sad, int geom, int Wd, int Hd,
                     float du, float dv) {
  if (Wd <= 0) return 1;
  return osc_iter_impl(mu, pre, post, W, H, nP, nSub, picks, angles, sad, geom, Wd, Hd, du, dv);
}

// The OSC forward pass alone (CUDAmex_oscIter.cu:140-259): every geometry
// with step 0.5 and border addressing.  mu [W,W,H] (FP64) -> out [W,H,nP].
int orc_osc_fp(const double* mu, int W, int H, float sad, const float* angles,
               int nP, int geom, double* out) {
  if (!mu || !angles || !out || W <= 0 || H <= 0 || nP < 0) return 1;
  if (geom < 0 || geom > 2) return 1;
  const float u0 = float(W - 1) / 2, v0 = float(H - 1) / 2;
  const float bx = -(float)W / 2.0f, by = bx, bz = -(float)H / 2.0f;
  const float step = 0.5f;
  const long long P = (long long)W * H;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
  for (long long r = 0; r < P * nP; ++r) {
    const int view = (int)(r / P);
    const int pix = (int)(r % P);
    float sb, cb;
    trig(angles[view], &sb, &cb);
    float s[3], e[3];
    std_ray(geom, pix % W, pix / W, u0, v0, sb, cb, sad, sad, s, e);
    const Ray ray = clip_ray(s[0], s[1], s[2], e[0], e[1], e[2], bx, by, bz, step);
    out[r] = march(ray, step, mu, W, W, H, bx, by, bz, true);
  }
  return 0;
}

int orc_tv_gradient(const double* in, int Nx, int Ny, int Nz, double* out) {
  if (!in || !out || Nx <= 0 || Ny <= 0 || Nz <= 0) return 1;
  const size_t sx = 1, sy = (size_t)Nx, sz = (size_t)Nx * Ny;
  const double eps = (double)1.0e-6f;  // float eps = 1.0e-6 (:124)
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (long long iz = 0; iz < Nz; ++iz) {
    for (int iy = 0; iy < Ny; ++iy) {
      for (int ix = 0; ix < Nx; ++ix) {
        const size_t i = ix * sx + iy * sy + iz * sz;
        // :121 interior only; the reference leaves the border unwritten
        // (uninitialised), defined here as 0.
        if (!(ix >= 1 && iy >= 1 && iz >= 1 && ix < Nx - 1 && iy < Ny - 1 &&
              iz < Nz - 1)) {
          out[i] = 0.0;
          continue;
        }
        const double x = in[i];
        const double xm = in[i - sx], xp = in[i + sx];
        const double ym = in[i - sy], yp = in[i + sy];
        const double zm = in[i - sz], zp = in[i + sz];
        const double xmyp = in[i - sx + sy], xpym = in[i + sx - sy];
        const double ymzp = in[i - sy + sz], ypzm = in[i + sy - sz];
        const double xmzp = in[i - sx + sz], xpzm = in[i + sx - sz];
        // :146-152
        double t = ((x - xm) + (x - ym) + (x - zm)) /
                   (eps + std::sqrt((x - xm) * (x - xm) + (x - ym) * (x - ym) +
                                    (x - zm) * (x - zm)));
        t -= (xp - x) / (eps + std::sqrt((xp - x) * (xp - x) +
                                         (xp - xpym) * (xp - xpym) +
                                         (xp - xpzm) * (xp - xpzm)));
        t -= (yp - x) / (eps + std::sqrt((yp - x) * (yp - x) +
                                         (yp - xmyp) * (yp - xmyp) +
                                         (yp - ypzm) * (yp - ypzm)));
        t -= (zp - x) / (eps + std::sqrt((zp - x) * (zp - x) +
                                         (zp - xmzp) * (zp - xmzp) +
                                         (zp - ymzp) * (zp - ymzp)));
        out[i] = t;
      }
    }
  }
  return 0;
}

// CUDAmex_TVmin_3D.cu:221-234: n_steps of x <- x + (-c/||g||) g.
int orc_tvmin3d(double* vol, int Nx, int Ny, int Nz, double c, int n_steps) {
  if (!vol || Nx <= 0 || Ny <= 0 || Nz <= 0 || n_steps < 0) return 1;
  const size_t N = (size_t)Nx * Ny * Nz;
  std::vector<double> g(N);
  for (int it = 0; it < n_steps; ++it) {
    orc_tv_gradient(vol, Nx, Ny, Nz, g.data());
    double ss = 0.0;
#pragma omp parallel for reduction(+ : ss) num_threads(nthreads())
    for (long long i = 0; i < (long long)N; ++i) ss += g[i] * g[i];
    const double a = -c / std::sqrt(ss);
#pragma omp parallel for num_threads(nthreads())
    for (long long i = 0; i < (long long)N; ++i) vol[i] = a * g[i] + vol[i];
  }
  return 0;
}

// OSC_TV_recon.m:76-78 (MATLAB round = half away from zero).  A one-iteration
// run divides 0 by 0 in the reference; it uses s_final here.
int orc_num_subsets(int s_init, int s_final, double p_val, int max_iters,
                    int k) {
  if (max_iters <= 1) return s_final;
  const double v = (double)(s_init - s_final) /
                       std::pow((double)(max_iters - 1), p_val) *
                       std::pow((double)(max_iters - k), p_val) +
                   (double)s_final;
  return (int)std::round(v);
}

// OSC_TV_recon.m:80-102 with the randperm first pick given (0-based).
int orc_subset_order(int n, int first, int32_t* picks) {
  if (n <= 0 || first < 0 || first >= n || !picks) return 1;
  std::vector<int> nums(n);
  for (int i = 0; i < n; ++i) nums[i] = i + 1;
  int cur = first + 1;
  picks[0] = cur - 1;
  for (int s = 2; s <= n; ++s) {
    std::vector<int> lo, hi;
    for (int v : nums) {
      if (v < cur) lo.push_back(v);
      if (v > cur) hi.push_back(v);
    }
    std::vector<int>& side = (lo.size() > hi.size()) ? lo : hi;
    if (side.empty()) return 2;
    const size_t pos = (side.size() + 1) / 2 - 1;  // ceil(n/2), 1-based
    cur = side[pos];
    side.erase(side.begin() + pos);
    nums.clear();
    nums.insert(nums.end(), lo.begin(), lo.end());
    nums.insert(nums.end(), hi.begin(), hi.end());
    picks[s - 1] = cur - 1;
  }
  return 0;
}

// OSC_TV_recon.m:33-74 (display omitted).
int orc_osc_tv(const float* pre_in, const float* post_in, int W, int H,
               int nP, const float* angles, float sad, int geom, int n_iter,
               double tv_const, int n_sub_init, int n_sub_final, double p_val,
               const int32_t* first_picks, double* mu_out, orc_iter_cb cb,
               void* user) {
  if (!pre_in || !post_in || !angles || !mu_out || !first_picks ||
      n_iter < 0 || W <= 0 || H <= 0 || nP <= 0)
    return 1;
  const size_t N = (size_t)W * W * H;
  const size_t M = (size_t)W * H * nP;
  // :33 mu = 1e-10 (single)
  for (size_t i = 0; i < N; ++i) mu_out[i] = (double)1e-10f;
  // :35-37 clamp to epsilon = 1e-6
  std::vector<float> pre(M), post(M);
  for (size_t i = 0; i < M; ++i) {
    pre[i] = pre_in[i] < 1e-6 ? (float)1e-6 : pre_in[i];
    post[i] = post_in[i] < 1e-6 ? (float)1e-6 : post_in[i];
  }
  // :41,62 from iteration 2 on, element (1) of pre and post is 0.
  std::vector<float> pre2(pre), post2(post);
  pre2[0] = 0.f;
  post2[0] = 0.f;
  std::vector<double> mu_old(N);
  for (int k = 1; k <= n_iter; ++k) {
    std::memcpy(mu_old.data(), mu_out, N * sizeof(double));
    mu_old[0] = 0.0;  // :45 mu_old(1) = 0
    const int nsub =
        orc_num_subsets(n_sub_init, n_sub_final, p_val, n_iter, k);
    if (nsub <= 0) return 3;
    std::vector<int32_t> picks(nsub);
    int fp = first_picks[k - 1];
    if (fp < 0 || fp >= nsub) fp = ((fp % nsub) + nsub) % nsub;
    if (orc_subset_order(nsub, fp, picks.data())) return 4;
    const float* a = (k == 1) ? pre.data() : pre2.data();
    const float* b = (k == 1) ? post.data() : post2.data();
    int rc = orc_osc_iter(mu_out, a, b, W, H, nP, nsub, picks.data(), angles,
                          sad, geom);
    if (rc) return rc;
    if (k > 1) {
      // :65-67 d_a = ||mu_old - mu||, NaN differences dropped
      double ss = 0.0;
      for (size_t i = 0; i < N; ++i) {
        const double d = mu_old[i] - mu_out[i];
        if (!std::isnan(d)) ss += d * d;
      }
      const double d_a = std::sqrt(ss);
      rc = orc_tvmin3d(mu_out, W, W, H, tv_const * d_a, 20);  // :68
      if (rc) return rc;
      for (size_t i = 0; i < N; ++i)  // :69-70
        if (!std::isfinite(mu_out[i])) mu_out[i] = 0.0;
    }
    if (cb) cb(k, mu_out, user);
  }
  return 0;
}

// designFilter (preFilterSinogram.m:95-152).
int orc_filter_response(int W, int filter, double d, double* Hout, int cap) {
  if (W <= 0 || filter < 0 || filter > 5) return -1;
  int order = 64;
  while (order < 2 * W) order *= 2;  // max(64, 2^nextpow2(2*len))
  if (order > cap || !Hout) return -order;
  if (filter == 0) {
    for (int i = 0; i < order; ++i) Hout[i] = 1.0;
    return order;
  }
  const double pi = 3.14159265358979323846;
  const int half = order / 2;
  std::vector<double> h(order, 0.0);
  // :117-121 band-limited ramp impulse response, symmetric extension
  std::vector<double> hr(half + 1, 0.0);
  hr[0] = 0.25;
  for (int n = 1; n <= half; n += 2) hr[n] = -1.0 / ((pi * n) * (pi * n));
  for (int n = 0; n <= half; ++n) h[n] = hr[n];
  for (int n = 1; n < half; ++n) h[half + n] = hr[half - n];
  // :122-123 filt = 2*real(fft(h)), first half+1 entries
  std::vector<double> filt(half + 1);
  for (int m = 0; m <= half; ++m) {
    double acc = 0.0;
    for (int n = 0; n < order; ++n) {
      const long long ph = ((long long)m * n) % order;
      acc += h[n] * std::cos(2.0 * pi * (double)ph / order);
    }
    filt[m] = 2.0 * acc;
  }
  for (int m = 1; m <= half; ++m) {
    const double w = 2.0 * pi * m / order;  // :125
    switch (filter) {
      case 1:
        break;
      case 2:
        filt[m] *= std::sin(w / (2 * d)) / (w / (2 * d));
        break;
      case 3:
        filt[m] *= std::cos(w / (2 * d));
        break;
      case 4:
        filt[m] *= (.54 + .46 * std::cos(w / d));
        break;
      case 5:
        filt[m] *= (1 + std::cos(w / d)) / 2;
        break;
    }
  }
  for (int m = 0; m <= half; ++m)
    if (2.0 * pi * m / order > pi * d) filt[m] = 0.0;  // :151
  for (int m = 0; m <= half; ++m) Hout[m] = filt[m];  // :152
  for (int m = 1; m < half; ++m) Hout[half + m] = filt[half - m];
  return order;
}

namespace {
double s_function(double b) {  // parker_weight.m:233-240
  if (std::fabs(b) < 0.5) return 0.5 * (1 + std::sin(3.14159265358979323846 * b));
  if (b >= 0.5) return 1.0;
  return 0.0;  // b <= -0.5, or NaN (the zeros() default)
}
}  // namespace

// parker_weight.m:29-72: the Parker window per view i and row element j
// (W of them: the reference computes alpha over size(sino, 2) = H = W).
int orc_parker_window(int W, int nP, const float* angles, int geom, double sad, double q,
                      double* out) {
  if (!angles || !out || W <= 0 || nP < 1 || geom < 0 || geom > 2) return 1;
  const double pi = 3.14159265358979323846;
  std::vector<double> alpha(W, 0.0);  // :29-32
  if (geom != 0)
    for (int j = 0; j < W; ++j) alpha[j] = std::atan((-W / 2.0 + 0.5 + j) / sad);
  bool incr = true;  // :36-39, all(diff(angles) >= 0)
  for (int i = 1; i < nP; ++i)
    if (!(angles[i] - angles[i - 1] >= 0)) incr = false;
  if (incr)
    for (int j = 0; j < W; ++j) alpha[j] = -alpha[j];
  const double delta = std::fabs(alpha[W - 1] - alpha[0]) / 2;  // :42-43
  const double extent = std::fabs((double)(angles[nP - 1] - angles[0]));
  const double eps = std::max(extent - (pi + 2 * delta), 0.0);  // :59
  auto b2 = [&](double a) { return q * (2 * delta - 2 * a + eps); };  // :96-99
  for (int i = 0; i < nP; ++i) {  // :64-70
    const double beta = std::fabs((double)(angles[i] - angles[0]));
    for (int j = 0; j < W; ++j) {
      const double a = alpha[j];
      out[(size_t)i * W + j] =
          0.5 * (s_function(beta / b2(a) - 0.5) +
                 s_function((beta - 2 * delta + 2 * a - eps) / b2(a) + 0.5) -
                 s_function((beta - pi + 2 * a) / b2(-a) - 0.5) -
                 s_function((beta - pi - 2 * delta - eps) / b2(-a) + 0.5));
    }
  }
  return 0;
}

// preFilterSinogram.m:29-90 with parker_weight.m:28-98.
int orc_prefilter(const float* sino, int W, int H, int nP,
                  const float* angles, int geom, double sad, int filter,
                  double cutoff, double q, double* out) {
  if (!sino || !angles || !out || W <= 0 || H <= 0 || nP < 2) return 1;
  if (geom < 0 || geom > 2) return 1;
  if (W != H) return 2;  // parker_weight.m:225 needs a square detector
  const double pi = 3.14159265358979323846;
  const size_t P = (size_t)W * H;
  std::vector<double> Hf(1 << 16);
  const int order = orc_filter_response(W, filter, cutoff, Hf.data(),
                                        (int)Hf.size());
  if (order <= 0) return 3;
  // Spatial kernel k = real(ifft(H)).
  std::vector<double> kern(order);
  for (int n = 0; n < order; ++n) {
    double acc = 0.0;
    for (int m = 0; m < order; ++m) {
      const long long ph = ((long long)m * n) % order;
      acc += Hf[m] * std::cos(2.0 * pi * (double)ph / order);
    }
    kern[n] = acc / order;
  }
  // Parker weights (parker_weight.m:29-72), indexed by the row u.
  std::vector<double> win((size_t)nP * W);
  orc_parker_window(W, nP, angles, geom, sad, q, win.data());
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
  for (long long r = 0; r < (long long)H * nP; ++r) {
    const int i = (int)(r / H), v = (int)(r % H);
    std::vector<double> x(W);
    for (int u = 0; u < W; ++u) {
      double w = (double)sino[P * i + (size_t)W * v + u];
      const double U = (u + 1) - (W - 1) / 2.0;  // :40-41,54-56 (1-based)
      const double V = (v + 1) - (H - 1) / 2.0;
      if (geom == 1) w *= sad / std::sqrt(sad * sad + U * U);
      if (geom == 2) w *= sad / std::sqrt(sad * sad + U * U + V * V);
      x[u] = w * win[(size_t)i * W + u];
    }
    const double dbeta =
        (i > 0) ? (double)(angles[i] - angles[i - 1]) / 2
                : (double)(angles[1] - angles[0]) / 2;  // :80-84
    for (int u = 0; u < W; ++u) {
      double acc = 0.0;
      for (int j = 0; j < W; ++j) acc += x[j] * kern[(u - j + order) % order];
      out[P * i + (size_t)W * v + u] = acc * dbeta;
    }
  }
  return 0;
}

}  // extern "C"
