// mexct_bench.cpp -- standalone C++ benchmark of libmexct through its C ABI.
//
// The same headline step as bench.py, with nothing but the CUDA runtime and
// include/mexct.h: a cone-beam (geomFlag 2 by default) FP of a float32
// random-ellipsoid volume plus the BP of that sinogram, device-resident
// buffers from cudaMalloc, CUDA events on the launching stream, then the same
// step through the host entry points (mexct_fp / mexct_bp) with pinned host
// buffers, copies inside the timed region.  Prints one JSON line.
//
//   mexct_bench [--size N] [--views V] [--geom G] [--steps K] [--warmup W]
//
// GUPS = 2 * N^3 * views * steps / time (one FP and one BP per step).
#include <cuda_runtime.h>
#include <execinfo.h>
#include <signal.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mexct.h"

namespace {

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));                  \
      std::exit(1);                                                                  \
    }                                                                                \
  } while (0)
#define MK(x)                                                                        \
  do {                                                                               \
    mexct_status s_ = (x);                                                           \
    if (s_ != MEXCT_OK) {                                                            \
      std::fprintf(stderr, "%s: status %d: %s\n", #x, s_, mexct_last_error());       \
      std::exit(1);                                                                  \
    }                                                                                \
  } while (0)

// splitmix64: a seeded stream of uniform doubles in [0, 1).
struct Rng {
  uint64_t s;
  double next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  }
  double uni(double a, double b) { return a + (b - a) * next(); }
};

// Seeded random-ellipsoid phantom [n,n,n] (x fastest): 12 ellipsoids with
// centres in the inner 70 % of the field of view, semi-axes 10..min(150, n/2)
// voxels, random rotations about z and additive values in [-0.01, 0.03],
// clipped at 0.  Only the workload's shape matters for timing.
std::vector<float> phantom(int n, uint64_t seed) {
  std::vector<float> v((size_t)n * n * n, 0.f);
  Rng r{seed};
  const double half = 0.35 * n, amax = std::min(150.0, n / 2.0);
  for (int e = 0; e < 12; ++e) {
    const double cx = r.uni(-half, half), cy = r.uni(-half, half), cz = r.uni(-half, half);
    const double ax = r.uni(10, amax), ay = r.uni(10, amax), az = r.uni(10, amax);
    const double th = r.uni(0, 2 * M_PI), val = r.uni(-0.01, 0.03);
    const double c = std::cos(th), s = std::sin(th);
    const double rmax = std::max(ax, std::max(ay, az));
    const int z0 = std::max(0, (int)std::floor(cz - az + (n - 1) / 2.0));
    const int z1 = std::min(n - 1, (int)std::ceil(cz + az + (n - 1) / 2.0));
    const int y0 = std::max(0, (int)std::floor(cy - rmax + (n - 1) / 2.0));
    const int y1 = std::min(n - 1, (int)std::ceil(cy + rmax + (n - 1) / 2.0));
    const int x0 = std::max(0, (int)std::floor(cx - rmax + (n - 1) / 2.0));
    const int x1 = std::min(n - 1, (int)std::ceil(cx + rmax + (n - 1) / 2.0));
    for (int k = z0; k <= z1; ++k) {
      const double Z = (k - (n - 1) / 2.0 - cz) / az;
      for (int j = y0; j <= y1; ++j) {
        const double Y = j - (n - 1) / 2.0 - cy;
        for (int i = x0; i <= x1; ++i) {
          const double X = i - (n - 1) / 2.0 - cx;
          const double u = (c * X + s * Y) / ax, w = (-s * X + c * Y) / ay;
          if (u * u + w * w + Z * Z <= 1.0) v[(size_t)i + (size_t)n * (j + (size_t)n * k)] += (float)val;
        }
      }
    }
  }
  for (float& x : v) x = std::max(x, 0.f);
  return v;
}

// A crash prints the stage and a backtrace to stderr before the process ends.
const char* volatile g_stage = "start";
void on_fatal(int sig) {
  char msg[160];
  const int n = std::snprintf(msg, sizeof msg, "mexct_bench: signal %d during %s\n", sig, g_stage);
  if (n > 0) (void)!write(2, msg, (size_t)n);
  void* frames[48];
  const int k = backtrace(frames, 48);
  backtrace_symbols_fd(frames, k, 2);
  _exit(128 + sig);
}

}  // namespace

int main(int argc, char** argv) {
  signal(SIGSEGV, on_fatal);
  signal(SIGBUS, on_fatal);
  signal(SIGABRT, on_fatal);
  int n = 512, views = 720, geom = 2, steps = 5, warmup = 3;
  for (int i = 1; i + 1 < argc; i += 2) {
    const std::string a = argv[i];
    const int v = std::atoi(argv[i + 1]);
    if (a == "--size") n = v;
    else if (a == "--views") views = v;
    else if (a == "--geom") geom = v;
    else if (a == "--steps") steps = v;
    else if (a == "--warmup") warmup = v;
    else {
      std::fprintf(stderr, "unknown option %s\n", a.c_str());
      return 2;
    }
  }
  if (n <= 0 || views <= 0 || steps <= 0 || warmup < 0 || geom < 0 || geom > 2) {
    std::fprintf(stderr, "bad arguments\n");
    return 2;
  }
  const size_t N = (size_t)n * n * n, S = (size_t)n * n * views;
  g_stage = "phantom";
  std::vector<float> vol = phantom(n, 2024);
  std::vector<float> ang(views);
  for (int j = 0; j < views; ++j) ang[j] = (float)(2.0 * M_PI * j / (views - 1 > 0 ? views - 1 : 1));

  g_stage = "device set-up";
  CK(cudaSetDevice(0));
  mexct_ctx* ctx = nullptr;
  MK(mexct_ctx_create(0, &ctx));
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  float *d_vol = nullptr, *d_sino = nullptr, *d_rec = nullptr;
  CK(cudaMalloc(&d_vol, N * sizeof(float)));
  CK(cudaMalloc(&d_sino, S * sizeof(float)));
  CK(cudaMalloc(&d_rec, N * sizeof(float)));
  CK(cudaMemcpy(d_vol, vol.data(), N * sizeof(float), cudaMemcpyHostToDevice));
  const float sad = 1000.f;

  g_stage = "warm-up steps";
  auto fp = [&] { MK(mexct_fp_dev(ctx, d_vol, n, n, sad, ang.data(), views, geom, d_sino, st)); };
  auto bp = [&] { MK(mexct_bp_dev(ctx, d_sino, n, n, views, sad, ang.data(), geom, d_rec, st)); };
  for (int i = 0; i < warmup; ++i) {
    fp();
    bp();
  }
  CK(cudaStreamSynchronize(st));
  cudaEvent_t e0, e1, e2;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventCreate(&e2));
  // Per-operator times of one call each.
  CK(cudaEventRecord(e0, st));
  fp();
  CK(cudaEventRecord(e1, st));
  bp();
  CK(cudaEventRecord(e2, st));
  CK(cudaEventSynchronize(e2));
  float fp_ms = 0.f, bp_ms = 0.f;
  CK(cudaEventElapsedTime(&fp_ms, e0, e1));
  CK(cudaEventElapsedTime(&bp_ms, e1, e2));
  // The timed steps.
  g_stage = "timed steps";
  CK(cudaDeviceSynchronize());
  CK(cudaEventRecord(e0, st));
  for (int i = 0; i < steps; ++i) {
    fp();
    bp();
  }
  CK(cudaEventRecord(e1, st));
  CK(cudaEventSynchronize(e1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  const double gups = 2.0 * (double)N * views * steps / (ms / 1e3) / 1e9;

  // End to end through the host entry points, pinned host buffers.
  g_stage = "host entry points";
  float *h_vol = nullptr, *h_sino = nullptr, *h_rec = nullptr;
  CK(cudaMallocHost(&h_vol, N * sizeof(float)));
  CK(cudaMallocHost(&h_sino, S * sizeof(float)));
  CK(cudaMallocHost(&h_rec, N * sizeof(float)));
  std::memcpy(h_vol, vol.data(), N * sizeof(float));
  // each call's host wall time, for the median split of a step
  std::vector<double> t_fp, t_bp;
  auto e2e_step = [&] {
    const auto a = std::chrono::steady_clock::now();
    MK(mexct_fp(ctx, h_vol, n, n, sad, ang.data(), views, geom, h_sino));
    const auto b = std::chrono::steady_clock::now();
    MK(mexct_bp(ctx, h_sino, n, n, views, sad, ang.data(), geom, h_rec));
    const auto c = std::chrono::steady_clock::now();
    t_fp.push_back(std::chrono::duration<double>(b - a).count());
    t_bp.push_back(std::chrono::duration<double>(c - b).count());
  };
  for (int i = 0; i < 2; ++i) e2e_step();  // the first calls grow the context's buffers
  t_fp.clear();
  t_bp.clear();
  const int ke = std::max(1, steps);
  const auto t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < ke; ++i) e2e_step();
  const double es = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  const double e2e = 2.0 * (double)N * views * ke / es / 1e9;
  auto median_ms = [](std::vector<double> v) {
    std::sort(v.begin(), v.end());
    return v.empty() ? 0.0 : 1e3 * v[v.size() / 2];
  };
  const double e2e_fp_ms = median_ms(t_fp), e2e_bp_ms = median_ms(t_bp);

  std::printf(
      "{\"metric\": \"FP+BP GUPS at %d^3 x %d views (geomFlag %d), plain FP32\", \"value\": %.3f, "
      "\"unit\": \"GUPS\", \"n_gpus\": 1, \"steps\": %d, \"warmup\": %d, \"ms_per_step\": %.3f, "
      "\"fp_ms\": %.3f, \"bp_ms\": %.3f, \"dtype\": \"f32\", \"impl\": \"mexct_bench (C++, C ABI, "
      "cudaMalloc buffers)\", \"e2e\": {\"value\": %.3f, \"unit\": \"GUPS\", \"h2d_bytes_per_step\": "
      "%zu, \"d2h_bytes_per_step\": %zu, \"path\": \"mexct_fp + mexct_bp, pinned host buffers\", "
      "\"fp_call_ms_median\": %.3f, \"bp_call_ms_median\": %.3f}}\n",
      n, views, geom, gups, steps, warmup, ms / steps, fp_ms, bp_ms, e2e, 4 * (N + S), 4 * (S + N),
      e2e_fp_ms, e2e_bp_ms);
  std::fflush(stdout);
  g_stage = "clean-up";
  cudaFreeHost(h_vol);
  cudaFreeHost(h_sino);
  cudaFreeHost(h_rec);
  cudaFree(d_vol);
  cudaFree(d_sino);
  cudaFree(d_rec);
  cudaStreamDestroy(st);
  MK(mexct_ctx_destroy(ctx));
  return 0;
}
