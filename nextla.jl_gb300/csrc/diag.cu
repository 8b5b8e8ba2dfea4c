// diag.cu -- launch counting, trailing-update timing and the FP64 peak probe.
//
// These are measurement hooks for benchmarks, not part of NextLA's API:
//   tqr_launch_count()      kernels this library has launched so far
//   tqr_profile_enable(on)  time every trailing-update launch (band tsmqr /
//                           unmqr of the tile driver) with CUDA events on the
//                           stream it runs on
//   tqr_profile_read(...)   launches, summed device time and summed
//                           algorithmic flops of the timed launches
//   tqr_fp64_peak_probe     a DFMA throughput kernel: 16 * iters * blocks *
//                           threads flops of independent FMA chains, the FP64
//                           ceiling a SIMT kernel can reach on this GPU
//   tqr_fp64_mma_probe      the FP64 tensor-core (DMMA) counterpart: warps
//                           issue independent mma.sync.m8n8k4.f64 chains, or a
//                           chosen number of warps per CTA run DMMA while the
//                           others run DFMA chains, to show whether the two
//                           paths add up
#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

static std::atomic<unsigned long long> g_launches{0};

void count_launch(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

struct ProfRec {
  cudaEvent_t a, b;
  double flops;
};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<ProfRec> g_prof_live;
static std::vector<cudaEvent_t> g_prof_pool;

static cudaEvent_t pool_get() {
  if (!g_prof_pool.empty()) {
    cudaEvent_t e = g_prof_pool.back();
    g_prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

bool profiling() { return g_prof_on; }

void *prof_begin(cudaStream_t st) {
  std::lock_guard<std::mutex> l(g_prof_mu);
  if (!g_prof_on) return nullptr;
  cudaEvent_t a = pool_get();
  cudaEventRecord(a, st);
  return (void *)a;
}

void prof_end(void *tok, cudaStream_t st, double flops) {
  if (!tok) return;
  std::lock_guard<std::mutex> l(g_prof_mu);
  cudaEvent_t b = pool_get();
  cudaEventRecord(b, st);
  g_prof_live.push_back({(cudaEvent_t)tok, b, flops});
}

__global__ void __launch_bounds__(256) k_fp64_probe(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// 256 threads = 8 warps per CTA.  Warps below dmma_warps run 4 independent
// accumulator chains of mma.sync.m8n8k4.f64 (512 flops per warp and MMA);
// the others run 8 independent DFMA chains per thread (2 flops per lane and
// FMA).  Each warp writes its accumulators so nothing is dead code.
__global__ void __launch_bounds__(256) k_fp64_mma_probe(double *out, int iters, int dmma_warps, double a,
                                                         double b) {
  const int warp = threadIdx.x >> 5;
  const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (warp < dmma_warps) {
    double d[4][2];
    for (int c = 0; c < 4; ++c) { d[c][0] = threadIdx.x + c; d[c][1] = threadIdx.x - c; }
    const double fa = a * (1 + (threadIdx.x & 3)), fb = b;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < 4; ++c)
        asm volatile(
            "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
            : "+d"(d[c][0]), "+d"(d[c][1])
            : "d"(fa), "d"(fb));
    }
    out[o] = d[0][0] + d[0][1] + d[1][0] + d[1][1] + d[2][0] + d[2][1] + d[3][0] + d[3][1];
  } else {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
           x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[o] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  }
}

}  // namespace tqr

extern "C" {

unsigned long long tqr_launch_count(void) { return tqr::g_launches.load(); }

void tqr_profile_enable(int on) {
  std::lock_guard<std::mutex> l(tqr::g_prof_mu);
  tqr::g_prof_on = (on != 0);
}

int tqr_profile_read(long long *launches, double *device_ms, double *flops) {
  std::lock_guard<std::mutex> l(tqr::g_prof_mu);
  long long n = 0;
  double ms = 0, fl = 0;
  for (auto &r : tqr::g_prof_live) {
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e != cudaSuccess) return (int)e;
    float t = 0;
    cudaEventElapsedTime(&t, r.a, r.b);
    ms += t;
    fl += r.flops;
    ++n;
    tqr::g_prof_pool.push_back(r.a);
    tqr::g_prof_pool.push_back(r.b);
  }
  tqr::g_prof_live.clear();
  if (launches) *launches = n;
  if (device_ms) *device_ms = ms;
  if (flops) *flops = fl;
  return 0;
}

int tqr_fp64_peak_probe(int blocks, int iters, double *out, cudaStream_t stream) {
  if (blocks <= 0) return -1;
  if (iters <= 0) return -2;
  if (!out) return -3;
  tqr::k_fp64_probe<<<blocks, 256, 0, stream>>>(out, iters, 1.0000001, 1e-9);
  tqr::count_launch(1);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

}  // extern "C"

extern "C" int tqr_fp64_mma_probe(int blocks, int iters, int dmma_warps, double *out, double *dmma_flops,
                                  double *dfma_flops, cudaStream_t stream) {
  if (blocks <= 0) return -1;
  if (iters <= 0) return -2;
  if (dmma_warps < 0 || dmma_warps > 8) return -3;
  if (!out) return -4;
  // scale factors of magnitude one keep the chains finite for any iters
  tqr::k_fp64_mma_probe<<<blocks, 256, 0, stream>>>(out, iters, dmma_warps, 0.999999999, 1e-12);
  tqr::count_launch(1);
  if (dmma_flops) *dmma_flops = (double)blocks * dmma_warps * 4.0 * iters * 512.0;
  if (dfma_flops) *dfma_flops = (double)blocks * (8 - dmma_warps) * 32.0 * 8.0 * iters * 2.0;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}
