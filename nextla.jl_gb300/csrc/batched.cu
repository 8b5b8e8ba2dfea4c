// batched.cu -- thousands of independent QR / least-squares problems of uneven
// size in one persistent launch.
//
// NextLA has no batched form; each problem here is the composition of its
// single-tile kernels on one m-by-n tile: geqrt! (src/geqrt.jl:22-68), the
// Q^T application of unmqr! (src/unmqr.jl:52-149) to the k right-hand sides,
// and the upper-triangular solve of LeftUpperTRSM! (src/trsm.jl:36-63,
// upper_left_kernel).  The right-hand sides ride along as extra columns of
// every ib-block's trailing update, which is the arithmetic of unmqr! run
// after geqrt! (the same reflectors applied block by block in the same order).
//
// Scheduling: a CTA owns one problem at a time and takes the next one from an
// atomic counter running over a host-made order (most flops first), so big
// problems start early and small ones fill the tail.  One launch covers the
// whole batch, allocates nothing and syncs with nothing, and its counter and
// per-CTA scratch live in the caller's workspace; a tiny reset kernel clears
// the counter, so reset + solve capture into a CUDA graph that is replayed as
// is (tqr_batched_graph).
//
// Tuning: the inner block size ib and the trailing-update strip width (8 or
// 16 columns) are chosen per problem from a table indexed by the column
// count, which tqr_batched_autotune fills by timing candidates on synthetic
// problems of each size class.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <vector>

#include "apply_dev.cuh"
#include "panel_dev.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

// Layout shared with the host bindings (include/tileqr.h).
struct BatchProblem {
  int m, n, k;            // rows, columns, right-hand sides
  int ib, nw;             // inner block size, trailing-update strip width
  int pad;
  long long a_off;        // A at A + a_off, column-major, lda = m
  long long b_off;        // B at B + b_off, column-major, ldb = m; X returns in rows 0:n
};
static_assert(sizeof(BatchProblem) == 40, "BatchProblem layout");

constexpr int kBatchMaxM = TQR_BATCH_MAX_M;
constexpr int kBatchMaxK = TQR_BATCH_MAX_K;
constexpr int kBatchMaxIb = 32;
// dynamic shared memory of the launch: two CTAs per SM
constexpr size_t kBatchSmem = 110 * 1024;
constexpr int kScrElems = kBatchMaxIb * kBatchMaxIb + kBatchMaxM;   // T block + tau per CTA

struct BatchHeader {           // first 256 bytes of the workspace
  int next;                    // problem counter (cleared before every launch)
  int bad;                     // descriptors rejected by the kernel
  int first_bad;               // smallest rejected problem index (INT_MAX if none)
  int pad[61];
};
static_assert(sizeof(BatchHeader) == 256, "BatchHeader layout");

__host__ __device__ inline bool problem_ok(const BatchProblem &p) {
  return p.m >= 1 && p.m <= kBatchMaxM && p.n >= 1 && p.n <= p.m && p.k >= 0 && p.k <= kBatchMaxK &&
         p.ib >= 1 && p.ib <= kBatchMaxIb && (p.nw == 8 || p.nw == 16) && p.a_off >= 0 && p.b_off >= 0;
}

template <typename R, int NW>
__device__ void update_columns(ApplyArgs<R> a, R *C, int ldc, int ncols, unsigned char *smem) {
  a.C = C; a.c_cs = ldc; a.ncols = ncols; a.nw = NW;
  for (int c0 = 0; c0 < ncols; c0 += NW) {
    apply_strip<R, NW>(a, c0, smem);
    __syncthreads();
  }
}

// One problem, one CTA: blocked Householder QR of A with the reflectors also
// applied to B, then R X = (Q^T B)[0:n] in place of B's first n rows.
template <typename R>
__device__ void solve_one(const BatchProblem &p, R *Abase, R *Bbase, R *Tscr, R *tauscr, unsigned char *smem)
{
  const int m = p.m, n = p.n, k = p.k, ib = p.ib;
  R *A = Abase + p.a_off;
  R *B = Bbase + p.b_off;
  const int lda = m, ldb = m;
  for (int i = 0; i < n; i += ib) {
    const int sb = min(ib, n - i);
    const int L = m - i;
    const bool pst = panel_smem<R>(L, sb, true, true) <= kBatchSmem;
    panel_qr_cta<R>(L, sb, A + ix(i, i, lda), lda, tauscr + i, Tscr, ib, pst, true, smem);
    ApplyArgs<R> a;
    a.mode = 0; a.L = L; a.k = sb; a.ib = sb; a.fwd = 1; a.transT = 1;
    a.c_rs = 1; a.A1 = nullptr; a.a_rs = 1; a.a_cs = 1;
    a.V = A + ix(i, i, lda); a.ldv = lda;
    a.T = Tscr; a.ldt = ib;
    a.stage_t = 1;
    const int nw = p.nw;
    const bool full = apply_smem_elems(L, sb, nw, true, true, true) * sizeof(R) <= kBatchSmem;
    a.stage_v = full;
    a.stage_c = full || apply_smem_elems(L, sb, nw, true, false, true) * sizeof(R) <= kBatchSmem;
    const int nt = n - i - sb;
    if (nw == 16) {
      if (nt > 0) update_columns<R, 16>(a, A + ix(i, i + sb, lda), lda, nt, smem);
      if (k > 0) update_columns<R, 16>(a, B + i, ldb, k, smem);
    } else {
      if (nt > 0) update_columns<R, 8>(a, A + ix(i, i + sb, lda), lda, nt, smem);
      if (k > 0) update_columns<R, 8>(a, B + i, ldb, k, smem);
    }
  }
  if (k == 0) return;
  // LeftUpperTRSM! arithmetic: x = b ./ diag, then for i = n..1:
  // x[r] -= (R[r,i] / R[r,r]) x[i] for r < i
  R *xs = reinterpret_cast<R *>(smem);        // n x k
  R *dg = xs + (size_t)n * k;                 // n
  for (int r = threadIdx.x; r < n; r += TQR_THREADS) dg[r] = A[ix(r, r, lda)];
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * k; idx += TQR_THREADS) {
    const int r = idx % n, c = idx / n;
    xs[r + (size_t)c * n] = div_(B[ix(r, c, ldb)], dg[r]);
  }
  __syncthreads();
  for (int i = n - 1; i > 0; --i) {
    for (int idx = threadIdx.x; idx < i * k; idx += TQR_THREADS) {
      const int r = idx % i, c = idx / i;
      xs[r + (size_t)c * n] -= div_(A[ix(r, i, lda)], dg[r]) * xs[i + (size_t)c * n];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < n * k; idx += TQR_THREADS) {
    const int r = idx % n, c = idx / n;
    B[ix(r, c, ldb)] = xs[r + (size_t)c * n];
  }
  __syncthreads();
}

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS, 2)
k_batched_gels(int nprob, const BatchProblem *__restrict__ probs, const int *__restrict__ order, R *A, R *B,
               BatchHeader *hdr, R *scratch)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_q;
  R *Tscr = scratch + (size_t)blockIdx.x * kScrElems;
  R *tauscr = Tscr + kBatchMaxIb * kBatchMaxIb;
  for (;;) {
    if (threadIdx.x == 0) s_q = atomicAdd(&hdr->next, 1);
    __syncthreads();
    const int q = s_q;
    __syncthreads();
    if (q >= nprob) break;
    const int id = order[q];
    if (id < 0 || id >= nprob) {
      if (threadIdx.x == 0) { atomicAdd(&hdr->bad, 1); atomicMin(&hdr->first_bad, q); }
      continue;
    }
    const BatchProblem p = probs[id];
    if (!problem_ok(p)) {
      if (threadIdx.x == 0) { atomicAdd(&hdr->bad, 1); atomicMin(&hdr->first_bad, id); }
      continue;
    }
    solve_one<R>(p, A, B, Tscr, tauscr, smem_raw);
  }
}

__global__ void k_batch_reset(BatchHeader *hdr) {
  if (threadIdx.x == 0) {
    hdr->next = 0;
    hdr->bad = 0;
    hdr->first_bad = 0x7fffffff;
  }
}

// Launch shape per device and precision, fixed on first use (before any
// capture): grid = resident CTAs per SM x SMs.
struct LaunchCfg {
  int grid = 0;
  cudaError_t err = cudaSuccess;
};
static std::mutex g_cfg_mu;
static LaunchCfg g_cfg[4][64];

// Launch-shape slot of an element type: double, float, ComplexF64, ComplexF32.
template <typename R> constexpr int cfg_slot() {
  return std::is_same<R, double>::value ? 0 : std::is_same<R, float>::value ? 1 : std::is_same<R, cx<double>>::value ? 2 : 3;
}

template <typename R>
static LaunchCfg launch_cfg() {
  int dev = 0;
  LaunchCfg c;
  if ((c.err = cudaGetDevice(&dev)) != cudaSuccess) return c;
  if (dev >= 64) { c.err = cudaErrorInvalidDevice; return c; }
  std::lock_guard<std::mutex> l(g_cfg_mu);
  LaunchCfg &g = g_cfg[cfg_slot<R>()][dev];
  if (g.grid > 0) return g;
  int sms = 0, per_sm = 0;
  if ((c.err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return c;
  if ((c.err = cudaFuncSetAttribute(k_batched_gels<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kBatchSmem)) != cudaSuccess)
    return c;
  if ((c.err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batched_gels<R>, TQR_THREADS,
                                                             kBatchSmem)) != cudaSuccess)
    return c;
  g.grid = sms * std::max(per_sm, 1);
  return g;
}

template <typename R>
static size_t work_bytes(int grid) {
  return sizeof(BatchHeader) + sizeof(R) * (size_t)grid * kScrElems;
}

template <typename R>
static int batched_launch(int nprob, const void *probs, const int *order, R *A, R *B, void *work, size_t lwork,
                          cudaStream_t st) {
  if (nprob < 0) return -1;
  if (nprob > 0 && !probs) return -2;
  if (nprob > 0 && !order) return -3;
  if (nprob > 0 && !A) return -4;
  if (nprob > 0 && !B) return -5;
  if (!work || ((uintptr_t)work & 255)) return -6;
  LaunchCfg c = launch_cfg<R>();
  if (c.err != cudaSuccess) return (int)c.err;
  if (lwork < work_bytes<R>(c.grid)) return -7;
  BatchHeader *hdr = (BatchHeader *)work;
  R *scratch = (R *)((unsigned char *)work + sizeof(BatchHeader));
  k_batch_reset<<<1, 32, 0, st>>>(hdr);
  count_launch();
  if (nprob > 0) {
    const int grid = std::min(c.grid, nprob);
    k_batched_gels<R><<<grid, TQR_THREADS, kBatchSmem, st>>>(nprob, (const BatchProblem *)probs, order, A, B,
                                                             hdr, scratch);
    count_launch();
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

// ---------------------------------------------------------------------------
// Per-problem residual of the least-squares solution (not part of the solve):
//   res = ||A^T (B - A X)||_F / (||A||_F (||A||_F ||X||_F + ||B||_F)),
// computed in FP64 from the original A0, B0 and the solution X (B's layout).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_batched_residual(int nprob, const BatchProblem *__restrict__ probs, const R *A0, const R *B0, const R *X,
                   double *res)
{
  extern __shared__ __align__(16) double rbuf[];         // m x k residual
  __shared__ double red[TQR_WARPS];
  for (int id = blockIdx.x; id < nprob; id += gridDim.x) {
    const BatchProblem p = probs[id];
    if (!problem_ok(p) || p.k == 0) {
      if (threadIdx.x == 0) res[id] = problem_ok(p) ? 0.0 : -1.0;
      continue;
    }
    const int m = p.m, n = p.n, k = p.k;
    const R *A = A0 + p.a_off;
    const R *B = B0 + p.b_off;
    const R *Xp = X + p.b_off;
    double sa = 0, sb = 0, sx = 0;
    for (int idx = threadIdx.x; idx < m * k; idx += TQR_THREADS) {
      const int r = idx % m, c = idx / m;
      double s = (double)B[ix(r, c, m)];
      sb += s * s;
      for (int j = 0; j < n; ++j) s -= (double)A[ix(r, j, m)] * (double)Xp[ix(j, c, m)];
      rbuf[idx] = s;
    }
    for (int idx = threadIdx.x; idx < m * n; idx += TQR_THREADS) {
      const double v = (double)A[idx];
      sa += v * v;
    }
    for (int idx = threadIdx.x; idx < n * k; idx += TQR_THREADS) {
      const double v = (double)Xp[ix(idx % n, idx / n, m)];
      sx += v * v;
    }
    __syncthreads();
    double sg = 0;
    for (int idx = threadIdx.x; idx < n * k; idx += TQR_THREADS) {
      const int j = idx % n, c = idx / n;
      double g = 0;
      for (int r = 0; r < m; ++r) g += (double)A[ix(r, j, m)] * rbuf[r + (size_t)c * m];
      sg += g * g;
    }
    sa = block_sum(sa, red);
    sb = block_sum(sb, red);
    sx = block_sum(sx, red);
    sg = block_sum(sg, red);
    if (threadIdx.x == 0) {
      const double na = sqrt(sa), nb = sqrt(sb), nx = sqrt(sx);
      const double den = na * (na * nx + nb);
      res[id] = den > 0 ? sqrt(sg) / den : sqrt(sg);
    }
    __syncthreads();
  }
}

template <typename R>
static int residual_launch(int nprob, const void *probs, const R *A0, const R *B0, const R *X, double *res,
                           cudaStream_t st) {
  if (nprob < 0) return -1;
  if (nprob == 0) return 0;
  if (!probs || !A0 || !B0 || !X || !res) return -2;
  const size_t sm = sizeof(double) * (size_t)kBatchMaxM * kBatchMaxK;
  cudaError_t e = cudaSuccess;
  if (sm > 48 * 1024)
    e = cudaFuncSetAttribute(k_batched_residual<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return (int)e;
  k_batched_residual<R><<<std::min(nprob, 4096), TQR_THREADS, sm, st>>>(nprob, (const BatchProblem *)probs, A0, B0,
                                                                       X, res);
  count_launch();
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

// ---------------------------------------------------------------------------
// Autotuner table: (ib, strip width) per column-count class
// n in (0,32], (32,64], (64,128], (128,256], (256,512].
// ---------------------------------------------------------------------------
constexpr int kClasses = 5;
struct Tune { int ib, nw; };
static Tune g_table[2][kClasses] = {
    {{16, 8}, {16, 16}, {16, 16}, {32, 16}, {32, 16}},
    {{16, 8}, {16, 16}, {16, 16}, {32, 16}, {32, 16}}};
static bool g_tuned[2] = {false, false};
static std::mutex g_tune_mu;

static int class_of(int n) {
  if (n <= 32) return 0;
  if (n <= 64) return 1;
  if (n <= 128) return 2;
  if (n <= 256) return 3;
  return 4;
}

// Synthetic tuning data: a splitmix64 hash per element mapped to [-1, 1).
template <typename R>
__global__ void k_fill_uniform(long long count, unsigned long long seed, R *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    unsigned long long z = (unsigned long long)i * 0x9E3779B97F4A7C15ull + seed;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    out[i] = (R)((double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0);
  }
}

template <typename R>
static int autotune(cudaStream_t st, int force) {
  const int isf = sizeof(R) == 4;
  std::lock_guard<std::mutex> l(g_tune_mu);
  if (g_tuned[isf] && !force) return 0;
  LaunchCfg c = launch_cfg<R>();
  if (c.err != cudaSuccess) return (int)c.err;
  // class representatives (m, n) and candidate (ib, nw)
  const int shape[kClasses][2] = {{64, 24}, {160, 48}, {256, 96}, {384, 192}, {512, 384}};
  const Tune cand[6] = {{8, 8}, {16, 8}, {16, 16}, {32, 8}, {32, 16}, {24, 16}};
  const int kr = 4;
  const int np = 2 * c.grid;   // two waves of the persistent grid
  const long long maxA = (long long)np * kBatchMaxM * kBatchMaxM;
  const long long maxB = (long long)np * kBatchMaxM * kr;
  const size_t wb = work_bytes<R>(c.grid);
  void *work = nullptr, *dprobs = nullptr;
  int *dorder = nullptr;
  R *dA = nullptr, *dB = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  auto chk = [&](cudaError_t e) { if (rc == 0 && e != cudaSuccess) rc = (int)e; };
  chk(cudaMalloc(&work, wb));
  chk(cudaMalloc(&dprobs, sizeof(BatchProblem) * np));
  chk(cudaMalloc((void **)&dorder, sizeof(int) * np));
  chk(cudaMalloc((void **)&dA, sizeof(R) * maxA));
  chk(cudaMalloc((void **)&dB, sizeof(R) * maxB));
  chk(cudaEventCreate(&e0));
  chk(cudaEventCreate(&e1));
  std::vector<int> order(np);
  std::iota(order.begin(), order.end(), 0);
  if (rc == 0) chk(cudaMemcpyAsync(dorder, order.data(), sizeof(int) * np, cudaMemcpyHostToDevice, st));
  Tune result[kClasses];
  for (int cl = 0; cl < kClasses && rc == 0; ++cl) {
    const int m = shape[cl][0], n = shape[cl][1];
    std::vector<BatchProblem> pr(np);
    float best = 1e30f;
    Tune bt = g_table[isf][cl];
    for (const Tune &t : cand) {
      if (t.ib > n || rc != 0) continue;
      for (int q = 0; q < np; ++q)
        pr[q] = {m, n, kr, t.ib, t.nw, 0, (long long)q * m * n, (long long)q * m * kr};
      chk(cudaMemcpyAsync(dprobs, pr.data(), sizeof(BatchProblem) * np, cudaMemcpyHostToDevice, st));
      float tbest = 1e30f;
      for (int rep = 0; rep < 3 && rc == 0; ++rep) {
        k_fill_uniform<R><<<1024, 256, 0, st>>>((long long)np * m * n, 1234 + rep, dA);
        k_fill_uniform<R><<<256, 256, 0, st>>>((long long)np * m * kr, 99 + rep, dB);
        chk(cudaEventRecord(e0, st));
        if (rc == 0) rc = batched_launch<R>(np, dprobs, dorder, dA, dB, work, wb, st);
        chk(cudaEventRecord(e1, st));
        chk(cudaEventSynchronize(e1));
        float ms = 0;
        chk(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) tbest = std::min(tbest, ms);    // the first run warms up
      }
      if (rc == 0 && tbest < best) { best = tbest; bt = t; }
    }
    result[cl] = bt;
  }
  // the pageable copies above read host vectors that must outlive them
  cudaStreamSynchronize(st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(work); cudaFree(dprobs); cudaFree(dorder); cudaFree(dA); cudaFree(dB);
  if (rc == 0) {
    for (int cl = 0; cl < kClasses; ++cl) g_table[isf][cl] = result[cl];
    g_tuned[isf] = true;
  }
  return rc;
}

}  // namespace tqr

using namespace tqr;

extern "C" {

int tqr_batched_problem_bytes(void) { return (int)sizeof(BatchProblem); }

int tqr_batched_plan(int dtype_bytes, int nprob, const int *m, const int *n, const int *k, void *problems,
                     int *order, long long *a_elems, long long *b_elems) {
  if (dtype_bytes != 4 && dtype_bytes != 8 && dtype_bytes != 16) return -1;
  if (nprob < 0) return -2;
  if (nprob > 0 && (!m || !n || !k || !problems || !order)) return -3;
  if (!a_elems || !b_elems) return -9;
  const int isf = dtype_bytes == 4;
  BatchProblem *P = (BatchProblem *)problems;
  std::vector<double> cost(nprob);
  long long ao = 0, bo = 0;
  for (int q = 0; q < nprob; ++q) {
    BatchProblem p;
    p.m = m[q]; p.n = n[q]; p.k = k[q];
    const Tune t = g_table[isf][class_of(p.n)];
    p.ib = std::min(t.ib, std::max(p.n, 1));
    p.nw = dtype_bytes == 16 ? 8 : t.nw;   // ComplexF64: 8-column strips (16-byte elements)
    p.pad = 0;
    p.a_off = ao; p.b_off = bo;
    if (!problem_ok(p)) return -(1000 + q);           // problem q out of range
    // 32-element alignment of every problem's first element
    ao += ((long long)p.m * p.n + 31) / 32 * 32;
    bo += ((long long)p.m * p.k + 31) / 32 * 32;
    const double mm = p.m, nn = p.n;
    cost[q] = 2 * mm * nn * nn - 2 * nn * nn * nn / 3 + 4 * mm * nn * p.k;
    P[q] = p;
  }
  std::vector<int> ord(nprob);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  std::copy(ord.begin(), ord.end(), order);
  *a_elems = std::max(ao, 1LL);
  *b_elems = std::max(bo, 1LL);
  return 0;
}

int tqr_batched_worksize(int dtype_bytes, size_t *bytes) {
  if (dtype_bytes != 4 && dtype_bytes != 8 && dtype_bytes != 16) return -1;
  if (!bytes) return -2;
  if (dtype_bytes == 16) {
    LaunchCfg c = launch_cfg<cx<double>>();
    if (c.err != cudaSuccess) return (int)c.err;
    *bytes = work_bytes<cx<double>>(c.grid);
    return 0;
  }
  LaunchCfg c = dtype_bytes == 4 ? launch_cfg<float>() : launch_cfg<double>();
  if (c.err != cudaSuccess) return (int)c.err;
  *bytes = dtype_bytes == 4 ? work_bytes<float>(c.grid) : work_bytes<double>(c.grid);
  if (dtype_bytes == 8) {   // also covers ComplexF32 (8-byte elements)
    LaunchCfg cc = launch_cfg<cx<float>>();
    if (cc.err != cudaSuccess) return (int)cc.err;
    *bytes = std::max(*bytes, work_bytes<cx<float>>(cc.grid));
  }
  return 0;
}

int tqr_batched_autotune(int dtype_bytes, int force, cudaStream_t stream) {
  if (dtype_bytes != 4 && dtype_bytes != 8) return -1;
  return dtype_bytes == 4 ? autotune<float>(stream, force) : autotune<double>(stream, force);
}

int tqr_batched_tuning(int dtype_bytes, int n, int *ib, int *nw) {
  if (dtype_bytes != 4 && dtype_bytes != 8) return -1;
  if (n < 1 || n > kBatchMaxM) return -2;
  if (!ib || !nw) return -3;
  const Tune t = g_table[dtype_bytes == 4][class_of(n)];
  *ib = t.ib;
  *nw = t.nw;
  return 0;
}

int tqr_dbatched_gels(int nprob, const void *problems, const int *order, double *A, double *B, void *work,
                      size_t lwork, cudaStream_t stream) {
  return batched_launch<double>(nprob, problems, order, A, B, work, lwork, stream);
}

int tqr_sbatched_gels(int nprob, const void *problems, const int *order, float *A, float *B, void *work,
                      size_t lwork, cudaStream_t stream) {
  return batched_launch<float>(nprob, problems, order, A, B, work, lwork, stream);
}

int tqr_zbatched_gels(int nprob, const void *problems, const int *order, tqr_zcomplex *A, tqr_zcomplex *B,
                      void *work, size_t lwork, cudaStream_t stream) {
  if (((uintptr_t)A | (uintptr_t)B) % alignof(cx<double>)) return -4;
  return batched_launch<cx<double>>(nprob, problems, order, (cx<double> *)A, (cx<double> *)B, work, lwork, stream);
}

int tqr_cbatched_gels(int nprob, const void *problems, const int *order, tqr_ccomplex *A, tqr_ccomplex *B,
                      void *work, size_t lwork, cudaStream_t stream) {
  if (((uintptr_t)A | (uintptr_t)B) % alignof(cx<float>)) return -4;
  return batched_launch<cx<float>>(nprob, problems, order, (cx<float> *)A, (cx<float> *)B, work, lwork, stream);
}

int tqr_batched_status(const void *work, int *bad, int *first_bad, cudaStream_t stream) {
  if (!work || !bad || !first_bad) return -1;
  int h[3];
  cudaError_t e = cudaMemcpyAsync(h, work, sizeof(h), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return (int)e;
  *bad = h[1];
  *first_bad = h[1] ? h[2] : -1;
  return 0;
}

int tqr_dbatched_residual(int nprob, const void *problems, const double *A0, const double *B0, const double *X,
                          double *res, cudaStream_t stream) {
  return residual_launch<double>(nprob, problems, A0, B0, X, res, stream);
}

int tqr_sbatched_residual(int nprob, const void *problems, const float *A0, const float *B0, const float *X,
                          double *res, cudaStream_t stream) {
  return residual_launch<float>(nprob, problems, A0, B0, X, res, stream);
}

int tqr_batched_graph(int dtype_bytes, int nprob, const void *problems, const int *order, void *A, void *B,
                      void *work, size_t lwork, void **graph_exec) {
  if (dtype_bytes != 4 && dtype_bytes != 8) return -1;
  if (!graph_exec) return -9;
  *graph_exec = nullptr;
  // fix the launch shape outside the capture
  LaunchCfg c = dtype_bytes == 4 ? launch_cfg<float>() : launch_cfg<double>();
  if (c.err != cudaSuccess) return (int)c.err;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return (int)e;
  cudaGraph_t g = nullptr;
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  int rc = 0;
  if (e == cudaSuccess) {
    rc = dtype_bytes == 4
             ? batched_launch<float>(nprob, problems, order, (float *)A, (float *)B, work, lwork, s)
             : batched_launch<double>(nprob, problems, order, (double *)A, (double *)B, work, lwork, s);
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (rc == 0 && e2 != cudaSuccess) rc = (int)e2;
  } else {
    rc = (int)e;
  }
  cudaGraphExec_t ex = nullptr;
  if (rc == 0) {
    e = cudaGraphInstantiate(&ex, g, 0);
    if (e != cudaSuccess) rc = (int)e;
  }
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(s);
  if (rc == 0) *graph_exec = (void *)ex;
  return rc;
}

int tqr_batched_graph_launch(void *graph_exec, cudaStream_t stream) {
  if (!graph_exec) return -1;
  cudaError_t e = cudaGraphLaunch((cudaGraphExec_t)graph_exec, stream);
  if (e == cudaSuccess) count_launch(2);
  return e == cudaSuccess ? 0 : (int)e;
}

int tqr_batched_graph_destroy(void *graph_exec) {
  if (!graph_exec) return 0;
  cudaError_t e = cudaGraphExecDestroy((cudaGraphExec_t)graph_exec);
  return e == cudaSuccess ? 0 : (int)e;
}

}  // extern "C"
