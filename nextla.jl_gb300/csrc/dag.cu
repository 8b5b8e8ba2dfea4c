// dag.cu -- the tile QR as one persistent kernel over a task DAG.
//
// The flat-tree tile QR (NextLA's geqrt!/tsqrt!/unmqr!/tsmqr! composed in
// PLASMA order, as the stream driver in tile.cu does) is cut into CTA-sized
// tasks on nw-wide column strips of the nb-by-nb tiles:
//
//   GB(k,b)      geqr2 + T of block b of the diagonal tile (k,k)        1 CTA
//   GA(k,b,s)    block b's reflectors applied to strip s of tile (k,k)   (larfb)
//   UN(k,j,s)    all of (k,k)'s reflectors applied to strip s of (k,j)   (unmqr)
//   TB(k,i,b)    tsqrt block b on [R of (k,k); tile (i,k)]               1 CTA
//   TA(k,i,b,s)  that block applied to strip s of (k,k) and (i,k)        (tsmqr, one block)
//   TM(k,i,j,s)  all of (i,k)'s reflectors applied to strip s of (k,j), (i,j)   (tsmqr)
//   TC(k,i,j,c)  FP32 only: the same for the 128-column chunk c of (k,j), (i,j) on the
//                tcgen05 tensor cores (tc_apply.cuh), in place of its 8 TM strips
//
// One launch with (SMs x resident CTAs) CTAs runs them all.  Each CTA takes
// the next task index from a global counter, waits until the task's inputs
// are written, runs it, and publishes its writes by bumping counters:
//   ver(i,j,s)   number of completed tasks that wrote strip s of tile (i,j)
//   done_g(k)    completed GB/GA tasks of diagonal tile k
//   done_t(k,i)  completed TB/TA tasks of tsqrt(k,i)
// Every writer of a strip is known in advance, so a task's wait targets are
// closed-form counts (item_deps below); the host check tqr_tile_dag_check
// recomputes them by replaying the task list.
//
// Task order: the host sorts the tasks by decreasing longest path to the end
// of the DAG (estimated durations), which is a topological order that runs
// the panel chain first.  Because tasks are taken strictly in that order, the
// lowest unfinished task always has its inputs done, so the schedule cannot
// deadlock even if only some CTAs are resident.  Every wait is still bounded
// by a %globaltimer deadline: on expiry the task sets an error word in the
// workspace and every CTA leaves; the host reads the word with
// tqr_tile_dag_status.
//
// The DAG path needs m, n multiples of nb, nb a multiple of ib and ib a
// multiple of nw (the benchmark shapes); other shapes use the stream driver.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include <type_traits>

#include "apply_dev.cuh"
#include "panel_dev.cuh"
#include "tc_apply.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

enum : uint8_t { IT_GB = 0, IT_GA = 1, IT_UN = 2, IT_TB = 3, IT_TA = 4, IT_TM = 5, IT_TC = 6 };

struct DagItem {
  uint8_t type, b;
  uint16_t k, i, j, s;
  uint16_t pad;
};
static_assert(sizeof(DagItem) == 12, "DagItem layout");

struct DagGeom {
  int m, n, nb, ib, nw;
  int MT, NT, KT, NS, SPB, NBK;
  // Optional right-hand sides: nrhs > 0 adds one tile column (index NTA) of
  // width nrhs that only receives trailing updates, so the factorisation also
  // forms Q^T B.  NTA is the number of tile columns of A.
  int nrhs, NTA;
  // tc = 1: the tsmqr updates of A's tile columns run as TC tasks on NCH
  // chunks of 128 columns (CPS strips each) per tile (FP32, nb = 256, ib = 32)
  int tc, NCH, CPS;
  // f64p = 1 (FP32 only): the panel tasks GB and TB compute in FP64
  // (panel_qr_cta_f64 / tsqrt_block_cta_f64) with the diagonal R triangles
  // kept in an FP64 array after the schedule in the workspace
  int f64p;
  __host__ __device__ int tm_tasks(int j) const { return (tc && j < NTA) ? NCH : strips(j); }
  __host__ __device__ int strips(int j) const { return j < NTA ? NS : (nrhs + nw - 1) / nw; }
  __host__ __device__ int width(int j) const { return j < NTA ? nb : nrhs; }
  __host__ __device__ int ver(int i, int j, int s) const { return (i * NT + j) * NS + s; }
  __host__ __device__ int done_g(int k) const { return MT * NT * NS + k; }
  __host__ __device__ int done_t(int k, int i) const { return MT * NT * NS + KT + k * MT + i; }
  __host__ __device__ int ncounters() const { return MT * NT * NS + KT + KT * MT; }
  // tasks of one geqrt (GB + GA) or one tsqrt (TB + TA)
  __host__ __device__ int panel_tasks() const { return NBK + NBK * NS - SPB * NBK * (NBK + 1) / 2; }
};

constexpr int kMaxDeps = 2 * 16 + 1;

// Wait targets: counter c must reach t before the task may run.
__host__ __device__ inline int item_deps(const DagGeom &g, const DagItem &it, int *c, int *t) {
  int n = 0;
  const int k = it.k, i = it.i, j = it.j, b = it.b, s = it.s;
  switch (it.type) {
    case IT_GB:
      for (int q = b * g.SPB; q < (b + 1) * g.SPB; ++q) { c[n] = g.ver(k, k, q); t[n++] = k + b; }
      break;
    case IT_GA:
      c[n] = g.ver(k, k, s); t[n++] = k + b;
      c[n] = g.ver(k, k, b * g.SPB); t[n++] = k + b + 1;
      break;
    case IT_UN:
      c[n] = g.done_g(k); t[n++] = g.panel_tasks();
      c[n] = g.ver(k, j, s); t[n++] = k;
      break;
    case IT_TB:
      // (k,k): geqrt and each earlier tsqrt wrote b+1 times, this tsqrt b times
      for (int q = b * g.SPB; q < (b + 1) * g.SPB; ++q) {
        c[n] = g.ver(k, k, q); t[n++] = k + (i - k) * (b + 1) + b;
        c[n] = g.ver(i, k, q); t[n++] = k + b;
      }
      break;
    case IT_TA: {
      const int bs = s / g.SPB;
      c[n] = g.ver(k, k, s); t[n++] = k + (i - k) * (bs + 1) + b;
      c[n] = g.ver(i, k, s); t[n++] = k + b;
      c[n] = g.ver(i, k, b * g.SPB); t[n++] = k + b + 1;
      break;
    }
    case IT_TM:
      c[n] = g.done_t(k, i); t[n++] = g.panel_tasks();
      c[n] = g.ver(k, j, s); t[n++] = i;
      c[n] = g.ver(i, j, s); t[n++] = k;
      break;
    case IT_TC:
      c[n] = g.done_t(k, i); t[n++] = g.panel_tasks();
      for (int q = s * g.CPS; q < (s + 1) * g.CPS; ++q) {
        c[n] = g.ver(k, j, q); t[n++] = i;
        c[n] = g.ver(i, j, q); t[n++] = k;
      }
      break;
  }
  return n;
}

// Counters a task bumps when it is done.
__host__ __device__ inline int item_updates(const DagGeom &g, const DagItem &it, int *c) {
  int n = 0;
  const int k = it.k, i = it.i, j = it.j, b = it.b, s = it.s;
  switch (it.type) {
    case IT_GB:
      for (int q = b * g.SPB; q < (b + 1) * g.SPB; ++q) c[n++] = g.ver(k, k, q);
      c[n++] = g.done_g(k);
      break;
    case IT_GA:
      c[n++] = g.ver(k, k, s);
      c[n++] = g.done_g(k);
      break;
    case IT_UN:
      c[n++] = g.ver(k, j, s);
      break;
    case IT_TB:
      for (int q = b * g.SPB; q < (b + 1) * g.SPB; ++q) {
        c[n++] = g.ver(k, k, q);
        c[n++] = g.ver(i, k, q);
      }
      c[n++] = g.done_t(k, i);
      break;
    case IT_TA:
      c[n++] = g.ver(k, k, s);
      c[n++] = g.ver(i, k, s);
      c[n++] = g.done_t(k, i);
      break;
    case IT_TM:
      c[n++] = g.ver(k, j, s);
      c[n++] = g.ver(i, j, s);
      break;
    case IT_TC:
      for (int q = s * g.CPS; q < (s + 1) * g.CPS; ++q) {
        c[n++] = g.ver(k, j, q);
        c[n++] = g.ver(i, j, q);
      }
      break;
  }
  return n;
}

// ---------------------------------------------------------------------------
// Workspace: [header 64 B][counters][items]
// ---------------------------------------------------------------------------
struct DagHeader {
  int head;        // next task index
  int error;       // 0 = ok; 1 = a wait timed out; 2 = schedule/arguments mismatch
  int err_item;    // task index that reported the error
  int err_type;
  long long key;   // geometry key of the uploaded schedule
  int nitems;
  int pad0;
  // statistics (nanoseconds summed over CTAs): time running each task type,
  // time spent waiting for inputs, and the first/last timestamps of the launch
  unsigned long long busy_ns[6];
  unsigned long long wait_ns;
  unsigned long long t_first, t_last;
  unsigned long long pad1[19];
};
static_assert(sizeof(DagHeader) == 256, "DagHeader layout");

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

template <typename R>
struct DagArgs {
  DagGeom g;
  R *A; int lda;
  R *B; int ldb;    // right-hand sides (tile column NTA) when g.nrhs > 0
  R *T; int ldt;
  R *tau; int ldtau;
  DagHeader *hdr;
  int *cnt;
  const DagItem *items;
  int nitems;
  long long key;
  unsigned long long timeout_ns;
  int hold = 0;     // failure-detection test: task 0 also waits for a header word nothing writes
  double *D = nullptr;   // g.f64p: FP64 diagonal R triangles, ib x (KT nb), ld ib
  // g.tc with tma: tensor maps of A for the TC tasks' TMA loads (32 x 128 and
  // 32 x 32 boxes); the kernel takes DagArgs as a __grid_constant__ parameter
  // so their addresses are valid operands
  CUtensorMap tmw, tmn;
  int tma = 0;
};

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Per-CTA tensor-core state of the TC tasks (FP32 only).
struct TcState {
  uint32_t tmem;
  uint64_t *bars;                 // tc::kBars mbarriers
  uint32_t phase[tc::kBars];
};

// Runs one task; false only if a TC task's tensor-core wait gave up.  TC:
// this instantiation carries the tensor-core task (FP32 only).
template <typename R, int NW, bool TC>
__device__ bool run_item(const DagArgs<R> &a, const DagItem &it, unsigned char *smem, TcState *tcs) {
  const DagGeom &g = a.g;
  const int nb = g.nb, ib = g.ib;
  const int k = it.k, i = it.i, j = it.j, b = it.b, s = it.s;
  auto tile = [&](int r, int c) {
    return c < g.NTA ? a.A + ix(r * nb, c * nb, a.lda) : a.B + ix(r * nb, 0, a.ldb);
  };
  auto tld = [&](int c) { return c < g.NTA ? a.lda : a.ldb; };
  auto ttile = [&](int r, int c) { return a.T + ix(r * ib, c * nb, a.ldt); };
  auto tautile = [&](int r, int c) { return a.tau + ix(c * nb, r, a.ldtau); };
  if (it.type == IT_GB) {
    R *Ab = tile(k, k) + ix(b * ib, b * ib, a.lda);
    if constexpr (std::is_same<R, float>::value) {
      if (a.D) {
        panel_qr_cta_f64(nb - b * ib, ib, Ab, a.lda, tautile(k, k) + b * ib, ttile(k, k) + ix(0, b * ib, a.ldt),
                         a.ldt, a.D + (size_t)(k * nb + b * ib) * ib, ib, smem);
        return true;
      }
    }
    panel_qr_cta<R, TC>(nb - b * ib, ib, Ab, a.lda, tautile(k, k) + b * ib, ttile(k, k) + ix(0, b * ib, a.ldt),
                    a.ldt, true, true, smem);
    return true;
  }
  if (it.type == IT_TB) {
    if constexpr (std::is_same<R, float>::value) {
      if (a.D) {
        double *Dk = a.D + (size_t)(k * nb + b * ib) * ib;
        float *A1 = tile(k, k) + ix(b * ib, b * ib, a.lda), *A2 = tile(i, k) + ix(0, b * ib, a.lda);
        float *Tb = ttile(i, k) + ix(0, b * ib, a.ldt), *tb = tautile(i, k) + b * ib;
        if (ib <= 32)
          tsqrt_block_f64x(nb, ib, Dk, ib, A1, a.lda, A2, a.lda, Tb, a.ldt, tb, smem);
        else
          tsqrt_block_cta_f64(nb, ib, Dk, ib, A1, a.lda, A2, a.lda, Tb, a.ldt, tb, smem);
        return true;
      }
    }
    tsqrt_block_cta<R, TC>(nb, ib, tile(k, k) + ix(b * ib, b * ib, a.lda), a.lda, tile(i, k) + ix(0, b * ib, a.lda),
                       a.lda, ttile(i, k) + ix(0, b * ib, a.ldt), a.ldt, tautile(i, k) + b * ib, true, smem);
    return true;
  }
  if (it.type == IT_TC) {
    if constexpr (TC && std::is_same<R, float>::value) {
      unsigned char *al = smem + ((1024 - (tc::saddr(smem) & 1023)) & 1023);
      const size_t c0 = (size_t)s * tc::kChunk;
      const tc::TcMaps mp{&a.tmw, &a.tmw, &a.tmn, k * nb, j * nb + (int)c0, i * nb, j * nb + (int)c0, i * nb, k * nb};
      return tc::tsmqr_chunk(nb, nb, tile(k, j) + c0 * a.lda, a.lda, tile(i, j) + c0 * a.lda, a.lda, tile(i, k),
                             a.lda, ttile(i, k), a.ldt, tcs->tmem, tcs->bars, tcs->phase, al, tc::kVFull,
                             a.tma ? &mp : nullptr);
    } else {
      return false;
    }
  }
  ApplyArgs<R> p;
  p.ib = ib;
  p.fwd = 1;
  p.transT = 1;              // 'L', 'C': blocks forward, W := T^T W
  p.c_rs = 1; p.c_cs = a.lda;
  p.a_rs = 1; p.a_cs = a.lda;
  p.ldv = a.lda;
  p.ldt = a.ldt;
  p.nw = g.nw;
  p.ncols = nb;
  p.stage_c = 1; p.stage_v = 1; p.stage_t = 1;
  p.A1 = nullptr;
  switch (it.type) {
    case IT_GA:
      p.mode = 0; p.L = nb - b * ib; p.k = ib;
      p.C = tile(k, k) + ix(b * ib, 0, a.lda);
      p.V = tile(k, k) + ix(b * ib, b * ib, a.lda);
      p.T = ttile(k, k) + ix(0, b * ib, a.ldt);
      break;
    case IT_UN:
      p.mode = 0; p.L = nb; p.k = nb;
      p.C = tile(k, j);
      p.c_cs = tld(j);
      p.ncols = g.width(j);
      p.V = tile(k, k);
      p.T = ttile(k, k);
      break;
    case IT_TA:
      p.mode = 1; p.L = nb; p.k = ib;
      p.C = tile(i, k);
      p.A1 = tile(k, k) + ix(b * ib, 0, a.lda);
      p.V = tile(i, k) + ix(0, b * ib, a.lda);
      p.T = ttile(i, k) + ix(0, b * ib, a.ldt);
      break;
    default:  // IT_TM
      p.mode = 1; p.L = nb; p.k = nb;
      p.C = tile(i, j);
      p.A1 = tile(k, j);
      p.c_cs = p.a_cs = tld(j);
      p.ncols = g.width(j);
      p.V = tile(i, k);
      p.T = ttile(i, k);
      break;
  }
  apply_strip<R, NW, TC>(p, s * NW, smem);
  return true;
}

template <typename R, int NW, bool TC>
__global__ void __launch_bounds__(TQR_THREADS, TC ? 1 : 2)
k_tile_dag(const __grid_constant__ DagArgs<R> a)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_it, s_err;
  const int tid = threadIdx.x;
  __shared__ unsigned long long s_tstart;
  __shared__ __align__(8) uint64_t s_bars[tc::kBars];
  __shared__ uint32_t s_tmem;
  bool first = true;
  if (tid == 0) s_err = (a.hdr->key != a.key || a.hdr->nitems != a.nitems) ? 2 : 0;
  __syncthreads();
  if (s_err) {
    if (tid == 0 && blockIdx.x == 0) atomicExch(&a.hdr->error, 2);
    return;
  }
  TcState tcs{0u, s_bars, {0u, 0u, 0u, 0u}};
  bool tc_failed = false;
  if constexpr (TC && std::is_same<R, float>::value) {
    if (a.g.tc) {
      // the tensor-core task's mbarriers and all TMEM columns (one CTA per SM)
      if (tid == 0) {
        for (int q = 0; q < tc::kBars; ++q)
          asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::saddr(&s_bars[q])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      }
      if ((tid >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::saddr(&s_tmem)),
                     "r"(tc::kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      tcs.tmem = s_tmem;
    }
  }
  for (;;) {
    if (tid == 0) s_it = atomicAdd(&a.hdr->head, 1);
    __syncthreads();
    const int idx = s_it;
    if (idx >= a.nitems) break;
    const DagItem it = a.items[idx];
    if (tid == 0) {
      int c[kMaxDeps], t[kMaxDeps];
      const int nd = item_deps(a.g, it, c, t);
      const unsigned long long t0 = global_ns();
      int err = 0;
      // test hook (tqr_tile_dag_wait_selftest): a wait that can only run out
      if (a.hold && idx == 0) {
        while (ld_acquire(reinterpret_cast<const int *>(&a.hdr->pad1[0])) == 0) {
          if (global_ns() - t0 > a.timeout_ns) {
            if (atomicCAS(&a.hdr->error, 0, 1) == 0) {
              a.hdr->err_item = idx;
              a.hdr->err_type = it.type;
            }
            err = 1;
            break;
          }
          __nanosleep(128);
        }
      }
      for (int d = 0; d < nd && !err; ++d) {
        while (ld_acquire(a.cnt + c[d]) < t[d]) {
          if (ld_acquire(&a.hdr->error) != 0) { err = 1; break; }
          if (global_ns() - t0 > a.timeout_ns) {
            if (atomicCAS(&a.hdr->error, 0, 1) == 0) {
              a.hdr->err_item = idx;
              a.hdr->err_type = it.type;
            }
            err = 1;
            break;
          }
          __nanosleep(128);
        }
      }
      s_err = err;
      const unsigned long long t1 = global_ns();
      s_tstart = t1;
      if (t1 > t0) atomicAdd(&a.hdr->wait_ns, t1 - t0);
      if (first) { atomicMin(&a.hdr->t_first, t0); first = false; }
    }
    __syncthreads();
    if (s_err) break;
    if (!run_item<R, NW, TC>(a, it, smem_raw, &tcs)) {
      // a tensor-core completion wait gave up: report, then stop this CTA
      if (tid == 0 && atomicCAS(&a.hdr->error, 0, 3) == 0) {
        a.hdr->err_item = idx;
        a.hdr->err_type = it.type;
      }
      tc_failed = true;
      break;
    }
    __syncthreads();
    if (tid == 0) {
      const unsigned long long t2 = global_ns();
      atomicAdd(&a.hdr->busy_ns[it.type < IT_TC ? it.type : IT_TM], t2 - s_tstart);
      atomicMax(&a.hdr->t_last, t2);
      __threadfence();
      int c[kMaxDeps];
      const int nu = item_updates(a.g, it, c);
      for (int u = 0; u < nu; ++u) atomicAdd(a.cnt + c[u], 1);
    }
  }
  if constexpr (TC && std::is_same<R, float>::value) {
    if (a.g.tc) {
      // after a failed wait: one more commit (it arrives once every earlier
      // MMA has completed) and one bounded wait for it
      if (tc_failed) {
        if (tid == 0) tc::commit(&s_bars[2]);
        tc::bar_wait(&s_bars[2], tcs.phase[2]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if ((tid >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tcs.tmem), "r"(tc::kTmemCols));
    }
  }
  (void)tc_failed;
}

// ---------------------------------------------------------------------------
// Host: schedule construction (cached per geometry)
// ---------------------------------------------------------------------------
struct Plan {
  DagGeom g;
  long long key;
  std::vector<DagItem> items;       // sorted
  // pinned host image of the upload: header at 0, items at 256 (page-locked so
  // the copies stay asynchronous); falls back to pageable memory
  unsigned char *pinned = nullptr;
  std::vector<unsigned char> pageable;
  size_t bytes_counters = 0, bytes_items = 0, bytes_d = 0, bytes_total = 0;
  const unsigned char *image() const { return pinned ? pinned : pageable.data(); }
  ~Plan() {
    if (pinned) cudaFreeHost(pinned);
  }
};

// Largest shared-memory need of any task, for elements of esize bytes (8: the
// real types, checked for the wider one; 16: ComplexF64).
static size_t dag_task_smem(int nb, int ib, int nw, int esize) {
  if (esize == 16)
    return std::max({apply_smem_elems(nb, ib, nw, true, true, true) * sizeof(cx<double>),
                     panel_smem<cx<double>>(nb, ib, true, true), tsqrt_smem<cx<double>>(nb, ib, true)});
  return std::max({apply_smem_elems(nb, ib, nw, true, true, true) * sizeof(double),
                   panel_smem<double>(nb, ib, true, true), tsqrt_smem<double>(nb, ib, true)});
}

// esize: bytes per element of the factorised matrix, rounded up to 8 (double,
// float and ComplexF32 share one geometry; ComplexF64 gets its own).
static bool dag_geom(int m, int n, int nb, int ib, DagGeom *g, int nrhs = 0, int esize = 8) {
  if (m <= 0 || n <= 0 || nb <= 0 || ib <= 0 || nrhs < 0 || nrhs > nb) return false;
  if (m % nb || n % nb || nb % ib) return false;
  if (nrhs > 0 && m < n) return false;         // the RHS tile column is never a panel
  if (nb > 256) return false;                  // one tile column of V per CTA in shared memory
  esize = esize > 8 ? 16 : 8;
  // 16-wide strips when two CTAs still fit per SM, else 8 (ib must be a multiple)
  int nw = 16;
  if (ib % 16 || 2 * (apply_smem_elems(nb, ib, 16, true, true, true) * esize + 1024) >
                     (size_t)TQR_SMEM_MAX + 1024)
    nw = 8;
  if (ib % nw) return false;
  g->m = m; g->n = n; g->nb = nb; g->ib = ib; g->nw = nw;
  g->nrhs = nrhs;
  g->tc = 0; g->NCH = nb / tc::kChunk; g->CPS = tc::kChunk / nw;
  g->f64p = 0;
  g->NTA = n / nb;
  g->MT = m / nb; g->NT = g->NTA + (nrhs > 0 ? 1 : 0); g->KT = std::min(g->MT, g->NTA);
  g->NS = nb / nw; g->SPB = ib / nw; g->NBK = nb / ib;
  if (2 * g->SPB + 1 > kMaxDeps) return false;
  if (g->MT > 65535 || g->NT > 65535 || g->NBK > 255) return false;
  // every task's shared memory must fit one CTA
  if (dag_task_smem(nb, ib, nw, esize) > (size_t)TQR_SMEM_MAX) return false;
  return true;
}

// The FP32 persistent kernel runs its tsmqr updates on the tensor cores
// unless a caller switches that off (tqr_tile_dag_tensor_cores(0)), e.g. to
// compare with the SIMT path.
static int g_tc_enabled = 1;
static bool tc_enabled() { return g_tc_enabled != 0; }
bool tile_tc_enabled() { return g_tc_enabled != 0; }

static long long geom_key(const DagGeom &g) {
  long long h = 1469598103934665603LL;
  for (int v : {g.m, g.n, g.nb, g.ib, g.nw, g.nrhs, g.tc, g.f64p}) h = (h ^ (long long)v) * 1099511628211LL;
  return h & 0x7fffffffffffffffLL;
}

// Natural (generation) order: the algorithm's own loop order, topological.
// Tasks of step k in the algorithm's loop order.
__host__ __device__ inline long long step_tasks(const DagGeom &g, int k) {
  const long long pt = g.panel_tasks();
  const long long rhs = g.NT > g.NTA ? g.strips(g.NTA) : 0;
  const long long right = (long long)(g.NTA - k - 1) * g.NS + rhs;
  const long long right_tm = (long long)(g.NTA - k - 1) * g.tm_tasks(0) + rhs;
  return pt + right + (long long)(g.MT - k - 1) * (pt + right_tm);
}

// Writes the tasks of step k into out[] in loop order; returns their count.
__host__ __device__ inline long long gen_step(const DagGeom &g, int k, DagItem *out) {
  long long n = 0;
  auto push = [&](uint8_t type, int i, int j, int b, int s) {
    DagItem it;
    it.type = type; it.b = (uint8_t)b; it.k = (uint16_t)k; it.i = (uint16_t)i; it.j = (uint16_t)j;
    it.s = (uint16_t)s; it.pad = 0;
    out[n++] = it;
  };
  for (int b = 0; b < g.NBK; ++b) {
    push(IT_GB, k, k, b, 0);
    for (int s = (b + 1) * g.SPB; s < g.NS; ++s) push(IT_GA, k, k, b, s);
  }
  for (int j = k + 1; j < g.NT; ++j)
    for (int s = 0; s < g.strips(j); ++s) push(IT_UN, k, j, 0, s);
  for (int i = k + 1; i < g.MT; ++i) {
    for (int b = 0; b < g.NBK; ++b) {
      push(IT_TB, i, k, b, 0);
      for (int s = (b + 1) * g.SPB; s < g.NS; ++s) push(IT_TA, i, k, b, s);
    }
    for (int j = k + 1; j < g.NT; ++j) {
      if (g.tc && j < g.NTA)
        for (int c = 0; c < g.NCH; ++c) push(IT_TC, i, j, 0, c);
      else
        for (int s = 0; s < g.strips(j); ++s) push(IT_TM, i, j, 0, s);
    }
  }
  return n;
}

// Task order for schedules written on the device (no host sort).  Tasks go
// in increasing key 4 min(column, k + 1) + row, ties in the loop order:
//   geqrt group of step k (GB, GA)        key 5k
//   every unmqr of step k (UN)            key 5k + 4
//   tsqrt group (k, i) (TB, TA)           key 4k + i
//   tsmqr row (k, i), all columns (TM)    key 4k + i + 4
// No producer has a larger key than its consumer: a tsqrt (k, i) needs the
// tsmqr (k - 1, i) on its tile, key 4(k - 1) + i + 4 = 4k + i; the geqrt of
// step k needs the tsmqr (k - 1, k), key 5k; a tsmqr needs its tsqrt, the
// tsmqr or unmqr above it in its column and the previous step's update of
// its tile, all with smaller keys.  With ties in the loop order, which is
// topological, the list is topological (tqr_tile_noalloc_check replays it).
// Capping the column at k + 1 keeps far columns' updates from being queued
// ahead of the next panels, and the row weight 1/4 lets the next step's
// panel chain start while the current step's lower rows are still queued:
// the list follows the critical path much as the host's longest-path sort
// does.  Bucket v holds the tasks of key v, step by step in loop order (for
// one step: geqrt, unmqr, the tsmqr row v - 4k - 4, then the tsqrt row
// v - 4k, which is their order in the loop).  Writes the tasks when out is
// non-null; returns their count.
__host__ __device__ inline int noalloc_buckets(const DagGeom &g) { return 5 * g.KT + g.MT + 4; }

// strips of the tile columns right of column k (one unmqr or tsmqr row)
__host__ __device__ inline long long right_strips(const DagGeom &g, int k) {
  long long n = 0;
  for (int j = k + 1; j < g.NT; ++j) n += g.strips(j);
  return n;
}

__host__ __device__ inline long long gen_bucket(const DagGeom &g, int v, DagItem *out) {
  long long n = 0;
  int k = 0;
  auto push = [&](uint8_t type, int i, int j, int b, int s) {
    DagItem it;
    it.type = type; it.b = (uint8_t)b; it.k = (uint16_t)k; it.i = (uint16_t)i; it.j = (uint16_t)j;
    it.s = (uint16_t)s; it.pad = 0;
    out[n++] = it;
  };
  for (k = 0; k < g.KT && 5 * k <= v; ++k) {     // every key of step k is >= 5k
    const int i2 = v - 4 * k - 4, i1 = v - 4 * k;
    const bool pg = v == 5 * k, un = v == 5 * k + 4;
    const bool tm = i2 > k && i2 < g.MT, ts = i1 > k && i1 < g.MT;
    if (!out) {
      n += (pg ? g.panel_tasks() : 0) + (ts ? g.panel_tasks() : 0) + (un ? right_strips(g, k) : 0) +
           (tm ? right_strips(g, k) : 0);
      continue;
    }
    if (pg)
      for (int b = 0; b < g.NBK; ++b) {
        push(IT_GB, k, k, b, 0);
        for (int s = (b + 1) * g.SPB; s < g.NS; ++s) push(IT_GA, k, k, b, s);
      }
    if (un)
      for (int j = k + 1; j < g.NT; ++j)
        for (int s = 0; s < g.strips(j); ++s) push(IT_UN, k, j, 0, s);
    if (tm)
      for (int j = k + 1; j < g.NT; ++j)
        for (int s = 0; s < g.strips(j); ++s) push(IT_TM, i2, j, 0, s);
    if (ts)
      for (int b = 0; b < g.NBK; ++b) {
        push(IT_TB, i1, k, b, 0);
        for (int s = (b + 1) * g.SPB; s < g.NS; ++s) push(IT_TA, i1, k, b, s);
      }
  }
  return n;
}

// Natural (generation) order: the algorithm's own loop order, topological.
static void gen_items(const DagGeom &g, std::vector<DagItem> &v) {
  long long total = 0;
  for (int k = 0; k < g.KT; ++k) total += step_tasks(g, k);
  v.resize((size_t)total);
  long long off = 0;
  for (int k = 0; k < g.KT; ++k) off += gen_step(g, k, v.data() + off);
}

static double item_cost(const DagGeom &g, const DagItem &it) {
  // relative durations (FP64 FMAs per task, panel tasks weighted for their
  // serial column steps)
  const double nb = g.nb, ib = g.ib, nw = g.nw;
  switch (it.type) {
    case IT_GB: return 3.0 * (nb - it.b * ib) * ib * ib + 64.0 * ib * 600;
    case IT_TB: return 3.0 * nb * ib * ib + 64.0 * ib * 600;
    case IT_GA: return 4.0 * (nb - it.b * ib) * ib * nw;
    case IT_TA: return 4.0 * nb * ib * nw;
    case IT_UN: return 2.0 * nb * nb * std::min<double>(nw, g.width(it.j));
    case IT_TC: return 4.0 * nb * nb * tc::kChunk / 6.0;     // tensor cores: ~6x a SIMT strip per column
    default: return 4.0 * nb * nb * std::min<double>(nw, g.width(it.j));
  }
}

// Bucket width of the priority sort in full-tile strip updates (0: exact
// longest-path order; tqr_tile_dag_order_quantum).
static double g_order_q = 0.0;

// Replays the natural order: for every counter the list of its writers.
// Returns false if a wait target is not what the replay gives (tested on the
// host by tqr_tile_dag_check).
static bool build_schedule(const DagGeom &g, std::vector<DagItem> &sorted, bool verify) {
  std::vector<DagItem> nat;
  gen_items(g, nat);
  const int N = (int)nat.size();
  std::vector<std::vector<int>> writers(g.ncounters());
  std::vector<std::vector<int>> preds(N);
  int c[kMaxDeps], t[kMaxDeps];
  bool ok = true;
  for (int x = 0; x < N; ++x) {
    const int nd = item_deps(g, nat[x], c, t);
    for (int d = 0; d < nd; ++d) {
      const auto &w = writers[c[d]];
      // every target is exactly the number of writers generated before the
      // task (for done counters: the whole group, which always precedes it)
      if (verify && t[d] != (int)w.size()) ok = false;
      if (t[d] > 0) {
        if (t[d] <= (int)w.size()) preds[x].push_back(w[t[d] - 1]);
        else ok = false;    // target never reached before this task
      }
    }
    const int nu = item_updates(g, nat[x], c);
    for (int u = 0; u < nu; ++u) writers[c[u]].push_back(x);
  }
  // done counters must end exactly at panel_tasks()
  for (int k = 0; k < g.KT; ++k) {
    if ((int)writers[g.done_g(k)].size() != g.panel_tasks()) ok = false;
    for (int i = k + 1; i < g.MT; ++i)
      if ((int)writers[g.done_t(k, i)].size() != g.panel_tasks()) ok = false;
  }
  // longest path to the end, natural order reversed
  std::vector<double> rank(N, 0.0);
  for (int x = N - 1; x >= 0; --x) {
    rank[x] += item_cost(g, nat[x]);
    for (int p : preds[x]) rank[p] = std::max(rank[p], rank[x]);
  }
  std::vector<int> order(N);
  for (int x = 0; x < N; ++x) order[x] = x;
  if (g_order_q > 0.0) {
    // ranks in buckets of q full-tile strip updates, loop order inside a
    // bucket: consecutive tasks then share their reflector tile while it is
    // in L2 (a predecessor's bucket is never lower, and loop order is
    // topological, so the order stays topological)
    const double unit = g_order_q * 4.0 * g.nb * g.nb * g.nw;
    std::vector<long long> bucket(N);
    for (int x = 0; x < N; ++x) bucket[x] = (long long)std::floor(rank[x] / unit);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return bucket[a] > bucket[b]; });
  } else {
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rank[a] > rank[b]; });
  }
  if (verify) {
    std::vector<int> pos(N);
    for (int x = 0; x < N; ++x) pos[order[x]] = x;
    for (int x = 0; x < N; ++x)
      for (int p : preds[x])
        if (pos[p] >= pos[x]) ok = false;   // sorted order must stay topological
  }
  sorted.resize(N);
  for (int x = 0; x < N; ++x) sorted[x] = nat[order[x]];
  return ok;
}

static std::mutex g_plan_mu;
static std::map<long long, std::shared_ptr<Plan>> g_plans;

static std::shared_ptr<Plan> get_plan(const DagGeom &g) {
  long long qbits = 0;
  std::memcpy(&qbits, &g_order_q, sizeof(qbits));
  const long long key = (geom_key(g) ^ (qbits * 1099511628211LL)) & 0x7fffffffffffffffLL;
  std::lock_guard<std::mutex> l(g_plan_mu);
  auto f = g_plans.find(key);
  if (f != g_plans.end()) return f->second;
  auto p = std::make_shared<Plan>();
  p->g = g;
  p->key = key;
  build_schedule(g, p->items, false);
  p->bytes_counters = align256(sizeof(int) * (size_t)g.ncounters());
  p->bytes_items = align256(sizeof(DagItem) * p->items.size());
  p->bytes_d = g.f64p ? align256(sizeof(double) * (size_t)g.ib * g.KT * g.nb) : 0;
  p->bytes_total = 256 + p->bytes_counters + p->bytes_items + p->bytes_d;
  const size_t img = 256 + sizeof(DagItem) * p->items.size();
  unsigned char *dst = nullptr;
  if (cudaMallocHost((void **)&p->pinned, img) == cudaSuccess) {
    dst = p->pinned;
  } else {
    p->pinned = nullptr;
    cudaGetLastError();
    p->pageable.resize(img);
    dst = p->pageable.data();
  }
  DagHeader h;
  std::memset(&h, 0, sizeof(h));
  h.key = key;
  h.nitems = (int)p->items.size();
  h.t_first = ~0ull;
  std::memset(dst, 0, 256);
  std::memcpy(dst, &h, sizeof(h));
  std::memcpy(dst + 256, p->items.data(), sizeof(DagItem) * p->items.size());
  g_plans[key] = p;
  return p;
}

template <typename R, int NW, bool TC = false>
static int launch_dag(const DagArgs<R> &a, size_t sm, double flops, cudaStream_t st, bool timed = true) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_tile_dag<R, NW, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) !=
      cudaSuccess)
    return (int)e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return (int)e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_dag<R, NW, TC>, TQR_THREADS, sm)) !=
      cudaSuccess)
    return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const int grid = std::min(sms * per_sm, a.nitems);
  void *tok = timed ? prof_begin(st) : nullptr;
  k_tile_dag<R, NW, TC><<<grid, TQR_THREADS, sm, st>>>(a);
  if (timed) prof_end(tok, st, flops);
  count_launch();
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

template <typename R>
static int tile_geqrf_dag(int m, int n, int nb, int ib, R *A, int lda, R *T, int ldt, R *tau,
                          int ldtau, void *work, size_t lwork, cudaStream_t st, int nrhs = 0,
                          R *B = nullptr, int ldb = 1, unsigned long long hold_ns = 0, bool f64p = false) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (nb <= 0) return -3;
  if (ib <= 0 || ib > nb) return -4;
  if (m == 0 || n == 0) return 0;
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g, nrhs, (int)sizeof(R))) return -3;   // shape outside the DAG path
  // FP32: trailing tsmqr updates on the tensor cores when the tile shape and
  // the float4 staging alignment allow it
  if (std::is_same<R, float>::value && nb == 256 && ib == tc::kIb && g.nw == 16 && tc_enabled() &&
      ((uintptr_t)A & 15) == 0 && (lda & 3) == 0)
    g.tc = 1;
  if (f64p) {
    if (!std::is_same<R, float>::value) return -3;
    g.f64p = 1;
  }
  if (lda < m) return -6;
  if (ldt < g.MT * ib) return -8;
  if (ldtau < n) return -10;
  if (!work || ((uintptr_t)work & 255)) return -11;
  if (nrhs > 0 && (!B || ldb < m)) return -13;
  auto plan = get_plan(g);
  if (lwork < plan->bytes_total) return -12;
  unsigned char *w = (unsigned char *)work;
  cudaError_t e;
  // header (key, zero head and error) + zeroed counters + the schedule, all
  // ordered on `st` ahead of the kernel
  const unsigned char *img = plan->image();
  if ((e = cudaMemcpyAsync(w, img, sizeof(DagHeader), cudaMemcpyHostToDevice, st)) != cudaSuccess) return (int)e;
  if ((e = cudaMemsetAsync(w + 256, 0, plan->bytes_counters, st)) != cudaSuccess) return (int)e;
  if ((e = cudaMemcpyAsync(w + 256 + plan->bytes_counters, img + 256, sizeof(DagItem) * plan->items.size(),
                           cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return (int)e;
  DagArgs<R> a;
  a.g = g;
  a.A = A; a.lda = lda;
  a.B = B; a.ldb = ldb;
  a.T = T; a.ldt = ldt;
  a.tau = tau; a.ldtau = ldtau;
  a.hdr = (DagHeader *)w;
  a.cnt = (int *)(w + 256);
  a.items = (const DagItem *)(w + 256 + plan->bytes_counters);
  a.nitems = (int)plan->items.size();
  a.key = plan->key;
  if (g.f64p) a.D = (double *)(w + 256 + plan->bytes_counters + plan->bytes_items);
  if constexpr (std::is_same<R, float>::value) {
    if (g.tc && tc_tma_enabled())
      a.tma = make_tmap_f32(&a.tmw, A, m, (long long)g.NTA * nb, lda, 32, tc::kChunk) == cudaSuccess &&
              make_tmap_f32(&a.tmn, A, m, (long long)g.NTA * nb, lda, 32, tc::kIb) == cudaSuccess;
  }
  a.timeout_ns = 20ull * 1000ull * 1000ull * 1000ull;   // 20 s for any single wait
  if (hold_ns) {
    a.timeout_ns = hold_ns;
    a.hold = 1;
  }
  size_t sm = std::max({apply_smem_elems(nb, ib, g.nw, true, true, true) * sizeof(R),
                        panel_smem<R>(nb, ib, true, true), tsqrt_smem<R>(nb, ib, true)});
  if (g.tc) sm = std::max(sm, tc::kSmem);
  if (g.f64p) sm = std::max({sm, panel_f64_smem(nb, ib), tsqrt_f64_smem(nb, ib), tsqrt_f64x_smem(nb, ib)});
  const double mn = (double)std::max(m, n), kn = (double)std::min(m, n);
  const double flops = 2.0 * mn * kn * kn - 2.0 * kn * kn * kn / 3.0;
  if constexpr (std::is_same<R, float>::value) {
    if (g.tc) return launch_dag<R, 16, true>(a, sm, flops, st);
  }
  return g.nw == 16 ? launch_dag<R, 16>(a, sm, flops, st) : launch_dag<R, 8>(a, sm, flops, st);
}

// ---------------------------------------------------------------------------
// Allocation-free variant.  Some callers cannot hand the library device
// memory for the schedule: code that runs while a framework's caching
// allocator owns the whole device (no room for a second allocator), host code
// that must not take the implicit device synchronisation of cudaMalloc /
// cudaFree in the middle of a pipeline, and bindings that have no way to keep
// a scratch buffer alive between calls.  For them the schedule and its
// counters live in one file-scope device array of fixed size that every GPU
// loading this library keeps until exit.  The task list is written on the
// device (the bucket order of gen_bucket, which is topological), so
// neither the host nor the device allocates anything per call.
// ---------------------------------------------------------------------------
constexpr size_t kStaticScratchBytes = size_t(4) << 20;   // 4 MiB (see tileqr.h)
static __device__ __align__(256) unsigned char g_tile_scratch[kStaticScratchBytes];

static std::mutex g_static_mu;
static void *g_static_ptr[64];

// Device address of g_tile_scratch on the current device (set-up on the
// first call per device; in host code the symbol itself is only a stand-in).
// The address is cached for the life of the device's primary context: after
// a cudaDeviceReset the cached address is stale, so the entry points that use
// it must not be called after a reset in the same process.
static cudaError_t static_scratch(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> l(g_static_mu);
  if (!g_static_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_tile_scratch);
    if (e != cudaSuccess) return e;
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return cudaSuccess;
}

// Clears the header and counters and writes the task list (CTA v writes
// bucket v of gen_bucket's order at its offset).  Everything the DAG kernel expects to start at zero is
// cleared here on every call, because the array keeps the previous call's
// contents.
__global__ void k_static_schedule(DagGeom g, unsigned char *w, size_t bytes_counters, long long key,
                                  int nitems) {
  int *cnt = reinterpret_cast<int *>(w + 256);
  const int ncnt = g.ncounters();
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < ncnt; x += gridDim.x * blockDim.x) cnt[x] = 0;
  if (blockIdx.x == 0) {
    int *hw = reinterpret_cast<int *>(w);
    for (int x = threadIdx.x; x < (int)(sizeof(DagHeader) / sizeof(int)); x += blockDim.x) hw[x] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
      DagHeader *h = reinterpret_cast<DagHeader *>(w);
      h->key = key;
      h->nitems = nitems;
      h->t_first = ~0ull;
    }
  }
  if (threadIdx.x == 0 && (int)blockIdx.x < noalloc_buckets(g)) {
    long long off = 0;
    for (int q = 0; q < (int)blockIdx.x; ++q) off += gen_bucket(g, q, nullptr);
    gen_bucket(g, blockIdx.x, reinterpret_cast<DagItem *>(w + 256 + bytes_counters) + off);
  }
}

static int tile_geqrf_noalloc(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt,
                              double *tau, int ldtau, cudaStream_t st) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (nb <= 0) return -3;
  if (ib <= 0 || ib > nb) return -4;
  if (m == 0 || n == 0) return 0;
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g)) return -3;
  if (lda < m) return -6;
  if (ldt < g.MT * ib) return -8;
  if (ldtau < n) return -10;
  long long nitems = 0;
  for (int k = 0; k < g.KT; ++k) nitems += step_tasks(g, k);
  const size_t bytes_counters = align256(sizeof(int) * (size_t)g.ncounters());
  const size_t need = 256 + bytes_counters + sizeof(DagItem) * (size_t)nitems;
  if (need > kStaticScratchBytes || nitems > 0x7fffffff) return TQR_ERR_SCRATCH_TOO_SMALL;
  void *wv = nullptr;
  cudaError_t e = static_scratch(&wv);
  if (e != cudaSuccess) return (int)e;
  unsigned char *w = static_cast<unsigned char *>(wv);
  const long long key = geom_key(g);
  k_static_schedule<<<noalloc_buckets(g), TQR_THREADS, 0, st>>>(g, w, bytes_counters, key, (int)nitems);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
  DagArgs<double> a;
  a.g = g;
  a.A = A; a.lda = lda;
  a.B = nullptr; a.ldb = 1;
  a.T = T; a.ldt = ldt;
  a.tau = tau; a.ldtau = ldtau;
  a.hdr = reinterpret_cast<DagHeader *>(w);
  a.cnt = reinterpret_cast<int *>(w + 256);
  a.items = reinterpret_cast<const DagItem *>(w + 256 + bytes_counters);
  a.nitems = (int)nitems;
  a.key = key;
  a.timeout_ns = 20ull * 1000ull * 1000ull * 1000ull;
  const size_t sm = std::max({apply_smem_elems(nb, ib, g.nw, true, true, true) * sizeof(double),
                              panel_smem<double>(nb, ib, true, true), tsqrt_smem<double>(nb, ib, true)});
  return g.nw == 16 ? launch_dag<double, 16>(a, sm, 0.0, st, false)
                    : launch_dag<double, 8>(a, sm, 0.0, st, false);
}

// Workspace of the FP64-panel form of geometry g: the same schedule plus the
// FP64 diagonal triangles (the task list and counters do not depend on it).
static size_t f64p_bytes(const DagGeom &g) {
  return get_plan(g)->bytes_total + align256(sizeof(double) * (size_t)g.ib * g.KT * g.nb);
}

// tqr_dsgels factors with FP64 panels unless a caller switches that off
// (tqr_dsgels_fp64_panels(0)), e.g. to compare with the all-FP32 panels.
static int g_f64p_enabled = 1;
bool dsgels_f64p_enabled() { return g_f64p_enabled != 0; }

int stile_gels_dag_mixed(int m, int n, int nrhs, int nb, int ib, float *A, int lda, float *T, int ldt,
                         float *tau, int ldtau, float *B, int ldb, void *work, size_t lwork, cudaStream_t stream) {
  if (nrhs < 0 || nrhs > nb) return -3;
  int rc = tile_geqrf_dag<float>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, work, lwork, stream, nrhs, B, ldb, 0,
                                 g_f64p_enabled != 0);
  if (rc != 0) return rc;
  return nrhs > 0 ? tqr_strsm_lun(n, nrhs, A, lda, B, ldb, stream) : 0;
}

}  // namespace tqr

using namespace tqr;

extern "C" {

int tqr_dsgels_fp64_panels(int on) {
  const int old = g_f64p_enabled;
  g_f64p_enabled = on ? 1 : 0;
  return old;
}

int tqr_stile_geqrf_dag_f64p(int m, int n, int nb, int ib, float *A, int lda, float *T, int ldt, float *tau,
                             int ldtau, void *work, size_t lwork, cudaStream_t stream) {
  return tile_geqrf_dag<float>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, work, lwork, stream, 0, nullptr, 1, 0,
                               true);
}

int tqr_tile_dag_worksize(int m, int n, int nb, int ib, size_t *bytes) {
  if (!bytes) return -5;
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g)) {
    *bytes = 0;
    return 1;    // not eligible: use tqr_?tile_geqrf (stream driver, no workspace)
  }
  // one size for every element type: ComplexF64 may schedule narrower strips
  // (more tasks) than the real types
  size_t b = get_plan(g)->bytes_total;
  DagGeom gz;
  if (dag_geom(m, n, nb, ib, &gz, 0, 16)) b = std::max(b, get_plan(gz)->bytes_total);
  b = std::max(b, f64p_bytes(g));
  *bytes = b;
  return 0;
}

int tqr_tile_gels_worksize(int m, int n, int nrhs, int nb, int ib, size_t *bytes) {
  if (!bytes) return -6;
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g, nrhs)) {
    *bytes = 0;
    return 1;
  }
  *bytes = std::max(get_plan(g)->bytes_total, f64p_bytes(g));
  return 0;
}

// Least squares in one persistent launch plus a triangular solve: B rides
// along as an extra tile column of the factorisation (so it leaves as Q^T B),
// then R X = (Q^T B)[0:n].  X overwrites B[0:n, 0:nrhs].
int tqr_dtile_gels_dag(int m, int n, int nrhs, int nb, int ib, double *A, int lda, double *T, int ldt,
                       double *tau, int ldtau, double *B, int ldb, void *work, size_t lwork,
                       cudaStream_t stream) {
  if (nrhs < 0 || nrhs > nb) return -3;
  int rc = tile_geqrf_dag<double>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, work, lwork, stream, nrhs, B, ldb);
  if (rc != 0) return rc;
  return nrhs > 0 ? tqr_dtrsm_lun(n, nrhs, A, lda, B, ldb, stream) : 0;
}

int tqr_stile_gels_dag(int m, int n, int nrhs, int nb, int ib, float *A, int lda, float *T, int ldt,
                       float *tau, int ldtau, float *B, int ldb, void *work, size_t lwork,
                       cudaStream_t stream) {
  if (nrhs < 0 || nrhs > nb) return -3;
  int rc = tile_geqrf_dag<float>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, work, lwork, stream, nrhs, B, ldb);
  if (rc != 0) return rc;
  return nrhs > 0 ? tqr_strsm_lun(n, nrhs, A, lda, B, ldb, stream) : 0;
}

int tqr_dtile_geqrf_dag(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt,
                        double *tau, int ldtau, void *work, size_t lwork, cudaStream_t stream) {
  return tile_geqrf_dag<double>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, work, lwork, stream);
}

int tqr_stile_geqrf_dag(int m, int n, int nb, int ib, float *A, int lda, float *T, int ldt,
                        float *tau, int ldtau, void *work, size_t lwork, cudaStream_t stream) {
  return tile_geqrf_dag<float>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, work, lwork, stream);
}

int tqr_ztile_geqrf_dag(int m, int n, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T, int ldt,
                        tqr_zcomplex *tau, int ldtau, void *work, size_t lwork, cudaStream_t stream) {
  using E = cx<double>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)tau) % alignof(E)) return -5;
  return tile_geqrf_dag<E>(m, n, nb, ib, (E *)A, lda, (E *)T, ldt, (E *)tau, ldtau, work, lwork, stream);
}

int tqr_ctile_geqrf_dag(int m, int n, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T, int ldt,
                        tqr_ccomplex *tau, int ldtau, void *work, size_t lwork, cudaStream_t stream) {
  using E = cx<float>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)tau) % alignof(E)) return -5;
  return tile_geqrf_dag<E>(m, n, nb, ib, (E *)A, lda, (E *)T, ldt, (E *)tau, ldtau, work, lwork, stream);
}

int tqr_tile_dag_wait_selftest(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt, double *tau,
                               int ldtau, void *work, size_t lwork, int wait_ms, cudaStream_t stream) {
  if (wait_ms <= 0 || wait_ms > 5000) return -13;
  return tile_geqrf_dag<double>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, work, lwork, stream, 0, nullptr, 1,
                                (unsigned long long)wait_ms * 1000000ull);
}

int tqr_tile_dag_status(const void *work, int *status, int *task, cudaStream_t stream) {
  if (!work) return -1;
  DagHeader h;
  cudaError_t e = cudaMemcpyAsync(&h, work, sizeof(h), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return (int)e;
  if (status) *status = h.error;
  if (task) *task = h.err_item;
  return 0;
}

int tqr_dtile_geqrf_noalloc(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt,
                            double *tau, int ldtau, cudaStream_t stream) {
  return tile_geqrf_noalloc(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, stream);
}

// Error word of the last tqr_dtile_geqrf_noalloc launch on this device: the
// header sits at the start of the static array, which no caller can address,
// so this reads it for them (a copy from the symbol, then a stream
// synchronisation; nothing is allocated).
// One 64-bit identity per task: type (3 bits), block b (8), strip or chunk s
// (5: at most nb / nw = 32 strips), step k, row i and column j (16 each).
static unsigned long long item_id(const DagItem &it) {
  return ((unsigned long long)it.type << 61) | ((unsigned long long)it.b << 53) | ((unsigned long long)it.s << 48) |
         ((unsigned long long)it.k << 32) | ((unsigned long long)it.i << 16) | (unsigned long long)it.j;
}

int tqr_tile_noalloc_check(int m, int n, int nb, int ib, long long *ntasks) {
  const auto id = item_id;
  // Host replay of the allocation-free schedule's order: every wait target of
  // every task is reached by the writers listed before it, and the list holds
  // each task of the loop order exactly once.
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g)) return -1;
  std::vector<DagItem> v;
  for (int q = 0; q < noalloc_buckets(g); ++q) {
    const size_t off = v.size();
    const long long c = gen_bucket(g, q, nullptr);
    v.resize(off + (size_t)c);
    if (gen_bucket(g, q, v.data() + off) != c) return 4;     // counting and writing agree
  }
  std::vector<DagItem> nat;
  gen_items(g, nat);
  if (v.size() != nat.size()) return 1;
  // the same tasks as the loop order, each once
  {
    std::vector<unsigned long long> a(v.size()), b(nat.size());
    for (size_t x = 0; x < v.size(); ++x) { a[x] = id(v[x]); b[x] = id(nat[x]); }
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b) return 5;
  }
  std::vector<int> seen(g.ncounters(), 0);
  int c[kMaxDeps], t[kMaxDeps];
  for (const DagItem &it : v) {
    const int nd = item_deps(g, it, c, t);
    for (int d = 0; d < nd; ++d)
      if (seen[c[d]] < t[d]) return 2;
    const int nu = item_updates(g, it, c);
    for (int u = 0; u < nu; ++u) ++seen[c[u]];
  }
  for (int k = 0; k < g.KT; ++k) {
    if (seen[g.done_g(k)] != g.panel_tasks()) return 3;
    for (int i = k + 1; i < g.MT; ++i)
      if (seen[g.done_t(k, i)] != g.panel_tasks()) return 3;
  }
  if (ntasks) *ntasks = (long long)v.size();
  return 0;
}

// Host simulation of the persistent kernel running a task list: `workers`
// CTAs take tasks strictly in list order, each waits for the task's producers
// (the writers that bring its wait counters to their targets), then runs it
// for item_cost units.  Returns the makespan in those units.
static double simulate_order(const DagGeom &g, const std::vector<DagItem> &list, int workers) {
  const auto id = item_id;
  std::vector<DagItem> nat;
  gen_items(g, nat);
  const int N = (int)nat.size();
  std::map<unsigned long long, int> index;
  for (int x = 0; x < N; ++x) index[id(nat[x])] = x;
  // producers of every task, by replaying the loop order's counter writes
  std::vector<std::vector<int>> writers(g.ncounters()), preds(N);
  int c[kMaxDeps], t[kMaxDeps];
  for (int x = 0; x < N; ++x) {
    const int nd = item_deps(g, nat[x], c, t);
    for (int d = 0; d < nd; ++d)
      if (t[d] > 0) preds[x].push_back(writers[c[d]][t[d] - 1]);
    const int nu = item_updates(g, nat[x], c);
    for (int u = 0; u < nu; ++u) writers[c[u]].push_back(x);
  }
  std::vector<double> fin(N, -1.0);
  std::vector<double> free_at(workers, 0.0);     // a heap of the workers' free times
  double span = 0.0;
  for (const DagItem &it : list) {
    const int x = index.at(id(it));
    std::pop_heap(free_at.begin(), free_at.end(), std::greater<double>());
    double start = free_at.back();
    for (int p : preds[x]) {
      if (fin[p] < 0.0) return -1.0;             // a producer after its consumer
      start = std::max(start, fin[p]);
    }
    fin[x] = start + item_cost(g, nat[x]);
    span = std::max(span, fin[x]);
    free_at.back() = fin[x];
    std::push_heap(free_at.begin(), free_at.end(), std::greater<double>());
  }
  return span;
}

int tqr_tile_dag_simulate(int m, int n, int nb, int ib, int workers, double *noalloc_span, double *sorted_span,
                          double *ideal_span) {
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g)) return -1;
  if (workers < 1) return -5;
  std::vector<DagItem> sorted, buck;
  build_schedule(g, sorted, false);
  for (int q = 0; q < noalloc_buckets(g); ++q) {
    const size_t off = buck.size();
    buck.resize(off + (size_t)gen_bucket(g, q, nullptr));
    gen_bucket(g, q, buck.data() + off);
  }
  double total = 0.0;
  for (const DagItem &it : sorted) total += item_cost(g, it);
  const double a = simulate_order(g, buck, workers), b = simulate_order(g, sorted, workers);
  if (a < 0.0 || b < 0.0) return 2;
  if (noalloc_span) *noalloc_span = a;
  if (sorted_span) *sorted_span = b;
  if (ideal_span) *ideal_span = total / workers;
  return 0;
}

int tqr_tile_noalloc_status(int *status, int *task, cudaStream_t stream) {
  void *wv = nullptr;
  cudaError_t e = static_scratch(&wv);
  if (e != cudaSuccess) return (int)e;
  DagHeader h;
  e = cudaMemcpyFromSymbolAsync(&h, g_tile_scratch, sizeof(h), 0, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return (int)e;
  if (status) *status = h.error;
  if (task) *task = h.err_item;
  return 0;
}

int tqr_tile_dag_stats(const void *work, unsigned long long *out, cudaStream_t stream) {
  if (!work || !out) return -1;
  DagHeader h;
  cudaError_t e = cudaMemcpyAsync(&h, work, sizeof(h), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return (int)e;
  for (int q = 0; q < 6; ++q) out[q] = h.busy_ns[q];
  out[6] = h.wait_ns;
  out[7] = h.t_first;
  out[8] = h.t_last;
  return 0;
}

int tqr_tile_dag_check_rhs(int m, int n, int nrhs, int nb, int ib, long long *ntasks) {
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g, nrhs)) return 1;
  std::vector<DagItem> items;
  const bool ok = build_schedule(g, items, true);
  if (ntasks) *ntasks = (long long)items.size();
  return ok ? 0 : 2;
}

int tqr_tile_dag_occupancy(int dtype_bytes, int tensor_cores, int *ctas_per_sm, int *smem_bytes) {
  if ((dtype_bytes != 4 && dtype_bytes != 8) || !ctas_per_sm || !smem_bytes) return -1;
  const int nb = 256, ib = 32;
  size_t sm = 0;
  cudaError_t e;
  int per = 0;
  if (dtype_bytes == 8) {
    sm = std::max({apply_smem_elems(nb, ib, 16, true, true, true) * sizeof(double), panel_smem<double>(nb, ib, true, true),
                   tsqrt_smem<double>(nb, ib, true)});
    if ((e = cudaFuncSetAttribute(k_tile_dag<double, 16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sm)) != cudaSuccess)
      return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tile_dag<double, 16, false>, TQR_THREADS, sm);
  } else {
    sm = std::max({apply_smem_elems(nb, ib, 16, true, true, true) * sizeof(float), panel_smem<float>(nb, ib, true, true),
                   tsqrt_smem<float>(nb, ib, true)});
    if (tensor_cores) {
      sm = std::max(sm, tc::kSmem);
      if ((e = cudaFuncSetAttribute(k_tile_dag<float, 16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sm)) != cudaSuccess)
        return (int)e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tile_dag<float, 16, true>, TQR_THREADS, sm);
    } else {
      if ((e = cudaFuncSetAttribute(k_tile_dag<float, 16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sm)) != cudaSuccess)
        return (int)e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tile_dag<float, 16, false>, TQR_THREADS, sm);
    }
  }
  if (e != cudaSuccess) return (int)e;
  *ctas_per_sm = per;
  *smem_bytes = (int)sm;
  return 0;
}

double tqr_tile_dag_order_quantum(double q) {
  std::lock_guard<std::mutex> l(g_plan_mu);
  const double old = g_order_q;
  g_order_q = q > 0.0 ? q : 0.0;
  return old;
}

int tqr_tile_dag_tensor_cores(int on) {
  const int old = g_tc_enabled;
  g_tc_enabled = on ? 1 : 0;
  return old;
}

int tqr_tile_dag_check_tc(int m, int n, int nrhs, int nb, int ib, long long *ntasks) {
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g, nrhs)) return 1;
  if (nb != 256 || ib != tc::kIb || g.nw != 16) return 1;
  g.tc = 1;
  std::vector<DagItem> items;
  if (!build_schedule(g, items, true)) return 2;
  long long total = 0;
  for (int k = 0; k < g.KT; ++k) total += step_tasks(g, k);
  if (total != (long long)items.size()) return 3;
  if (ntasks) *ntasks = (long long)items.size();
  return 0;
}

int tqr_tile_dag_check(int m, int n, int nb, int ib, long long *ntasks) {
  DagGeom g;
  if (!dag_geom(m, n, nb, ib, &g)) return 1;
  std::vector<DagItem> items;
  const bool ok = build_schedule(g, items, true);
  if (ntasks) *ntasks = (long long)items.size();
  return ok ? 0 : 2;
}

}  // extern "C"
