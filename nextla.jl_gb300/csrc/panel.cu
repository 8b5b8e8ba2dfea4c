// panel.cu -- Householder panel kernels (one CTA per panel).
//
//  k_panel_qr     geqr2 with the larft T build fused in (NextLA src/geqr2.jl:23-105
//                 and src/larft.jl:53-86,112-124 for direct 'F', storev 'C').
//  k_tsqrt_block  one ib-block of tsqrt: reflectors of [A1 (upper); A2] and the
//                 T block (NextLA src/tsqrt.jl:46-126).
//  k_larft        stand-alone larft for every direct/storev combination
//                 (NextLA src/larft.jl:48-203).
//
// The reference runs each of these as a single work-item.  Here the CTA works
// on every column together.  Both factorisations share one column step:
//
//   geqr2 at column i:  alpha = P[i,i], x = P[i+1:m, i], "row" = P[i, :]
//   tsqrt at column i:  alpha = A1[i,i], x = A2[0:m, i], "row" = A1[i, :]
//
//   xnorm^2 = sum x^2; beta, tau, scale (one thread, broadcast); x *= scale;
//   d_j = -tau (row[j] + x^T P[x rows, j]) for every other column j (j > i:
//   the w of the rank-1 apply; j < i: the V^H v of the T column -- geqr2 keeps
//   the row term there because row i of column j < i is part of v_j, tsqrt
//   drops it because the A1 part of v_j is e_j);  row[j] += d_j and
//   P[x rows, j] += x d_j for j > i;  T[0:i, i] = T[0:i, 0:i] d[0:i].
//
// FP64 runs at ~7.9 GFLOP/s per SM on GB300, so the step is organised around
// FP64 instruction count: the dot products use one thread per (column, row
// group) with the row groups combined by a single add per group (no shuffle
// trees), the Householder scalars (sqrt and two divisions) are computed once,
// and the panel and T live in shared memory.
#include "common.cuh"
#include "tileqr_internal.h"

namespace tqr {

template <typename R>
struct ColumnStep {
  R *P;       // x region rows live here (geqr2: the panel; tsqrt: A2)
  int ldp;
  R *row;     // row i of the factored matrix: row[j * rs]
  int rs;
  R *Ts;      // T (nc-by-nc upper), ld = ldts, or nullptr
  int ldts;
  R *part;    // TQR_THREADS partial sums
  R *d;       // nc: -tau * (row[j] + x^T P[:, j])
  R *scal;    // 4
};

// One column step.  x rows are [x0, m) of P, column i.  Returns false when
// the reflector is the identity (tau = 0).  Contains the syncs it needs; all
// threads call it with identical arguments.
template <typename R>
__device__ bool column_step(const ColumnStep<R> &c, int i, int x0, int m, int nc, bool tsqrt_form,
                            R *tau_out, bool zero_t_on_skip)
{
  const int tid = threadIdx.x;
  R *xcol = c.P + (size_t)i * c.ldp;
  // ---- norm of x ----
  R s = 0;
  for (int r = x0 + tid; r < m; r += TQR_THREADS) {
    R v = xcol[r];
    s = fma(v, v, s);
  }
  s = warp_sum(s);
  if ((tid & 31) == 0) c.part[tid >> 5] = s;
  __syncthreads();
  if (tid == 0) {
    R t = 0;
#pragma unroll
    for (int w = 0; w < TQR_WARPS; ++w) t += c.part[w];
    if (t != R(0)) {
      R beta, tv, sc;
      householder(c.row[(size_t)i * c.rs], t, beta, tv, sc);
      c.scal[0] = beta; c.scal[1] = tv; c.scal[2] = sc; c.scal[3] = R(1);
    } else {
      c.scal[3] = R(0);
    }
  }
  __syncthreads();
  if (c.scal[3] == R(0)) {
    if (tid == 0) *tau_out = R(0);
    if (zero_t_on_skip && c.Ts)
      for (int p = tid; p <= i; p += TQR_THREADS) c.Ts[p + (size_t)i * c.ldts] = R(0);
    __syncthreads();
    return false;
  }
  const R beta = c.scal[0], tv = c.scal[1], sc = c.scal[2];
  for (int r = x0 + tid; r < m; r += TQR_THREADS) xcol[r] *= sc;
  __syncthreads();
  // ---- d_j for all j != i (j < i only when T is built) ----
  const int jlo = c.Ts ? 0 : i + 1;
  const int nj = nc - jlo;
  if (nj > 0) {
    if (nj <= TQR_THREADS) {
      const int G = TQR_THREADS / nj;          // row groups
      const int j = jlo + tid % nj, g = tid / nj;
      if (g < G) {
        R a0 = 0, a1 = 0;
        if (j != i) {
          const R *pc = c.P + (size_t)j * c.ldp;
          int r = x0 + g;
          for (; r + G < m; r += 2 * G) {
            a0 = fma(pc[r], xcol[r], a0);
            a1 = fma(pc[r + G], xcol[r + G], a1);
          }
          if (r < m) a0 = fma(pc[r], xcol[r], a0);
        }
        c.part[g * nj + (j - jlo)] = a0 + a1;
      }
      __syncthreads();
      if (tid < nj) {
        const int jj = jlo + tid;
        R acc = 0;
        for (int gg = 0; gg < G; ++gg) acc += c.part[gg * nj + tid];
        if (jj > i || (!tsqrt_form && jj < i)) acc += c.row[(size_t)jj * c.rs];
        c.d[jj] = -tv * acc;
      }
    } else {
      const int lane = tid & 31, warp = tid >> 5;
      for (int j = jlo + warp; j < nc; j += TQR_WARPS) {
        if (j == i) continue;
        const R *pc = c.P + (size_t)j * c.ldp;
        R a = 0;
        for (int r = x0 + lane; r < m; r += 32) a = fma(pc[r], xcol[r], a);
        a = warp_sum(a);
        if (lane == 0) {
          if (j > i || (!tsqrt_form && j < i)) a += c.row[(size_t)j * c.rs];
          c.d[j] = -tv * a;
        }
      }
    }
  }
  __syncthreads();
  // ---- rank-1 update of the columns right of i ----
  {
    const int ncol = nc - i - 1, rows = m - x0;
    for (int j = i + 1 + tid; j < nc; j += TQR_THREADS) c.row[(size_t)j * c.rs] += c.d[j];
    for (int idx = tid; idx < ncol * rows; idx += TQR_THREADS) {
      const int rr = idx % rows, j = i + 1 + idx / rows;
      R *pc = c.P + (size_t)j * c.ldp;
      pc[x0 + rr] = fma(c.d[j], xcol[x0 + rr], pc[x0 + rr]);
    }
  }
  // ---- T column i ----
  if (c.Ts) {
    for (int p = tid; p < i; p += TQR_THREADS) {
      R acc = 0;
      for (int q = p; q < i; ++q) acc = fma(c.Ts[p + (size_t)q * c.ldts], c.d[q], acc);
      c.Ts[p + (size_t)i * c.ldts] = acc;
    }
    if (tid == 0) c.Ts[i + (size_t)i * c.ldts] = tv;
  }
  if (tid == 0) {
    c.row[(size_t)i * c.rs] = beta;
    *tau_out = tv;
  }
  __syncthreads();
  return true;
}

template <typename R>
__device__ inline R *carve(unsigned char *&p, size_t n) {
  R *r = reinterpret_cast<R *>(p);
  p += ((n * sizeof(R) + 15) / 16) * 16;
  return r;
}

// ---------------------------------------------------------------------------
// geqr2 (+ T).  P is the m-by-nc panel.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_panel_qr(int m, int nc, R *__restrict__ A, int lda, R *__restrict__ tau,
           R *__restrict__ T, int ldt, int staged, int stage_t)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x;
  ColumnStep<R> c;
  c.part = carve<R>(sp, TQR_THREADS);
  c.d = carve<R>(sp, nc);
  c.scal = carve<R>(sp, 4);
  if (T && stage_t) {
    c.ldts = odd_ld(nc);
    c.Ts = carve<R>(sp, (size_t)c.ldts * nc);
  } else {
    c.Ts = T;
    c.ldts = ldt;
  }
  if (staged) {
    c.ldp = odd_ld(m);
    c.P = carve<R>(sp, (size_t)c.ldp * nc);
    for (int idx = tid; idx < m * nc; idx += TQR_THREADS) {
      int r = idx % m, cc = idx / m;
      c.P[ix(r, cc, c.ldp)] = A[ix(r, cc, lda)];
    }
  } else {
    c.P = A;
    c.ldp = lda;
  }
  __syncthreads();
  const int k = min(m, nc);
  for (int i = 0; i < k; ++i) {
    c.row = c.P + i;
    c.rs = c.ldp;
    if (m - i <= 1) {                                  // geqr2.jl:32-35
      if (tid == 0) tau[i] = R(0);
      if (c.Ts)
        for (int p = tid; p <= i; p += TQR_THREADS) c.Ts[p + (size_t)i * c.ldts] = R(0);
      __syncthreads();
      continue;
    }
    column_step<R>(c, i, i + 1, m, nc, false, tau + i, true);
  }
  if (staged) {
    for (int idx = tid; idx < m * nc; idx += TQR_THREADS) {
      int r = idx % m, cc = idx / m;
      A[ix(r, cc, lda)] = c.P[ix(r, cc, c.ldp)];
    }
  }
  if (T && stage_t) {
    for (int idx = tid; idx < k * k; idx += TQR_THREADS) {
      int p = idx % k, q = idx / k;
      if (p <= q) T[ix(p, q, ldt)] = c.Ts[p + (size_t)q * c.ldts];
    }
  }
}

// ---------------------------------------------------------------------------
// One ib-block of tsqrt.  A1 points at A1[ii, ii] (sb-by-sb diagonal block,
// only its upper triangle is read or written), A2 at A2[0, ii] (m-by-sb),
// T at T[0, ii], tau at tau[ii].  A column whose A2 part is exactly zero gets
// tau = 0 and leaves its T column untouched, as the reference does
// (tsqrt.jl:61-64).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_tsqrt_block(int m, int sb, R *__restrict__ A1, int lda1, R *__restrict__ A2, int lda2,
              R *__restrict__ T, int ldt, R *__restrict__ tau, int staged)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x;
  ColumnStep<R> c;
  c.part = carve<R>(sp, TQR_THREADS);
  c.d = carve<R>(sp, sb);
  c.scal = carve<R>(sp, 4);
  const int ldb = odd_ld(sb);
  R *B = carve<R>(sp, (size_t)ldb * sb);
  c.ldts = odd_ld(sb);
  c.Ts = carve<R>(sp, (size_t)c.ldts * sb);
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      B[ix(r, cc, ldb)] = A1[ix(r, cc, lda1)];
      c.Ts[r + (size_t)cc * c.ldts] = T[ix(r, cc, ldt)];   // columns skipped below keep T
    }
  }
  if (staged) {
    c.ldp = odd_ld(m);
    c.P = carve<R>(sp, (size_t)c.ldp * sb);
    for (int idx = tid; idx < m * sb; idx += TQR_THREADS) {
      int r = idx % m, cc = idx / m;
      c.P[ix(r, cc, c.ldp)] = A2[ix(r, cc, lda2)];
    }
  } else {
    c.P = A2;
    c.ldp = lda2;
  }
  __syncthreads();
  c.rs = ldb;
  for (int i = 0; i < sb; ++i) {
    c.row = B + i;
    column_step<R>(c, i, 0, m, sb, true, tau + i, false);
  }
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      A1[ix(r, cc, lda1)] = B[ix(r, cc, ldb)];
      T[ix(r, cc, ldt)] = c.Ts[r + (size_t)cc * c.ldts];
    }
  }
  if (staged) {
    for (int idx = tid; idx < m * sb; idx += TQR_THREADS) {
      int r = idx % m, cc = idx / m;
      A2[ix(r, cc, lda2)] = c.P[ix(r, cc, c.ldp)];
    }
  }
}

// ---------------------------------------------------------------------------
// Stand-alone larft (all four direct/storev variants), one CTA.  The outer
// loop over reflectors stays serial as in the reference; the trailing-zero
// scan, the V^H v products and the triangular mat-vec are spread over the
// CTA.  Variant B keeps the reference's indexing (larft.jl:125-202).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_larft(int direct_f, int storev_c, int n, int k, const R *__restrict__ V, int ldv,
        const R *__restrict__ tau, R *__restrict__ T, int ldt)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *work = reinterpret_cast<R *>(smem_raw);   // k
  int *s_lastv = reinterpret_cast<int *>(work + (k > 0 ? k : 1));
  const int tid = threadIdx.x;
  auto Vc = [&](int r, int c) { return V[ix(r, c, ldv)]; };
  if (direct_f) {
    int prevlastv = n - 1;
    for (int i = 0; i < k; ++i) {
      prevlastv = max(prevlastv, i);
      const R ti = tau[i];
      if (ti == R(0)) {
        for (int j = tid; j <= i; j += TQR_THREADS) T[ix(j, i, ldt)] = R(0);
        __syncthreads();
        continue;
      }
      // lastv = last row (column for 'R') >= i+1 holding a nonzero, else i
      if (tid == 0) *s_lastv = i;
      __syncthreads();
      for (int r = n - 1 - tid; r >= i + 1; r -= TQR_THREADS) {
        R v = storev_c ? Vc(r, i) : Vc(i, r);
        if (v != R(0)) { atomicMax(s_lastv, r); break; }
      }
      __syncthreads();
      const int lastv = *s_lastv;
      const int j = min(lastv, prevlastv);
      for (int p = tid; p < i; p += TQR_THREADS) {
        R acc = 0;
        if (storev_c) {
          if (i + 1 <= j)
            for (int r = i + 1; r <= j; ++r) acc += Vc(r, p) * Vc(r, i);
          work[p] = -ti * Vc(i, p) + (-ti) * acc;
        } else {
          if (i > 0 && i + 1 <= j)
            for (int r = i + 1; r <= j; ++r) acc += Vc(p, r) * Vc(i, r);
          work[p] = -ti * Vc(p, i) + (-ti) * acc;
        }
      }
      prevlastv = (i > 0) ? max(prevlastv, lastv) : lastv;
      __syncthreads();
      for (int p = tid; p < i; p += TQR_THREADS) {
        R acc = 0;
        for (int q = p; q < i; ++q) acc += T[ix(p, q, ldt)] * work[q];
        T[ix(p, i, ldt)] = acc;
      }
      if (tid == 0) T[ix(i, i, ldt)] = ti;
      __syncthreads();
    }
  } else {
    int prevlastv = 0;
    for (int i = k - 1; i >= 0; --i) {
      const R ti = tau[i];
      if (ti == R(0)) {
        for (int j = i + tid; j < k; j += TQR_THREADS) T[ix(j, i, ldt)] = R(0);
        __syncthreads();
        continue;
      }
      if (i < k - 1) {
        if (tid == 0) *s_lastv = i;
        __syncthreads();
        // first index in 0..i-1 with V[idx, i] != 0 (the reference reads V[lastv, i]
        // for both storev values), else i
        for (int r = tid; r <= i - 1; r += TQR_THREADS) {
          if (Vc(r, i) != R(0)) { atomicMin(s_lastv, r); break; }
        }
        __syncthreads();
        const int lastv = *s_lastv;
        const int j = max(lastv, prevlastv);
        for (int p = i + 1 + tid; p < k; p += TQR_THREADS) {
          R acc = 0;
          R base;
          if (storev_c) {
            base = -ti * Vc(n - k + i, p);
            if (j <= n - k + i)
              for (int r = j; r <= n - k + i; ++r) acc += Vc(r, p) * Vc(r, k - 1);
          } else {
            base = -ti * Vc(p, n - k + i);
            if (j <= n - k + i - 1)
              for (int r = j; r <= n - k + i - 1; ++r) acc += Vc(p, r) * Vc(i, r);
          }
          work[p] = base + (-ti) * acc;
        }
        prevlastv = (i > 0) ? min(prevlastv, lastv) : lastv;
        __syncthreads();
        for (int p = i + 1 + tid; p < k; p += TQR_THREADS) {
          R acc = 0;
          for (int q = i + 1; q <= p; ++q) acc += T[ix(p, q, ldt)] * work[q];
          T[ix(p, i, ldt)] = acc;
        }
      }
      if (tid == 0) T[ix(i, i, ldt)] = ti;
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers (host).
// ---------------------------------------------------------------------------
static inline size_t rnd16(size_t b) { return ((b + 15) / 16) * 16; }

template <typename R>
static size_t panel_smem(int m, int nc, bool staged, bool stage_t) {
  size_t s = rnd16(sizeof(R) * TQR_THREADS) + rnd16(sizeof(R) * nc) + rnd16(sizeof(R) * 4);
  if (stage_t) s += rnd16(sizeof(R) * (size_t)odd_ld(nc) * nc);
  if (staged) s += rnd16(sizeof(R) * (size_t)odd_ld(m) * nc);
  return s;
}

template <typename K>
static cudaError_t allow_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename R>
cudaError_t launch_panel_qr(int m, int nc, R *A, int lda, R *tau, R *T, int ldt, cudaStream_t st) {
  const bool stage_t = (T != nullptr) && nc <= 64;
  bool staged = panel_smem<R>(m, nc, true, stage_t) <= (size_t)TQR_SMEM_MAX;
  size_t sm = panel_smem<R>(m, nc, staged, stage_t);
  if (sm > (size_t)TQR_SMEM_MAX) return cudaErrorInvalidValue;
  cudaError_t e = allow_smem(k_panel_qr<R>, sm);
  if (e != cudaSuccess) return e;
  k_panel_qr<R><<<1, TQR_THREADS, sm, st>>>(m, nc, A, lda, tau, T, ldt, staged ? 1 : 0, stage_t ? 1 : 0);
  count_launch();
  return cudaGetLastError();
}

template <typename R>
static size_t tsqrt_smem(int m, int sb, bool staged) {
  size_t s = rnd16(sizeof(R) * TQR_THREADS) + rnd16(sizeof(R) * sb) + rnd16(sizeof(R) * 4) +
             2 * rnd16(sizeof(R) * (size_t)odd_ld(sb) * sb);
  if (staged) s += rnd16(sizeof(R) * (size_t)odd_ld(m) * sb);
  return s;
}

template <typename R>
cudaError_t launch_tsqrt_block(int m, int sb, R *A1, int lda1, R *A2, int lda2, R *T, int ldt,
                               R *tau, cudaStream_t st) {
  bool staged = tsqrt_smem<R>(m, sb, true) <= (size_t)TQR_SMEM_MAX;
  size_t sm = tsqrt_smem<R>(m, sb, staged);
  if (sm > (size_t)TQR_SMEM_MAX) return cudaErrorInvalidValue;
  cudaError_t e = allow_smem(k_tsqrt_block<R>, sm);
  if (e != cudaSuccess) return e;
  k_tsqrt_block<R><<<1, TQR_THREADS, sm, st>>>(m, sb, A1, lda1, A2, lda2, T, ldt, tau, staged ? 1 : 0);
  count_launch();
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_larft(int direct_f, int storev_c, int n, int k, const R *V, int ldv,
                         const R *tau, R *T, int ldt, cudaStream_t st) {
  size_t sm = sizeof(R) * (size_t)(k > 0 ? k : 1) + 16;
  if (sm > (size_t)TQR_SMEM_MAX) return cudaErrorInvalidValue;
  cudaError_t e = allow_smem(k_larft<R>, sm);
  if (e != cudaSuccess) return e;
  k_larft<R><<<1, TQR_THREADS, sm, st>>>(direct_f, storev_c, n, k, V, ldv, tau, T, ldt);
  count_launch();
  return cudaGetLastError();
}

template cudaError_t launch_panel_qr<double>(int, int, double *, int, double *, double *, int, cudaStream_t);
template cudaError_t launch_panel_qr<float>(int, int, float *, int, float *, float *, int, cudaStream_t);
template cudaError_t launch_tsqrt_block<double>(int, int, double *, int, double *, int, double *, int, double *, cudaStream_t);
template cudaError_t launch_tsqrt_block<float>(int, int, float *, int, float *, int, float *, int, float *, cudaStream_t);
template cudaError_t launch_larft<double>(int, int, int, int, const double *, int, const double *, double *, int, cudaStream_t);
template cudaError_t launch_larft<float>(int, int, int, int, const float *, int, const float *, float *, int, cudaStream_t);

}  // namespace tqr
