// panel.cu -- stand-alone panel kernels (one CTA per panel) and launchers.
//
//  k_panel_qr     geqr2 with the larft T build fused in (NextLA src/geqr2.jl:23-105
//                 and src/larft.jl:53-86,112-124 for direct 'F', storev 'C').
//  k_tsqrt_block  one ib-block of tsqrt (NextLA src/tsqrt.jl:46-126).
//  k_larft        stand-alone larft for every direct/storev combination
//                 (NextLA src/larft.jl:48-203).
//
// The per-panel algorithms are panel_qr_cta / tsqrt_block_cta (panel_dev.cuh).
#include "panel_cluster.cuh"
#include "tileqr_internal.h"

namespace tqr {

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_panel_qr(int m, int nc, R *__restrict__ A, int lda, R *__restrict__ tau,
           R *__restrict__ T, int ldt, int staged, int stage_t)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  panel_qr_cta<R>(m, nc, A, lda, tau, T, ldt, staged != 0, stage_t != 0, smem_raw);
}

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_tsqrt_block(int m, int sb, R *__restrict__ A1, int lda1, R *__restrict__ A2, int lda2,
              R *__restrict__ T, int ldt, R *__restrict__ tau, int staged, int tt)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  tsqrt_block_cta<R>(m, sb, A1, lda1, A2, lda2, T, ldt, tau, staged != 0, smem_raw, tt);
}

template <typename E>
__global__ void __launch_bounds__(TQR_THREADS)
k_panel_cluster(const ClusterPanelArgs<E> a, int C)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cluster_panel<E>(a, C, smem_raw);
}

// ---------------------------------------------------------------------------
// Stand-alone larft (all four direct/storev variants), one CTA.  The outer
// loop over reflectors stays serial as in the reference; the trailing-zero
// scan, the V^H v products and the triangular mat-vec are spread over the
// CTA.  Variant B keeps the reference's indexing (larft.jl:125-202).  For
// complex elements the conjugates sit where the reference puts them
// (larft.jl:71-84, 98-108, 146-158, 171-180).
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
            for (int r = i + 1; r <= j; ++r) acc += conj_(Vc(r, p)) * Vc(r, i);
          work[p] = -ti * conj_(Vc(i, p)) + (-ti) * acc;
        } else {
          if (i > 0 && i + 1 <= j)
            for (int r = i + 1; r <= j; ++r) acc += Vc(p, r) * conj_(Vc(i, r));
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
            base = -ti * conj_(Vc(n - k + i, p));
            if (j <= n - k + i)
              for (int r = j; r <= n - k + i; ++r) acc += conj_(Vc(r, p)) * Vc(r, k - 1);
          } else {
            base = -ti * Vc(p, n - k + i);
            if (j <= n - k + i - 1)
              for (int r = j; r <= n - k + i - 1; ++r) acc += Vc(p, r) * conj_(Vc(i, r));
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
// ---------------------------------------------------------------------------
// Launchers (host).
// ---------------------------------------------------------------------------
template <typename K>
static cudaError_t allow_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Cluster size for a panel touching mrow rows: 0 when one CTA is the better
// choice (too few rows to split) or the columns exceed the cluster kernel's.
static int cluster_size_for(int mrow, int nc) {
  if (nc > 64) return 0;
  return mrow >= 192 ? 8 : (mrow >= 96 ? 4 : (mrow >= 64 ? 2 : 0));
}

// Launches the cluster panel; *used = false (and nothing launched) when the
// shape is better left to one CTA or its rows do not fit a cluster of 8.
template <typename E>
static cudaError_t launch_cluster(const ClusterPanelArgs<E> &a, int mrow, cudaStream_t st, bool *used) {
  *used = false;
  const int C = cluster_size_for(mrow, a.nc);
  if (!C) return cudaSuccess;
  const size_t sm = cluster_panel_smem<E>(mrow, a.nc, C);
  if (sm > (size_t)TQR_SMEM_MAX) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_panel_cluster<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, 1, 1);
  cfg.blockDim = dim3(TQR_THREADS, 1, 1);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, k_panel_cluster<E>, a, C);
  count_launch();
  *used = true;
  return e == cudaSuccess ? cudaGetLastError() : e;
}

template <typename R>
cudaError_t launch_panel_qr(int m, int nc, R *A, int lda, R *tau, R *T, int ldt, cudaStream_t st, bool cluster) {
  if (cluster) {
    ClusterPanelArgs<R> a{0, m, nc, A, lda, nullptr, 1, T, ldt, tau, -1};
    bool used = false;
    cudaError_t e = launch_cluster<R>(a, m, st, &used);
    if (used || e != cudaSuccess) return e;
  }
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
cudaError_t launch_tsqrt_block(int m, int sb, R *A1, int lda1, R *A2, int lda2, R *T, int ldt,
                               R *tau, cudaStream_t st, int tt, bool cluster) {
  const int mrow = tt >= 0 ? (m < tt + sb ? m : tt + sb) : m;
  if (cluster) {
    ClusterPanelArgs<R> a{1, m, sb, A2, lda2, A1, lda1, T, ldt, tau, tt};
    bool used = false;
    cudaError_t e = launch_cluster<R>(a, mrow, st, &used);
    if (used || e != cudaSuccess) return e;
  }
  bool staged = tsqrt_smem<R>(mrow, sb, true) <= (size_t)TQR_SMEM_MAX;
  size_t sm = tsqrt_smem<R>(mrow, sb, staged);
  if (sm > (size_t)TQR_SMEM_MAX) return cudaErrorInvalidValue;
  cudaError_t e = allow_smem(k_tsqrt_block<R>, sm);
  if (e != cudaSuccess) return e;
  k_tsqrt_block<R><<<1, TQR_THREADS, sm, st>>>(m, sb, A1, lda1, A2, lda2, T, ldt, tau, staged ? 1 : 0, tt);
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

template cudaError_t launch_panel_qr<double>(int, int, double *, int, double *, double *, int, cudaStream_t, bool);
template cudaError_t launch_panel_qr<float>(int, int, float *, int, float *, float *, int, cudaStream_t, bool);
template cudaError_t launch_tsqrt_block<double>(int, int, double *, int, double *, int, double *, int, double *, cudaStream_t, int, bool);
template cudaError_t launch_tsqrt_block<float>(int, int, float *, int, float *, int, float *, int, float *, cudaStream_t, int, bool);
template cudaError_t launch_larft<double>(int, int, int, int, const double *, int, const double *, double *, int, cudaStream_t);
template cudaError_t launch_larft<float>(int, int, int, int, const float *, int, const float *, float *, int, cudaStream_t);

#define TQR_PANEL_INST(E)                                                                                         \
  template cudaError_t launch_panel_qr<E>(int, int, E *, int, E *, E *, int, cudaStream_t, bool);                       \
  template cudaError_t launch_tsqrt_block<E>(int, int, E *, int, E *, int, E *, int, E *, cudaStream_t, int, bool);     \
  template cudaError_t launch_larft<E>(int, int, int, int, const E *, int, const E *, E *, int, cudaStream_t);
TQR_PANEL_INST(cx<double>)
TQR_PANEL_INST(cx<float>)
#undef TQR_PANEL_INST

}  // namespace tqr
