// tile.cu -- tile-QR driver, Q application, triangular solve and least squares.
//
// NextLA.jl ships the tile kernels only; the tile QR that composes them is the
// flat-tree PLASMA order
//     for k:  geqrt(A_kk);  unmqr('L','C') on A_kj (j > k);
//             for i > k:  tsqrt(A_kk, A_ik);  tsmqr('L','C') on (A_kj, A_ik-> A_ij)
// Every A_kj (j > k) lies in the same row band, so the unmqr and each tsmqr of
// a step are single calls over the whole band (one launch, one CTA per column
// strip).  The panel chain (geqrt, tsqrt) runs on a high-priority stream and
// the band updates on a second stream; tsmqr(k, i) waits only for tsqrt(k, i),
// so the serial tsqrt chain overlaps the updates.
//
// Layouts (column-major, 0-based):
//   A    m-by-n, lda >= m; R in the upper triangle of A[0:n, 0:n] on exit, V_kk
//        below the diagonal of the diagonal tiles, V_ik in the tiles below.
//   T    (MT*ib)-by-n, ldt >= MT*ib; T_ik occupies rows [i*ib, i*ib+ib),
//        columns [k*nb, k*nb + nb) -- the same ib-by-nb block NextLA's
//        geqrt!/tsqrt! write (src/geqrt.jl:49, src/tsqrt.jl:153).
//   tau  n-by-MT, ldtau >= n; tau of tile (i, k), column c at tau[k*nb + c + i*ldtau].
#include <mutex>

#include "common.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

using namespace tqr;

namespace {

// The kernels the driver composes: the C-ABI routines' bodies with the
// one-CTA panels, whose per-task arithmetic is the persistent schedule's, so
// the two drivers give the same bits.
template <typename R> struct K {
  static int geqrt(int m, int n, int ib, R *A, int lda, R *T, int ldt, R *tau, cudaStream_t s) {
    return geqrt_impl<R>(m, n, ib, A, lda, T, ldt, tau, s, false);
  }
  static int tsqrt(int m, int n, int ib, int m1, R *A1, int lda1, R *A2, int lda2, R *T, int ldt, R *tau,
                   cudaStream_t s) {
    return tsqrt_impl<R>(m, n, ib, m1, A1, lda1, A2, lda2, T, ldt, tau, s, false);
  }
  static int unmqr(char side, char trans, int m, int n, int k, int ib, const R *A, int lda, const R *T, int ldt,
                   R *C, int ldc, cudaStream_t s) {
    return unmqr_impl<R>(side, trans, m, n, k, ib, A, lda, T, ldt, C, ldc, s);
  }
  static int tsmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, R *A1, int lda1,
                   R *A2, int lda2, const R *V, int ldv, const R *T, int ldt, cudaStream_t s) {
    return tsmqr_impl<R>(side, trans, m1, n1, m2, n2, k, ib, A1, lda1, A2, lda2, V, ldv, T, ldt, s);
  }
};

// Internal streams of one device: a high-priority panel stream and a
// low-priority update stream, plus the events that order them.
struct DevStreams {
  bool init = false;
  cudaStream_t panel = nullptr, update = nullptr;
  cudaEvent_t fork = nullptr, ev_p = nullptr, ev_u = nullptr, join = nullptr;
};
constexpr int kMaxDev = 64;
DevStreams g_dev[kMaxDev];
std::mutex g_mu;

cudaError_t get_streams(DevStreams **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  DevStreams &d = g_dev[dev];
  if (!d.init) {
    int lo = 0, hi = 0;
    if ((e = cudaDeviceGetStreamPriorityRange(&lo, &hi)) != cudaSuccess) return e;
    if ((e = cudaStreamCreateWithPriority(&d.panel, cudaStreamNonBlocking, hi)) != cudaSuccess) return e;
    if ((e = cudaStreamCreateWithPriority(&d.update, cudaStreamNonBlocking, lo)) != cudaSuccess) return e;
    for (cudaEvent_t *ev : {&d.fork, &d.ev_p, &d.ev_u, &d.join})
      if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess) return e;
    d.init = true;
  }
  *out = &d;
  return cudaSuccess;
}

#define TQR_TRY(x)                 \
  do {                             \
    int _r = (x);                  \
    if (_r != 0) return _r;        \
  } while (0)
#define TQR_CU(x)                  \
  do {                             \
    cudaError_t _e = (x);          \
    if (_e != cudaSuccess) return (int)_e; \
  } while (0)

template <typename R>
int tile_geqrf(int m, int n, int nb, int ib, R *A, int lda, R *T, int ldt, R *tau, int ldtau,
               cudaStream_t st) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (nb <= 0) return -3;
  if (ib <= 0 || ib > nb) return -4;
  if (m == 0 || n == 0) return 0;
  const int MT = (m + nb - 1) / nb, NT = (n + nb - 1) / nb, KT = MT < NT ? MT : NT;
  if (lda < m) return -6;
  if (ldt < MT * ib) return -8;
  if (ldtau < n) return -10;
  std::lock_guard<std::mutex> lock(g_mu);
  DevStreams *ds = nullptr;
  TQR_CU(get_streams(&ds));
  cudaStream_t P = ds->panel, U = ds->update;
  TQR_CU(cudaEventRecord(ds->fork, st));
  TQR_CU(cudaStreamWaitEvent(P, ds->fork, 0));
  TQR_CU(cudaStreamWaitEvent(U, ds->fork, 0));
  for (int k = 0; k < KT; ++k) {
    const int mk = nb < m - k * nb ? nb : m - k * nb;
    const int nk = nb < n - k * nb ? nb : n - k * nb;
    const int kk = mk < nk ? mk : nk;
    const int ntrail = n - (k + 1) * nb;            // columns right of the panel
    R *Akk = A + ix(k * nb, k * nb, lda);
    R *Tkk = T + ix(k * ib, k * nb, ldt);
    TQR_TRY(K<R>::geqrt(mk, nk, ib, Akk, lda, Tkk, ldt, tau + ix(k * nb, k, ldtau), P));
    if (ntrail > 0) {
      TQR_CU(cudaEventRecord(ds->ev_p, P));
      TQR_CU(cudaStreamWaitEvent(U, ds->ev_p, 0));
      void *tok = prof_begin(U);
      TQR_TRY(K<R>::unmqr('L', 'C', mk, ntrail, kk, ib, Akk, lda, Tkk, ldt,
                          A + ix(k * nb, (k + 1) * nb, lda), lda, U));
      prof_end(tok, U, 2.0 * ntrail * kk * (2.0 * mk - kk));
    }
    for (int i = k + 1; i < MT; ++i) {
      const int mi = nb < m - i * nb ? nb : m - i * nb;
      R *Aik = A + ix(i * nb, k * nb, lda);
      R *Tik = T + ix(i * ib, k * nb, ldt);
      TQR_TRY(K<R>::tsqrt(mi, nk, ib, mk, Akk, lda, Aik, lda, Tik, ldt, tau + ix(k * nb, i, ldtau), P));
      if (ntrail > 0) {
        TQR_CU(cudaEventRecord(ds->ev_p, P));
        TQR_CU(cudaStreamWaitEvent(U, ds->ev_p, 0));
        void *tok = prof_begin(U);
        TQR_TRY(K<R>::tsmqr('L', 'C', mk, ntrail, mi, ntrail, kk, ib, A + ix(k * nb, (k + 1) * nb, lda), lda,
                            A + ix(i * nb, (k + 1) * nb, lda), lda, Aik, lda, Tik, ldt, U));
        prof_end(tok, U, 4.0 * mi * kk * (double)ntrail);
      }
    }
    TQR_CU(cudaEventRecord(ds->ev_u, U));
    TQR_CU(cudaStreamWaitEvent(P, ds->ev_u, 0));
  }
  TQR_CU(cudaEventRecord(ds->join, P));
  TQR_CU(cudaStreamWaitEvent(st, ds->join, 0));
  return 0;
}

template <typename R>
int tile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const R *A, int lda, const R *T,
               int ldt, R *B, int ldb, cudaStream_t st) {
  if (trans != 'N' && trans != 'C' && trans != 'T') return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (nb <= 0) return -5;
  if (ib <= 0 || ib > nb) return -6;
  if (m == 0 || n == 0 || nrhs == 0) return 0;
  const int MT = (m + nb - 1) / nb, NT = (n + nb - 1) / nb, KT = MT < NT ? MT : NT;
  if (lda < m) return -8;
  if (ldt < MT * ib) return -10;
  if (ldb < m) return -12;
  auto band = [&](int k, int &mk, int &kk) {
    mk = nb < m - k * nb ? nb : m - k * nb;
    const int nk = nb < n - k * nb ? nb : n - k * nb;
    kk = mk < nk ? mk : nk;
  };
  if (trans != 'N') {
    for (int k = 0; k < KT; ++k) {
      int mk, kk;
      band(k, mk, kk);
      TQR_TRY(K<R>::unmqr('L', 'C', mk, nrhs, kk, ib, A + ix(k * nb, k * nb, lda), lda,
                          T + ix(k * ib, k * nb, ldt), ldt, B + ix(k * nb, 0, ldb), ldb, st));
      for (int i = k + 1; i < MT; ++i) {
        const int mi = nb < m - i * nb ? nb : m - i * nb;
        TQR_TRY(K<R>::tsmqr('L', 'C', mk, nrhs, mi, nrhs, kk, ib, B + ix(k * nb, 0, ldb), ldb,
                            B + ix(i * nb, 0, ldb), ldb, A + ix(i * nb, k * nb, lda), lda,
                            T + ix(i * ib, k * nb, ldt), ldt, st));
      }
    }
  } else {
    for (int k = KT - 1; k >= 0; --k) {
      int mk, kk;
      band(k, mk, kk);
      for (int i = MT - 1; i > k; --i) {
        const int mi = nb < m - i * nb ? nb : m - i * nb;
        TQR_TRY(K<R>::tsmqr('L', 'N', mk, nrhs, mi, nrhs, kk, ib, B + ix(k * nb, 0, ldb), ldb,
                            B + ix(i * nb, 0, ldb), ldb, A + ix(i * nb, k * nb, lda), lda,
                            T + ix(i * ib, k * nb, ldt), ldt, st));
      }
      TQR_TRY(K<R>::unmqr('L', 'N', mk, nrhs, kk, ib, A + ix(k * nb, k * nb, lda), lda,
                          T + ix(k * ib, k * nb, ldt), ldt, B + ix(k * nb, 0, ldb), ldb, st));
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Upper-triangular solve R X = B.  Blocked from the bottom: the diagonal
// block is solved by one CTA per right-hand side with the arithmetic of
// NextLA's LeftUpperTRSM! kernel (src/trsm.jl:38-63: b scaled by the
// diagonal, then b[r] -= (R[r,i] / R[r,r]) b[i]); the rows above are updated
// with C -= R_blk X_blk.  No size limit (the reference kernel stops at 1024).
// ---------------------------------------------------------------------------

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_trsv_block(int nb, const R *__restrict__ Rm, int ldr, R *__restrict__ B, int ldb)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *b = reinterpret_cast<R *>(smem_raw);
  R *dg = b + nb;
  R *col = B + (size_t)blockIdx.x * ldb;
  for (int r = threadIdx.x; r < nb; r += TQR_THREADS) {
    dg[r] = Rm[ix(r, r, ldr)];
    b[r] = div_(col[r], dg[r]);
  }
  __syncthreads();
  for (int i = nb - 1; i > 0; --i) {
    const R bi = b[i];
    for (int r = threadIdx.x; r < i; r += TQR_THREADS) b[r] -= div_(Rm[ix(r, i, ldr)], dg[r]) * bi;
    __syncthreads();
  }
  for (int r = threadIdx.x; r < nb; r += TQR_THREADS) col[r] = b[r];
}

// C (m-by-n) -= A (m-by-k) * B (k-by-n).  64-row by 16-column output tile per
// CTA, 32-deep k chunks through shared memory, 4 outputs per thread.
template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_gemm_nn_sub(int m, int n, int k, const R *__restrict__ A, int lda, const R *__restrict__ B, int ldb,
              R *__restrict__ C, int ldc)
{
  __shared__ R As[32][65];
  __shared__ R Bs[16][33];
  const int r0 = blockIdx.x * 64, c0 = blockIdx.y * 16;
  const int tid = threadIdx.x;
  const int tr = tid % 64, tc = tid / 64;          // rows tr; columns tc, tc+4, tc+8, tc+12
  R acc[4] = {0, 0, 0, 0};
  for (int k0 = 0; k0 < k; k0 += 32) {
    for (int idx = tid; idx < 64 * 32; idx += TQR_THREADS) {
      int r = idx % 64, kk = idx / 64;
      As[kk][r] = (r0 + r < m && k0 + kk < k) ? A[ix(r0 + r, k0 + kk, lda)] : R(0);
    }
    for (int idx = tid; idx < 32 * 16; idx += TQR_THREADS) {
      int kk = idx % 32, c = idx / 32;
      Bs[c][kk] = (k0 + kk < k && c0 + c < n) ? B[ix(k0 + kk, c0 + c, ldb)] : R(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      const R a = As[kk][tr];
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j] += a * Bs[tc + 4 * j][kk];
    }
    __syncthreads();
  }
  if (r0 + tr < m) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (c0 + tc + 4 * j < n) C[ix(r0 + tr, c0 + tc + 4 * j, ldc)] -= acc[j];
  }
}

template <typename R>
int trsm_lun(int n, int nrhs, const R *Rm, int ldr, R *B, int ldb, cudaStream_t st) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (n == 0 || nrhs == 0) return 0;
  if (ldr < n) return -4;
  if (ldb < n) return -6;
  const int bs = 256;
  TQR_CU(cudaFuncSetAttribute(k_trsv_block<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TQR_SMEM_MAX));
  for (int b0 = ((n - 1) / bs) * bs; b0 >= 0; b0 -= bs) {
    const int nbk = bs < n - b0 ? bs : n - b0;
    k_trsv_block<R><<<nrhs, TQR_THREADS, 2 * nbk * sizeof(R), st>>>(nbk, Rm + ix(b0, b0, ldr), ldr, B + b0, ldb);
    count_launch();
    TQR_CU(cudaGetLastError());
    if (b0 > 0) {
      dim3 grid((b0 + 63) / 64, (nrhs + 15) / 16);
      k_gemm_nn_sub<R><<<grid, TQR_THREADS, 0, st>>>(b0, nrhs, nbk, Rm + ix(0, b0, ldr), ldr, B + b0, ldb, B, ldb);
      count_launch();
      TQR_CU(cudaGetLastError());
    }
  }
  return 0;
}

template <typename R>
int tile_gels(int m, int n, int nrhs, int nb, int ib, R *A, int lda, R *T, int ldt, R *tau, int ldtau,
              R *B, int ldb, cudaStream_t st) {
  if (m < n) return -1;   // overdetermined or square systems only
  TQR_TRY(tile_geqrf<R>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, st));
  TQR_TRY(tile_unmqr<R>('C', m, n, nrhs, nb, ib, A, lda, T, ldt, B, ldb, st));
  TQR_TRY(trsm_lun<R>(n, nrhs, A, lda, B, ldb, st));
  return 0;
}

}  // namespace

extern "C" {

int tqr_dtile_geqrf(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt, double *tau,
                    int ldtau, cudaStream_t stream) {
  return tile_geqrf<double>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, stream);
}
int tqr_stile_geqrf(int m, int n, int nb, int ib, float *A, int lda, float *T, int ldt, float *tau,
                    int ldtau, cudaStream_t stream) {
  return tile_geqrf<float>(m, n, nb, ib, A, lda, T, ldt, tau, ldtau, stream);
}
int tqr_dtile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const double *A, int lda,
                    const double *T, int ldt, double *B, int ldb, cudaStream_t stream) {
  return tile_unmqr<double>(trans, m, n, nrhs, nb, ib, A, lda, T, ldt, B, ldb, stream);
}
int tqr_stile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const float *A, int lda,
                    const float *T, int ldt, float *B, int ldb, cudaStream_t stream) {
  return tile_unmqr<float>(trans, m, n, nrhs, nb, ib, A, lda, T, ldt, B, ldb, stream);
}
int tqr_ztile_geqrf(int m, int n, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T, int ldt,
                    tqr_zcomplex *tau, int ldtau, cudaStream_t stream) {
  using E = cx<double>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)tau) % alignof(E)) return -5;
  return tile_geqrf<E>(m, n, nb, ib, (E *)A, lda, (E *)T, ldt, (E *)tau, ldtau, stream);
}
int tqr_ctile_geqrf(int m, int n, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T, int ldt,
                    tqr_ccomplex *tau, int ldtau, cudaStream_t stream) {
  using E = cx<float>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)tau) % alignof(E)) return -5;
  return tile_geqrf<E>(m, n, nb, ib, (E *)A, lda, (E *)T, ldt, (E *)tau, ldtau, stream);
}
int tqr_ztile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const tqr_zcomplex *A, int lda,
                    const tqr_zcomplex *T, int ldt, tqr_zcomplex *B, int ldb, cudaStream_t stream) {
  using E = cx<double>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)B) % alignof(E)) return -7;
  return tile_unmqr<E>(trans, m, n, nrhs, nb, ib, (const E *)A, lda, (const E *)T, ldt, (E *)B, ldb, stream);
}
int tqr_ctile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const tqr_ccomplex *A, int lda,
                    const tqr_ccomplex *T, int ldt, tqr_ccomplex *B, int ldb, cudaStream_t stream) {
  using E = cx<float>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)B) % alignof(E)) return -7;
  return tile_unmqr<E>(trans, m, n, nrhs, nb, ib, (const E *)A, lda, (const E *)T, ldt, (E *)B, ldb, stream);
}
int tqr_ztrsm_lun(int n, int nrhs, const tqr_zcomplex *R, int ldr, tqr_zcomplex *B, int ldb, cudaStream_t stream) {
  using E = cx<double>;
  if (((uintptr_t)R | (uintptr_t)B) % alignof(E)) return -3;
  return trsm_lun<E>(n, nrhs, (const E *)R, ldr, (E *)B, ldb, stream);
}
int tqr_ctrsm_lun(int n, int nrhs, const tqr_ccomplex *R, int ldr, tqr_ccomplex *B, int ldb, cudaStream_t stream) {
  using E = cx<float>;
  if (((uintptr_t)R | (uintptr_t)B) % alignof(E)) return -3;
  return trsm_lun<E>(n, nrhs, (const E *)R, ldr, (E *)B, ldb, stream);
}
int tqr_ztile_gels(int m, int n, int nrhs, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T, int ldt,
                   tqr_zcomplex *tau, int ldtau, tqr_zcomplex *B, int ldb, cudaStream_t stream) {
  using E = cx<double>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)tau | (uintptr_t)B) % alignof(E)) return -6;
  return tile_gels<E>(m, n, nrhs, nb, ib, (E *)A, lda, (E *)T, ldt, (E *)tau, ldtau, (E *)B, ldb, stream);
}
int tqr_ctile_gels(int m, int n, int nrhs, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T, int ldt,
                   tqr_ccomplex *tau, int ldtau, tqr_ccomplex *B, int ldb, cudaStream_t stream) {
  using E = cx<float>;
  if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)tau | (uintptr_t)B) % alignof(E)) return -6;
  return tile_gels<E>(m, n, nrhs, nb, ib, (E *)A, lda, (E *)T, ldt, (E *)tau, ldtau, (E *)B, ldb, stream);
}
int tqr_dtrsm_lun(int n, int nrhs, const double *R, int ldr, double *B, int ldb, cudaStream_t stream) {
  return trsm_lun<double>(n, nrhs, R, ldr, B, ldb, stream);
}
int tqr_strsm_lun(int n, int nrhs, const float *R, int ldr, float *B, int ldb, cudaStream_t stream) {
  return trsm_lun<float>(n, nrhs, R, ldr, B, ldb, stream);
}
int tqr_dtile_gels(int m, int n, int nrhs, int nb, int ib, double *A, int lda, double *T, int ldt,
                   double *tau, int ldtau, double *B, int ldb, cudaStream_t stream) {
  return tile_gels<double>(m, n, nrhs, nb, ib, A, lda, T, ldt, tau, ldtau, B, ldb, stream);
}
int tqr_stile_gels(int m, int n, int nrhs, int nb, int ib, float *A, int lda, float *T, int ldt,
                   float *tau, int ldtau, float *B, int ldb, cudaStream_t stream) {
  return tile_gels<float>(m, n, nrhs, nb, ib, A, lda, T, ldt, tau, ldtau, B, ldb, stream);
}

}  // extern "C"
