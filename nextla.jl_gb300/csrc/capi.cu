// capi.cu -- C-ABI entry points mirroring NextLA.jl's tile kernels.
//
// Every entry point checks its arguments the way the reference's Julia method
// does and returns -i for an illegal i-th argument (1-based position in the C
// signature; the reference throws ArgumentError), 0 on success, or a positive
// cudaError_t code when a launch fails.  All calls are asynchronous on
// `stream`; the reference is blocking, so a binding that wants its semantics
// synchronises the stream after the call (the Python and Julia front ends do).
// The `work` arguments of the reference are accepted and not used: the W
// blocks of every routine live in shared memory.
#include <cstdint>

#include "common.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

using namespace tqr;

namespace {

inline bool is_side(char c) { return c == 'L' || c == 'R'; }
inline bool is_trans(char c) { return c == 'N' || c == 'C' || c == 'T'; }
inline int rc(cudaError_t e) { return e == cudaSuccess ? 0 : (int)e; }

// C-ABI element pointer -> device element pointer (same layout)
template <typename R, typename C> inline R *dp(C *p) { return reinterpret_cast<R *>(p); }
template <typename R, typename C> inline const R *dp(const C *p) { return reinterpret_cast<const R *>(p); }
template <typename R> inline bool al(const void *p) { return ((uintptr_t)p % alignof(R)) == 0; }

template <typename R>
int geqr2_impl(int m, int n, R *A, int lda, R *tau, cudaStream_t st) {
  if (m < 0) return -1;                      // src/geqr2.jl:108-113
  if (n < 0) return -2;
  if (lda < (m > 1 ? m : 1)) return -4;
  if (m == 0 || n == 0) return 0;
  return rc(launch_panel_qr<R>(m, n, A, lda, tau, (R *)nullptr, 1, st, true));
}

template <typename R>
int larft_impl(char direct, char storev, int n, int k, const R *V, int ldv, const R *tau, R *T,
               int ldt, cudaStream_t st) {
  if (n == 0) return 0;                      // src/larft.jl:206
  if (direct != 'F' && direct != 'B') return -1;
  if (storev != 'C' && storev != 'R') return -2;
  if (n < 0) return -3;
  if (k < 0) return -4;
  if (k == 0) return 0;
  if (ldt < k) return -9;
  return rc(launch_larft<R>(direct == 'F', storev == 'C', n, k, V, ldv, tau, T, ldt, st));
}

template <typename R>
int larfb_impl(char side, char trans, char direct, char storev, int m, int n, int k, const R *V,
               int ldv, const R *T, int ldt, R *C, int ldc, cudaStream_t st) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;  // src/larfb.jl:38-40
  if (direct != 'F') return -3;              // src/larfb.jl:42-44
  if (storev != 'C') return -4;
  if (!is_side(side)) return -1;
  if (!is_trans(trans)) return -2;
  if (ldv < (side == 'L' ? m : n)) return -9;
  if (ldt < k) return -11;
  if (ldc < m) return -13;
  if (k > (side == 'L' ? m : n)) return -7;
  return rc(launch_apply<R>(0, side, trans, m, n, k, k, C, ldc, (R *)nullptr, 0, V, ldv, T, ldt, st));
}

}  // namespace

namespace tqr {

template <typename R>
int geqrt_impl(int m, int n, int ib, R *A, int lda, R *T, int ldt, R *tau, cudaStream_t st, bool cluster) {
  if (m < 0) return -1;                      // src/geqrt.jl:24-34
  if (n < 0) return -2;
  if (ib < 0 || (ib == 0 && m > 0 && n > 0)) return -3;
  if (m == 0 || n == 0 || ib == 0) return 0;
  if (lda < m) return -5;
  if (ldt < ib) return -7;
  const int k = m < n ? m : n;
  for (int i = 0; i < k; i += ib) {          // src/geqrt.jl:44-67
    const int sb = ib < k - i ? ib : k - i;
    R *av = A + ix(i, i, lda);
    R *tv = T + ix(0, i, ldt);
    cudaError_t e = launch_panel_qr<R>(m - i, sb, av, lda, tau + i, tv, ldt, st, cluster);
    if (e != cudaSuccess) return rc(e);
    if (n > i + sb) {
      e = launch_apply<R>(0, 'L', 'C', m - i, n - i - sb, sb, sb, A + ix(i, i + sb, lda), lda,
                          (R *)nullptr, 0, av, lda, tv, ldt, st);
      if (e != cudaSuccess) return rc(e);
    }
  }
  return 0;
}

template <typename R>
int unmqr_impl(char side, char trans, int m, int n, int k, int ib, const R *A, int lda, const R *T,
               int ldt, R *C, int ldc, cudaStream_t st) {
  if (!is_side(side)) return -1;             // src/unmqr.jl:54-91
  const int nq = side == 'L' ? m : n;
  if (!is_trans(trans)) return -2;
  if (m < 0) return -3;
  if (n < 0) return -4;
  if (k < 0) return -5;
  if (k > nq) k = nq;                        // src/unmqr.jl:83
  if (ib < 0) return -6;
  if (lda < (nq > 1 ? nq : 1) && nq > 0) return -8;
  if (m == 0 || n == 0 || k == 0) return 0;
  if (ib == 0) return -6;                    // a zero step is an error in the reference loop
  if (ldt < (ib < k ? ib : k)) return -10;
  if (ldc < m) return -12;
  return rc(launch_apply<R>(0, side, trans, m, n, k, ib, C, ldc, (R *)nullptr, 0, A, lda, T, ldt, st));
}

template <typename R>
int tsmqr_impl(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, R *A1,
               int lda1, R *A2, int lda2, const R *V, int ldv, const R *T, int ldt, cudaStream_t st) {
  if (!is_side(side)) return -1;             // src/tsmqr.jl:51-91
  if (!is_trans(trans)) return -2;
  if (m1 < 0) return -3;
  if (n1 < 0) return -4;
  if (m2 < 0 || (m2 != m1 && side == 'R')) return -5;
  if (n2 < 0 || (n2 != n1 && side == 'L')) return -6;
  if (k < 0) return -7;
  if (ib < 0) return -8;
  const int kmax = side == 'L' ? m1 : n1;    // src/tsmqr.jl:93-96 (stored-k clamp is the caller's)
  if (k > kmax) k = kmax;
  if (m1 == 0 || n1 == 0 || m2 == 0 || n2 == 0 || k == 0 || ib == 0) return 0;
  if (lda1 < m1) return -10;
  if (lda2 < m2) return -12;
  if (ldv < (side == 'L' ? m2 : n2)) return -14;
  if (ldt < (ib < k ? ib : k)) return -16;
  return rc(launch_apply<R>(1, side, trans, m2, n2, k, ib, A2, lda2, A1, lda1, V, ldv, T, ldt, st));
}

}  // namespace tqr

namespace {

template <typename R>
int parfb_impl(char side, char trans, char direct, char storev, int m1, int n1, int m2, int n2,
               int k, int l, R *A1, int lda1, R *A2, int lda2, const R *V, int ldv, const R *T,
               int ldt, R *work, int ldwork, cudaStream_t st) {
  if (!is_side(side)) return -1;             // src/parfb.jl:47-85
  if (!is_trans(trans)) return -2;
  if (direct != 'F' && direct != 'B') return -3;
  if (storev != 'C' && storev != 'R') return -4;
  if (m1 < 0) return -5;
  if (n1 < 0) return -6;
  if (m2 < 0 || (side == 'R' && m1 != m2)) return -7;
  if (n2 < 0 || (side == 'L' && n1 != n2)) return -8;
  if (k < 0) return -9;
  if (l < 0 || l > k) return -10;
  if (m1 == 0 || n1 == 0 || n2 == 0 || k == 0) return 0;
  if (m2 == 0) return 0;
  // Forward, columnwise reflectors (the forms tsmqr! and ttmqr! use) run in
  // the fused apply: a triangular part of order l makes reflector q hold rows
  // (columns for side R) [0, mv - l + q] of V, mv = m2 (n2): pamm's trapezoid
  // (src/pamm.jl:104-127, 153-175).  The other forms go through pamm with the
  // caller's work (k x n2 for side L, m2 x k for R).
  const int mv = side == 'L' ? m2 : n2;
  if (direct != 'F' || storev != 'C') {
    if (!work || ldwork < (side == 'L' ? k : m2)) return -20;
    return parfb_general<R>(side, trans, direct, storev, m2, n2, k, l, A1, lda1, A2, lda2, V, ldv, T, ldt, work,
                            ldwork, st);
  }
  return rc(launch_apply<R>(1, side, trans, m2, n2, k, k, A2, lda2, A1, lda1, V, ldv, T, ldt, st,
                            l > 0 ? mv - l : -1));
}

template <typename R>
int ttmqr_impl(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, R *A1,
               int lda1, R *A2, int lda2, const R *V, int ldv, const R *T, int ldt, cudaStream_t st) {
  if (!is_side(side)) return -1;             // src/ttmqr.jl:3-37
  if (!is_trans(trans)) return -2;
  if (m1 < 0) return -3;
  if (n1 < 0) return -4;
  if (m2 < 0 || (m2 != m1 && side == 'R')) return -5;
  if (n2 < 0 || (n2 != n1 && side == 'L')) return -6;
  if (k < 0) return -7;
  const int kmax = side == 'L' ? m1 : n1;
  if (k > kmax) k = kmax;
  if (ib < 0) return -8;
  if (m1 == 0 || n1 == 0 || m2 == 0 || n2 == 0 || k == 0 || ib == 0) return 0;
  if (lda1 < m1) return -10;
  if (lda2 < m2) return -12;
  if (ldv < (side == 'L' ? m2 : n2)) return -14;
  if (ldt < (ib < k ? ib : k)) return -16;
  // block i touches A2 rows (columns) [0, min(i + kb, m2)), reflector q of V
  // rows [0, q]: the apply's triangular form with offset 0
  return rc(launch_apply<R>(1, side, trans, m2, n2, k, ib, A2, lda2, A1, lda1, V, ldv, T, ldt, st, 0));
}

template <typename R>
int ttqrt_impl(int m, int n, int ib, R *A1, int lda1, R *A2, int lda2, R *T, int ldt, R *tau,
               cudaStream_t st) {
  if (m < 0) return -1;                      // src/ttqrt.jl:86-101
  if (n < 0) return -2;
  if (ib < 0) return -3;
  if (m == 0 || n == 0 || ib == 0) return 0;
  const int k = m < n ? m : n;
  if (lda1 < k) return -5;
  if (lda2 < m) return -7;
  if (ldt < (ib < k ? ib : k)) return -9;
  for (int ii = 0; ii < k; ii += ib) {       // src/ttqrt.jl:102-117
    const int sb = (k - ii) < ib ? (k - ii) : ib;
    cudaError_t e = launch_tsqrt_block<R>(m, sb, A1 + ix(ii, ii, lda1), lda1, A2 + ix(0, ii, lda2),
                                          lda2, T + ix(0, ii, ldt), ldt, tau + ii, st, ii, true);
    if (e != cudaSuccess) return rc(e);
    if (n > ii + sb) {
      const int mi = (ii + sb) < m ? (ii + sb) : m;
      e = launch_apply<R>(1, 'L', 'C', mi, n - ii - sb, sb, ib, A2 + ix(0, ii + sb, lda2), lda2,
                          A1 + ix(ii, ii + sb, lda1), lda1, A2 + ix(0, ii, lda2), lda2,
                          T + ix(0, ii, ldt), ldt, st, ii);
      if (e != cudaSuccess) return rc(e);
    }
  }
  return 0;
}

}  // namespace

namespace tqr {

template <typename R>
int tsqrt_impl(int m, int n, int ib, int m1, R *A1, int lda1, R *A2, int lda2, R *T, int ldt,
               R *tau, cudaStream_t st, bool cluster) {
  if (m < 0) return -1;                      // src/tsqrt.jl:129-144
  if (n < 0) return -2;
  if (ib < 0) return -3;
  if (m1 < 0) return -4;
  const int k = m1 < n ? m1 : n;
  if (m == 0 || n == 0 || ib == 0 || k == 0) return 0;
  if (lda1 < m1) return -6;
  if (lda2 < m) return -8;
  if (ldt < ib) return -10;
  for (int ii = 0; ii < k; ii += ib) {       // src/tsqrt.jl:146-155
    const int sb = (k - ii) < ib ? (k - ii) : ib;
    cudaError_t e = launch_tsqrt_block<R>(m, sb, A1 + ix(ii, ii, lda1), lda1, A2 + ix(0, ii, lda2),
                                          lda2, T + ix(0, ii, ldt), ldt, tau + ii, st, -1, cluster);
    if (e != cudaSuccess) return rc(e);
    if (n > ii + sb) {
      e = launch_apply<R>(1, 'L', 'C', m, n - ii - sb, sb, ib, A2 + ix(0, ii + sb, lda2), lda2,
                          A1 + ix(ii, ii + sb, lda1), lda1, A2 + ix(0, ii, lda2), lda2,
                          T + ix(0, ii, ldt), ldt, st);
      if (e != cudaSuccess) return rc(e);
    }
  }
  return 0;
}

#define TQR_IMPL_INST(R)                                                                                  \
  template int geqrt_impl<R>(int, int, int, R *, int, R *, int, R *, cudaStream_t, bool);                \
  template int tsqrt_impl<R>(int, int, int, int, R *, int, R *, int, R *, int, R *, cudaStream_t, bool); \
  template int unmqr_impl<R>(char, char, int, int, int, int, const R *, int, const R *, int, R *, int,   \
                             cudaStream_t);                                                              \
  template int tsmqr_impl<R>(char, char, int, int, int, int, int, int, R *, int, R *, int, const R *, int, \
                             const R *, int, cudaStream_t);
TQR_IMPL_INST(double)
TQR_IMPL_INST(float)
TQR_IMPL_INST(cx<double>)
TQR_IMPL_INST(cx<float>)
#undef TQR_IMPL_INST

}  // namespace tqr

extern "C" {

// P: the BLAS-style prefix; CT: the element type of the C signature
// (tileqr.h); R: the device element type (the same type for real elements,
// cx<double> / cx<float> for tqr_zcomplex / tqr_ccomplex, which share their
// layout).  A pointer not aligned to the element size (16 bytes for
// ComplexF64, 8 for ComplexF32) is an illegal argument.
#define TQR_INSTANTIATE(P, CT, R)                                                                    \
  int tqr_##P##geqr2(int m, int n, CT *A, int lda, CT *tau, CT *work, cudaStream_t stream) {         \
    (void)work;                                                                                      \
    if (!al<R>(A)) return -3;                                                                        \
    if (!al<R>(tau)) return -5;                                                                      \
    return geqr2_impl<R>(m, n, dp<R>(A), lda, dp<R>(tau), stream);                                   \
  }                                                                                                  \
  int tqr_##P##larft(char direct, char storev, int n, int k, const CT *V, int ldv, const CT *tau,    \
                     CT *T, int ldt, cudaStream_t stream) {                                          \
    if (!al<R>(V)) return -5;                                                                        \
    if (!al<R>(tau)) return -7;                                                                      \
    if (!al<R>(T)) return -8;                                                                        \
    return larft_impl<R>(direct, storev, n, k, dp<R>(V), ldv, dp<R>(tau), dp<R>(T), ldt, stream);    \
  }                                                                                                  \
  int tqr_##P##larfb(char side, char trans, char direct, char storev, int m, int n, int k,           \
                     const CT *V, int ldv, const CT *T, int ldt, CT *C, int ldc, CT *work,           \
                     int ldwork, cudaStream_t stream) {                                              \
    (void)work; (void)ldwork;                                                                        \
    if (!al<R>(V)) return -8;                                                                        \
    if (!al<R>(T)) return -10;                                                                       \
    if (!al<R>(C)) return -12;                                                                       \
    return larfb_impl<R>(side, trans, direct, storev, m, n, k, dp<R>(V), ldv, dp<R>(T), ldt,         \
                         dp<R>(C), ldc, stream);                                                     \
  }                                                                                                  \
  int tqr_##P##geqrt(int m, int n, int ib, CT *A, int lda, CT *T, int ldt, CT *tau, CT *work,        \
                     cudaStream_t stream) {                                                          \
    (void)work;                                                                                      \
    if (!al<R>(A)) return -4;                                                                        \
    if (!al<R>(T)) return -6;                                                                        \
    if (!al<R>(tau)) return -8;                                                                      \
    return geqrt_impl<R>(m, n, ib, dp<R>(A), lda, dp<R>(T), ldt, dp<R>(tau), stream, true);          \
  }                                                                                                  \
  int tqr_##P##unmqr(char side, char trans, int m, int n, int k, int ib, const CT *A, int lda,       \
                     const CT *T, int ldt, CT *C, int ldc, CT *work, int ldwork,                     \
                     cudaStream_t stream) {                                                          \
    (void)work; (void)ldwork;                                                                        \
    if (!al<R>(A)) return -7;                                                                        \
    if (!al<R>(T)) return -9;                                                                        \
    if (!al<R>(C)) return -11;                                                                       \
    return unmqr_impl<R>(side, trans, m, n, k, ib, dp<R>(A), lda, dp<R>(T), ldt, dp<R>(C), ldc,      \
                         stream);                                                                    \
  }                                                                                                  \
  int tqr_##P##tsqrt(int m, int n, int ib, int m1, CT *A1, int lda1, CT *A2, int lda2, CT *T,        \
                     int ldt, CT *tau, CT *work, cudaStream_t stream) {                              \
    (void)work;                                                                                      \
    if (!al<R>(A1)) return -5;                                                                       \
    if (!al<R>(A2)) return -7;                                                                       \
    if (!al<R>(T)) return -9;                                                                        \
    if (!al<R>(tau)) return -11;                                                                     \
    return tsqrt_impl<R>(m, n, ib, m1, dp<R>(A1), lda1, dp<R>(A2), lda2, dp<R>(T), ldt, dp<R>(tau),  \
                         stream, true);                                                              \
  }                                                                                                  \
  int tqr_##P##tsmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, CT *A1,   \
                     int lda1, CT *A2, int lda2, const CT *V, int ldv, const CT *T, int ldt,         \
                     CT *work, int lwork, cudaStream_t stream) {                                     \
    (void)work; (void)lwork;                                                                         \
    if (!al<R>(A1)) return -9;                                                                       \
    if (!al<R>(A2)) return -11;                                                                      \
    if (!al<R>(V)) return -13;                                                                       \
    if (!al<R>(T)) return -15;                                                                       \
    return tsmqr_impl<R>(side, trans, m1, n1, m2, n2, k, ib, dp<R>(A1), lda1, dp<R>(A2), lda2,       \
                         dp<R>(V), ldv, dp<R>(T), ldt, stream);                                      \
  }                                                                                                  \
  int tqr_##P##ttqrt(int m, int n, int ib, CT *A1, int lda1, CT *A2, int lda2, CT *T, int ldt,       \
                     CT *tau, CT *work, cudaStream_t stream) {                                       \
    (void)work;                                                                                      \
    if (!al<R>(A1)) return -4;                                                                       \
    if (!al<R>(A2)) return -6;                                                                       \
    if (!al<R>(T)) return -8;                                                                        \
    if (!al<R>(tau)) return -10;                                                                     \
    return ttqrt_impl<R>(m, n, ib, dp<R>(A1), lda1, dp<R>(A2), lda2, dp<R>(T), ldt, dp<R>(tau),      \
                         stream);                                                                    \
  }                                                                                                  \
  int tqr_##P##ttmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, CT *A1,   \
                     int lda1, CT *A2, int lda2, const CT *V, int ldv, const CT *T, int ldt,         \
                     CT *work, int lwork, cudaStream_t stream) {                                     \
    (void)work; (void)lwork;                                                                         \
    if (!al<R>(A1)) return -9;                                                                       \
    if (!al<R>(A2)) return -11;                                                                      \
    if (!al<R>(V)) return -13;                                                                       \
    if (!al<R>(T)) return -15;                                                                       \
    return ttmqr_impl<R>(side, trans, m1, n1, m2, n2, k, ib, dp<R>(A1), lda1, dp<R>(A2), lda2,       \
                         dp<R>(V), ldv, dp<R>(T), ldt, stream);                                      \
  }                                                                                                  \
  int tqr_##P##parfb(char side, char trans, char direct, char storev, int m1, int n1, int m2,        \
                     int n2, int k, int l, CT *A1, int lda1, CT *A2, int lda2, const CT *V,          \
                     int ldv, const CT *T, int ldt, CT *work, int ldwork, cudaStream_t stream) {     \
    if (!al<R>(A1)) return -11;                                                                      \
    if (!al<R>(A2)) return -13;                                                                      \
    if (!al<R>(V)) return -15;                                                                       \
    if (!al<R>(T)) return -17;                                                                       \
    if (!al<R>(work)) return -19;                                                                    \
    return parfb_impl<R>(side, trans, direct, storev, m1, n1, m2, n2, k, l, dp<R>(A1), lda1,         \
                         dp<R>(A2), lda2, dp<R>(V), ldv, dp<R>(T), ldt, dp<R>(work), ldwork, stream); \
  }

TQR_INSTANTIATE(d, double, double)
TQR_INSTANTIATE(s, float, float)
TQR_INSTANTIATE(z, tqr_zcomplex, cx<double>)
TQR_INSTANTIATE(c, tqr_ccomplex, cx<float>)

#undef TQR_INSTANTIATE

}  // extern "C"
