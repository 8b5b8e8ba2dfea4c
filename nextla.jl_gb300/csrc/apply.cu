// apply.cu -- stand-alone block-reflector apply kernel (larfb / unmqr / tsmqr /
// parfb) and its launcher.  One CTA per NW-wide strip of columns (rows for
// side R); strips never interact, so a call needs no global scratch.  The
// per-strip algorithm is apply_strip (apply_dev.cuh).
#include "apply_dev.cuh"
#include "tileqr_internal.h"

namespace tqr {

template <typename R, int NW>
__global__ void __launch_bounds__(TQR_THREADS)
k_apply(const ApplyArgs<R> a)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  apply_strip<R, NW>(a, blockIdx.x * NW, smem_raw);
}

// Fewest CTAs a stand-alone apply should run on before narrower strips are used.
constexpr int kMinStripCtas = 32;

template <typename R>
ApplyArgs<R> make_apply_args(int mode, char side, char trans, int m, int n, int k, int ib, R *C,
                             int ldc, R *A1, int lda1, const R *V, int ldv, const R *T, int ldt,
                             size_t *smem_bytes)
{
  ApplyArgs<R> a;
  const bool left = (side == 'L');
  a.mode = mode;
  a.k = k;
  a.ib = ib;
  a.fwd = (left && trans != 'N') || (!left && trans == 'N');
  a.transT = left ? (trans != 'N') : (trans == 'N');
  a.conj_c = is_cx<R> && !left;      // right side: the view is C^H
  a.C = C;
  a.A1 = A1;
  a.V = V; a.ldv = ldv;
  a.T = T; a.ldt = ldt;
  if (left) { a.L = m; a.ncols = n; a.c_rs = 1; a.c_cs = ldc; a.a_rs = 1; a.a_cs = lda1; }
  else      { a.L = n; a.ncols = m; a.c_rs = ldc; a.c_cs = 1; a.a_rs = lda1; a.a_cs = 1; }
  // Strip width and staging: prefer everything in shared memory with two
  // CTAs per SM and 16-wide strips, then narrower strips, then one CTA per SM,
  // then V and C read from global.
  const size_t cap = (size_t)TQR_SMEM_MAX;
  const size_t half = cap / 2 - 1024;
  bool sc = true, sv = true, stt = (ib <= 64);
  auto bytes = [&](int w) { return apply_smem_elems(a.L, ib, w, sc, sv, stt) * sizeof(R); };
  int nw = 16;
  if (bytes(16) > half) {
    if (bytes(8) <= half) nw = 8;
    else if (bytes(16) <= cap) nw = 16;
    else if (bytes(8) <= cap) nw = 8;
  }
  if (bytes(nw) > cap) sv = false;
  if (bytes(nw) > cap) sc = false;
  while (bytes(nw) > cap && nw > 1) nw = (nw == 16) ? 8 : (nw == 8 ? 4 : 1);
  // A narrow operand (a few right-hand sides) would leave all but a CTA or
  // two idle, each CTA working through every block at one SM's FP64 rate:
  // narrower strips spread it over more SMs.  The per-column arithmetic does
  // not depend on the strip width, so results are unchanged bit for bit.
  while (nw > 1 && (a.ncols + nw - 1) / nw < kMinStripCtas) nw = (nw == 16) ? 8 : (nw == 8 ? 4 : 1);
  a.nw = nw;
  a.stage_c = sc; a.stage_v = sv; a.stage_t = stt;
  *smem_bytes = bytes(nw);
  return a;
}

template <typename R, int NW>
static cudaError_t launch_nw(const ApplyArgs<R> &a, size_t sm, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_apply<R, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)TQR_SMEM_MAX);
  if (e != cudaSuccess) return e;
  const int grid = (a.ncols + NW - 1) / NW;
  k_apply<R, NW><<<grid, TQR_THREADS, sm, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

// side: 'L' or 'R'; trans: 'N' or not.  For mode 0, C is the m-by-n matrix the
// reflectors of V (rows = order of Q) act on; for mode 1, C is A2 and A1 is
// the separate triangular/rectangular part.
template <typename R>
cudaError_t launch_apply(int mode, char side, char trans, int m, int n, int k, int ib,
                         R *C, int ldc, R *A1, int lda1, const R *V, int ldv,
                         const R *T, int ldt, cudaStream_t st, int tt)
{
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  size_t sm = 0;
  ApplyArgs<R> a = make_apply_args<R>(mode, side, trans, m, n, k, ib, C, ldc, A1, lda1, V, ldv, T,
                                      ldt, &sm);
  a.tt = (mode == 1) ? tt : -1;
  if (sm > (size_t)TQR_SMEM_MAX) return cudaErrorInvalidValue;
  switch (a.nw) {
    case 16: return launch_nw<R, 16>(a, sm, st);
    case 8: return launch_nw<R, 8>(a, sm, st);
    case 4: return launch_nw<R, 4>(a, sm, st);
    default: return launch_nw<R, 1>(a, sm, st);
  }
}

template cudaError_t launch_apply<double>(int, char, char, int, int, int, int, double *, int, double *, int,
                                          const double *, int, const double *, int, cudaStream_t, int);
template cudaError_t launch_apply<float>(int, char, char, int, int, int, int, float *, int, float *, int,
                                         const float *, int, const float *, int, cudaStream_t, int);
template cudaError_t launch_apply<cx<double>>(int, char, char, int, int, int, int, cx<double> *, int, cx<double> *,
                                              int, const cx<double> *, int, const cx<double> *, int, cudaStream_t, int);
template cudaError_t launch_apply<cx<float>>(int, char, char, int, int, int, int, cx<float> *, int, cx<float> *, int,
                                             const cx<float> *, int, const cx<float> *, int, cudaStream_t, int);

}  // namespace tqr
