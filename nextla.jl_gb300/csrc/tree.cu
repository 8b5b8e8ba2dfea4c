// tree.cu -- tile QR with a binary reduction tree per panel, built from
// geqrt!/unmqr! on every tile and ttqrt!/ttmqr! between tile pairs
// (src/geqrt.jl:22-68, src/unmqr.jl:52-149, src/ttqrt.jl:81-119,
// src/ttmqr.jl:1-95).
//
// For panel k the flat tree chains MT - k tsqrt! calls; here every tile of the
// panel is factored at once (geqrt!), then pairs at distance s = 1, 2, 4, ...
// are merged by ttqrt!, so the serial chain per panel is 1 + ceil(log2(MT - k))
// tile steps.  A last row tile with fewer rows than the panel has columns
// would become a wide trapezoid that ttqrt! (min(m, n) reflectors) cannot
// reduce; it is merged whole into the tile above it by tsqrt!/tsmqr! first.
//
// Storage: A in place; tile (i,k) keeps geqrt's V below its diagonal with T_ik
// in T (rows i*ib, columns k*nb; NextLA's ib x nb layout per tile) and tau in
// tau[(k*nb + c) + i*ldtau]; for i > k, the merge reflectors (ttqrt's in its
// upper triangle, or tsqrt's in the whole tile for the ragged merge) with T2,
// tau2 in the same layouts.  Optional right-hand sides B (m x nrhs) receive
// Q^T B along the way.
//
// Each tile-level step is split the way the persistent kernel splits it: an
// ib-block panel (one CTA per tile or pair) and strip applies (one CTA per
// 16-column strip), each a launch over all tiles or pairs of the step.
#include <algorithm>
#include <vector>

#include "apply_dev.cuh"
#include "panel_dev.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

constexpr int kTreeNW = 16;
constexpr size_t kTreeSmem = 110976;

template <typename R>
struct TreeGeom {
  int m, n, nb, ib, MT, NT, KT, nrhs;
  R *A; int lda;
  R *B; int ldb;
  R *T, *T2; int ldt;
  R *tau, *tau2; int ldtau;
  __host__ __device__ int rows(int i) const { return min(nb, m - i * nb); }
  __host__ __device__ int cols(int k) const { return min(nb, n - k * nb); }
  __host__ __device__ R *tile(int i, int j) const { return A + (size_t)j * nb * lda + (size_t)i * nb; }
  __host__ __device__ R *ttile(R *base, int i, int k) const { return base + (size_t)k * nb * ldt + (size_t)i * ib; }
  __host__ __device__ R *tautile(R *base, int i, int k) const { return base + (size_t)i * ldtau + (size_t)k * nb; }
};

enum TreeOpType { OP_GE_PANEL = 0, OP_GE_APPLY = 1, OP_GE_TRAIL = 2, OP_PR_PANEL = 3, OP_PR_APPLY = 4,
                  OP_PR_TRAIL = 5 };

struct TreeOp {
  int type;
  int k, b;            // panel, ib-block
  int i0, istep;       // task t: top tile i = i0 + t * istep
  int s;               // pair partner p = i + s (pair ops)
  int ts;              // pair ops: 1 = tsqrt/tsmqr merge of a whole tile, 0 = ttqrt/ttmqr
  int trans;           // trailing ops: 0 applies Q^T (factorisation), 1 applies Q
  int a_cols;          // trailing ops: 1 = include A's trailing columns
};

// Trailing region of tile row i for a trailing op: strip y of (A columns
// right of panel k, then B's columns).  Returns false if y is past the end.
template <typename R>
__device__ bool trail_region(const TreeGeom<R> &g, const TreeOp &op, int i, int y, R *&C, int &ld, int &ncols,
                             int &c0) {
  const int ca = op.a_cols ? max(0, g.n - (op.k + 1) * g.nb) : 0;
  const int sa = (ca + kTreeNW - 1) / kTreeNW;
  if (y < sa) {
    C = g.tile(i, op.k + 1); ld = g.lda; ncols = ca; c0 = y * kTreeNW;
    return true;
  }
  y -= sa;
  const int sbn = (g.nrhs + kTreeNW - 1) / kTreeNW;
  if (y < sbn) {
    C = g.B + (size_t)i * g.nb; ld = g.ldb; ncols = g.nrhs; c0 = y * kTreeNW;
    return true;
  }
  return false;
}

template <typename R>
__device__ ApplyArgs<R> tree_args(int mode, int L, int k, int ib, int trans) {
  ApplyArgs<R> a;
  a.mode = mode; a.L = L; a.k = k; a.ib = ib;
  a.fwd = trans ? 0 : 1; a.transT = trans ? 0 : 1;
  a.c_rs = 1; a.a_rs = 1; a.a_cs = 1; a.A1 = nullptr;
  a.nw = kTreeNW;
  a.stage_c = 1; a.stage_v = 1; a.stage_t = 1;
  return a;
}

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS, 2) k_tree(const TreeGeom<R> g, const TreeOp op) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int t = blockIdx.x, y = blockIdx.y;
  const int k = op.k, ib = g.ib, nk = g.cols(k);
  const int i = op.i0 + t * op.istep;
  const int mi = g.rows(i);
  R *Aik = g.tile(i, k);
  switch (op.type) {
    case OP_GE_PANEL: {
      const int kk = min(mi, nk), c = op.b * ib;
      if (c >= kk) return;
      const int sb = min(ib, kk - c);
      panel_qr_cta<R>(mi - c, sb, Aik + ix(c, c, g.lda), g.lda, g.tautile(g.tau, i, k) + c,
                      g.ttile(g.T, i, k) + ix(0, c, g.ldt), g.ldt, true, true, smem);
      return;
    }
    case OP_GE_APPLY: {
      const int kk = min(mi, nk), c = op.b * ib;
      if (c >= kk) return;
      const int sb = min(ib, kk - c);
      const int c0 = c + sb + y * kTreeNW;
      if (c0 >= nk) return;
      ApplyArgs<R> a = tree_args<R>(0, mi - c, sb, sb, 0);
      a.C = Aik + c; a.c_cs = g.lda; a.ncols = nk;
      a.V = Aik + ix(c, c, g.lda); a.ldv = g.lda;
      a.T = g.ttile(g.T, i, k) + ix(0, c, g.ldt); a.ldt = g.ldt;
      apply_strip<R, kTreeNW>(a, c0, smem);
      return;
    }
    case OP_GE_TRAIL: {
      R *C; int ld, ncols, c0;
      if (!trail_region(g, op, i, y, C, ld, ncols, c0)) return;
      ApplyArgs<R> a = tree_args<R>(0, mi, min(mi, nk), ib, op.trans);
      a.C = C; a.c_cs = ld; a.ncols = ncols;
      a.V = Aik; a.ldv = g.lda;
      a.T = g.ttile(g.T, i, k); a.ldt = g.ldt;
      apply_strip<R, kTreeNW>(a, c0, smem);
      return;
    }
    default:
      break;
  }
  // pair ops: top tile i, partner p
  const int p = i + op.s, mp = g.rows(p);
  R *Apk = g.tile(p, k);
  const int kt = op.ts ? nk : min(mp, nk);     // merge reflectors
  switch (op.type) {
    case OP_PR_PANEL: {
      const int c = op.b * ib;
      if (c >= kt) return;
      const int sb = min(ib, kt - c);
      tsqrt_block_cta<R>(mp, sb, Aik + ix(c, c, g.lda), g.lda, Apk + ix(0, c, g.lda), g.lda,
                         g.ttile(g.T2, p, k) + ix(0, c, g.ldt), g.ldt, g.tautile(g.tau2, p, k) + c, true, smem,
                         op.ts ? -1 : c);
      return;
    }
    case OP_PR_APPLY: {
      const int c = op.b * ib;
      if (c >= kt) return;
      const int sb = min(ib, kt - c);
      const int c0 = c + sb + y * kTreeNW;
      if (c0 >= nk) return;
      const int L = op.ts ? mp : min(mp, c + sb);
      ApplyArgs<R> a = tree_args<R>(1, L, sb, sb, 0);
      a.C = Apk; a.c_cs = g.lda; a.ncols = nk;
      a.A1 = Aik + c; a.a_cs = g.lda;
      a.V = Apk + ix(0, c, g.lda); a.ldv = g.lda;
      a.T = g.ttile(g.T2, p, k) + ix(0, c, g.ldt); a.ldt = g.ldt;
      a.tt = op.ts ? -1 : c;
      apply_strip<R, kTreeNW>(a, c0, smem);
      return;
    }
    case OP_PR_TRAIL: {
      R *C; int ld, ncols, c0;
      if (!trail_region(g, op, p, y, C, ld, ncols, c0)) return;
      R *C1; int ld1, n1, c01;
      trail_region(g, op, i, y, C1, ld1, n1, c01);
      ApplyArgs<R> a = tree_args<R>(1, mp, kt, ib, op.trans);
      a.C = C; a.c_cs = ld; a.ncols = ncols;
      a.A1 = C1; a.a_cs = ld1;
      a.V = Apk; a.ldv = g.lda;
      a.T = g.ttile(g.T2, p, k); a.ldt = g.ldt;
      a.tt = op.ts ? -1 : 0;
      apply_strip<R, kTreeNW>(a, c0, smem);
      return;
    }
    default:
      return;
  }
}

template <typename R>
static cudaError_t tree_launch(const TreeGeom<R> &g, const TreeOp &op, int ntask, int ny, cudaStream_t st) {
  if (ntask <= 0 || ny <= 0) return cudaSuccess;
  k_tree<R><<<dim3(ntask, ny), TQR_THREADS, kTreeSmem, st>>>(g, op);
  count_launch();
  return cudaGetLastError();
}

template <typename R>
static int trail_strips(const TreeGeom<R> &g, int k, int a_cols) {
  const int ca = a_cols ? std::max(0, g.n - (k + 1) * g.nb) : 0;
  return (ca + kTreeNW - 1) / kTreeNW + (g.nrhs + kTreeNW - 1) / kTreeNW;
}

template <typename R>
static bool tree_ragged(const TreeGeom<R> &g, int k) {
  const int p = g.MT - 1;
  return p > k && g.rows(p) < g.cols(k);
}

// Merges of panel k at distance s among tiles [k, MTt): (first top tile,
// count).
static int tree_pairs(int k, int MTt, int s) {
  int c = 0;
  for (int i = k; i + s < MTt; i += 2 * s) ++c;
  return c;
}

template <typename R>
static cudaError_t tree_factor(const TreeGeom<R> &g, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_tree<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTreeSmem);
  if (e != cudaSuccess) return e;
  const int ib = g.ib;
  for (int k = 0; k < g.KT; ++k) {
    const int nk = g.cols(k);
    const bool rag = tree_ragged(g, k);
    const int MTt = rag ? g.MT - 1 : g.MT;
    const int nblk = (nk + ib - 1) / ib;
    const int ntile = MTt - k;
    TreeOp op{};
    op.k = k; op.i0 = k; op.istep = 1; op.a_cols = 1;
    for (int b = 0; b < nblk; ++b) {
      op.b = b;
      op.type = OP_GE_PANEL;
      if ((e = tree_launch(g, op, ntile, 1, st)) != cudaSuccess) return e;
      const int rest = nk - std::min(nk, (b + 1) * ib);
      op.type = OP_GE_APPLY;
      if ((e = tree_launch(g, op, ntile, (rest + kTreeNW - 1) / kTreeNW, st)) != cudaSuccess) return e;
    }
    op.type = OP_GE_TRAIL; op.trans = 0;
    if ((e = tree_launch(g, op, ntile, trail_strips(g, k, 1), st)) != cudaSuccess) return e;
    auto merge = [&](int i0, int s, int npair, int ts) -> cudaError_t {
      TreeOp q{};
      q.k = k; q.i0 = i0; q.istep = 2 * s; q.s = s; q.ts = ts; q.a_cols = 1;
      const int kt = ts ? nk : std::min(g.rows(i0 + s), nk);
      const int nb2 = (kt + ib - 1) / ib;
      cudaError_t e2;
      for (int b = 0; b < nb2; ++b) {
        q.b = b;
        q.type = OP_PR_PANEL;
        if ((e2 = tree_launch(g, q, npair, 1, st)) != cudaSuccess) return e2;
        const int rest = nk - std::min(nk, std::min(kt, (b + 1) * ib));
        q.type = OP_PR_APPLY;
        if ((e2 = tree_launch(g, q, npair, (rest + kTreeNW - 1) / kTreeNW, st)) != cudaSuccess) return e2;
      }
      q.type = OP_PR_TRAIL; q.trans = 0;
      return tree_launch(g, q, npair, trail_strips(g, k, 1), st);
    };
    if (rag && (e = merge(g.MT - 2, 1, 1, 1)) != cudaSuccess) return e;
    for (int s = 1; k + s < MTt; s *= 2)
      if ((e = merge(k, s, tree_pairs(k, MTt, s), 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// B := Q^T B (trans 0) or Q B (trans 1) through the stored tree factors.
template <typename R>
static cudaError_t tree_apply_q(const TreeGeom<R> &g, int trans, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_tree<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTreeSmem);
  if (e != cudaSuccess) return e;
  const int ny = (g.nrhs + kTreeNW - 1) / kTreeNW;
  for (int kx = 0; kx < g.KT; ++kx) {
    const int k = trans ? g.KT - 1 - kx : kx;
    const bool rag = tree_ragged(g, k);
    const int MTt = rag ? g.MT - 1 : g.MT;
    TreeOp ge{};
    ge.type = OP_GE_TRAIL; ge.k = k; ge.i0 = k; ge.istep = 1; ge.trans = trans; ge.a_cols = 0;
    auto pair = [&](int i0, int s, int npair, int ts) {
      TreeOp q{};
      q.type = OP_PR_TRAIL; q.k = k; q.i0 = i0; q.istep = 2 * s; q.s = s; q.ts = ts; q.trans = trans;
      q.a_cols = 0;
      return tree_launch(g, q, npair, ny, st);
    };
    if (!trans) {
      if ((e = tree_launch(g, ge, MTt - k, ny, st)) != cudaSuccess) return e;
      if (rag && (e = pair(g.MT - 2, 1, 1, 1)) != cudaSuccess) return e;
      for (int s = 1; k + s < MTt; s *= 2)
        if ((e = pair(k, s, tree_pairs(k, MTt, s), 0)) != cudaSuccess) return e;
    } else {
      int smax = 1;
      while (k + smax < MTt) smax *= 2;
      for (int s = smax / 2; s >= 1; s /= 2)
        if ((e = pair(k, s, tree_pairs(k, MTt, s), 0)) != cudaSuccess) return e;
      if (rag && (e = pair(g.MT - 2, 1, 1, 1)) != cudaSuccess) return e;
      if ((e = tree_launch(g, ge, MTt - k, ny, st)) != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template <typename R>
static int tree_geom(int m, int n, int nrhs, int nb, int ib, R *A, int lda, R *B, int ldb, R *T, R *T2, int ldt,
                     R *tau, R *tau2, int ldtau, TreeGeom<R> *g) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (nb <= 0 || nb > 256) return -3;
  if (ib <= 0 || ib > nb || ib > 32) return -4;
  g->m = m; g->n = n; g->nb = nb; g->ib = ib; g->nrhs = nrhs;
  g->MT = (m + nb - 1) / nb; g->NT = (n + nb - 1) / nb; g->KT = std::min(g->MT, g->NT);
  g->A = A; g->lda = lda; g->B = B; g->ldb = ldb;
  g->T = T; g->T2 = T2; g->ldt = ldt;
  g->tau = tau; g->tau2 = tau2; g->ldtau = ldtau;
  return 0;
}

template <typename R>
static int tree_geqrf_impl(int m, int n, int nb, int ib, R *A, int lda, R *T, R *T2, int ldt, R *tau, R *tau2,
                           int ldtau, int nrhs, R *B, int ldb, cudaStream_t st) {
  TreeGeom<R> g;
  int rc = tree_geom<R>(m, n, nrhs, nb, ib, A, lda, B, ldb, T, T2, ldt, tau, tau2, ldtau, &g);
  if (rc) return rc;
  if (m == 0 || n == 0) return 0;
  if (!A || lda < m) return -6;
  if (!T || !T2 || ldt < g.MT * ib) return -9;
  if (!tau || !tau2 || ldtau < n) return -12;
  if (nrhs < 0) return -13;
  if (nrhs > 0 && (!B || ldb < m)) return -15;
  // skipped reflectors leave their T columns untouched: start from zero
  cudaError_t e = cudaMemset2DAsync(T2, sizeof(R) * ldt, 0, sizeof(R) * g.MT * ib, n, st);
  if (e == cudaSuccess) e = tree_factor(g, st);
  return e == cudaSuccess ? 0 : (int)e;
}

template <typename R>
static int tree_unmqr_impl(char trans, int m, int n, int nrhs, int nb, int ib, const R *A, int lda, const R *T,
                           const R *T2, int ldt, R *B, int ldb, cudaStream_t st) {
  if (trans != 'N' && trans != 'C' && trans != 'T') return -1;
  TreeGeom<R> g;
  int rc = tree_geom<R>(m, n, nrhs, nb, ib, const_cast<R *>(A), lda, B, ldb, const_cast<R *>(T),
                        const_cast<R *>(T2), ldt, nullptr, nullptr, 1, &g);
  if (rc) return rc == -1 ? -2 : rc == -2 ? -3 : rc == -3 ? -5 : -6;
  if (nrhs < 0) return -4;
  if (m == 0 || n == 0 || nrhs == 0) return 0;
  if (!A || lda < m) return -8;
  if (!T || !T2 || ldt < g.MT * ib) return -11;
  if (!B || ldb < m) return -13;
  cudaError_t e = tree_apply_q(g, trans == 'N' ? 1 : 0, st);
  return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace tqr

using namespace tqr;

extern "C" {

int tqr_dtile_geqrf_tree(int m, int n, int nb, int ib, double *A, int lda, double *T, double *T2, int ldt,
                         double *tau, double *tau2, int ldtau, int nrhs, double *B, int ldb, cudaStream_t stream) {
  return tree_geqrf_impl<double>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, stream);
}

int tqr_stile_geqrf_tree(int m, int n, int nb, int ib, float *A, int lda, float *T, float *T2, int ldt,
                         float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb, cudaStream_t stream) {
  return tree_geqrf_impl<float>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, stream);
}

int tqr_dtile_unmqr_tree(char trans, int m, int n, int nrhs, int nb, int ib, const double *A, int lda,
                         const double *T, const double *T2, int ldt, double *B, int ldb, cudaStream_t stream) {
  return tree_unmqr_impl<double>(trans, m, n, nrhs, nb, ib, A, lda, T, T2, ldt, B, ldb, stream);
}

int tqr_stile_unmqr_tree(char trans, int m, int n, int nrhs, int nb, int ib, const float *A, int lda,
                         const float *T, const float *T2, int ldt, float *B, int ldb, cudaStream_t stream) {
  return tree_unmqr_impl<float>(trans, m, n, nrhs, nb, ib, A, lda, T, T2, ldt, B, ldb, stream);
}

}  // extern "C"
