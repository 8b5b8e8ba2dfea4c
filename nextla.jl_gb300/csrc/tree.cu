// tree.cu -- tile QR with a binary reduction tree per panel, built from
// geqrt!/unmqr! on every tile and ttqrt!/ttmqr! between tile pairs
// (src/geqrt.jl:22-68, src/unmqr.jl:52-149, src/ttqrt.jl:81-119,
// src/ttmqr.jl:1-95).
//
// For panel k the flat tree chains MT - k tsqrt! calls; here every tile of the
// panel is factored at once (geqrt!), then pairs at distance s = 1, 2, 4, ...
// are merged by ttqrt!, so the serial chain per panel is 1 + ceil(log2(MT - k))
// tile steps.  The hierarchical form (group size grp > 1, PLASMA's HQR) first
// reduces groups of grp consecutive tiles flat into their first tile (geqrt!
// on that leader, tsqrt!/tsmqr! of each other tile into it -- the flat tree's
// arithmetic), then the leaders by the binary tree at distances grp, 2 grp,
// ...: a chain of grp + log2 of the leader count per panel with the flat
// tree's update flops inside the groups.  A last row tile with fewer rows than the panel has columns
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
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "apply_dev.cuh"
#include "panel_dev.cuh"
#include "tc_wy.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

constexpr int kTreeNW = 16;
constexpr size_t kTreeSmem = 110976;
// Strip width per element type: 16 columns for the 8-byte and smaller
// elements, 8 for ComplexF64, whose 16-byte elements would not fit a strip
// with its V block in one CTA's shared memory otherwise.
template <typename R> struct TreeNW { static constexpr int value = kTreeNW; };
template <> struct TreeNW<cx<double>> { static constexpr int value = 8; };

// Dynamic shared memory of the tree kernels for element type R: the panel
// block, the tsqrt block and a staged strip apply at nb = 256, ib = 32
// (kTreeSmem for the real types; ComplexF64 takes one CTA per SM).
template <typename R>
static size_t tree_smem() {
  return std::max({kTreeSmem, apply_smem_elems(256, 32, TreeNW<R>::value, true, true, true) * sizeof(R),
                   panel_smem<R>(256, 32, true, true), tsqrt_smem<R>(256, 32, true)});
}

template <typename R>
struct TreeGeom {
  int m, n, nb, ib, MT, NT, KT, nrhs;
  int grp;           // tiles per flat group (1: the binary tree)
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
                  OP_PR_TRAIL = 5,
                  // task graph only, FP32, on the tensor cores, one 128-column
                  // chunk of A per task: the trailing update of a merge
                  // (tsmqr! for a tsqrt merge, ttmqr! for a ttqrt merge) and
                  // of a geqrt! (unmqr!)
                  OP_PR_TRAIL_TC = 6, OP_GE_TRAIL_TC = 7,
                  // compact-WY form of the two above (tc_wy.cuh): once per
                  // reflector tile, the stage images every chunk of its
                  // update shares (a "slot"); the chunk tasks then read it
                  OP_WY_BUILD = 8 };

// Slot of the compact-WY images of a reflector tile: geqrt!'s V of tile
// (row, k) (merge 0) or a merge's V in tile (row, k) (merge 1), two per tile
// row and kind, alternating with k.  A slot is rebuilt only after every chunk
// that read it two panels earlier (the graph builder tracks each slot as a
// region).
__host__ __device__ inline int wy_slot(int MT, int merge, int row, int k) { return ((merge * MT) + row) * 2 + (k & 1); }

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
  const int sa = (ca + TreeNW<R>::value - 1) / TreeNW<R>::value;
  if (y < sa) {
    C = g.tile(i, op.k + 1); ld = g.lda; ncols = ca; c0 = y * TreeNW<R>::value;
    return true;
  }
  y -= sa;
  const int sbn = (g.nrhs + TreeNW<R>::value - 1) / TreeNW<R>::value;
  if (y < sbn) {
    C = g.B + (size_t)i * g.nb; ld = g.ldb; ncols = g.nrhs; c0 = y * TreeNW<R>::value;
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
  a.nw = TreeNW<R>::value;
  a.stage_c = 1; a.stage_v = 1; a.stage_t = 1;
  return a;
}

// One step of the tree factorisation on top tile i (and partner i + op.s for
// the pair ops), strip y; shared by the stream driver and the persistent
// task-graph kernel.
template <typename R>
__device__ void tree_task(const TreeGeom<R> &g, const TreeOp &op, int i, int y, unsigned char *smem) {
  const int k = op.k, ib = g.ib, nk = g.cols(k);
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
      const int c0 = c + sb + y * TreeNW<R>::value;
      if (c0 >= nk) return;
      ApplyArgs<R> a = tree_args<R>(0, mi - c, sb, sb, 0);
      a.C = Aik + c; a.c_cs = g.lda; a.ncols = nk;
      a.V = Aik + ix(c, c, g.lda); a.ldv = g.lda;
      a.T = g.ttile(g.T, i, k) + ix(0, c, g.ldt); a.ldt = g.ldt;
      apply_strip<R, TreeNW<R>::value>(a, c0, smem);
      return;
    }
    case OP_GE_TRAIL: {
      R *C; int ld, ncols, c0;
      if (!trail_region(g, op, i, y, C, ld, ncols, c0)) return;
      ApplyArgs<R> a = tree_args<R>(0, mi, min(mi, nk), ib, op.trans);
      a.C = C; a.c_cs = ld; a.ncols = ncols;
      a.V = Aik; a.ldv = g.lda;
      a.T = g.ttile(g.T, i, k); a.ldt = g.ldt;
      apply_strip<R, TreeNW<R>::value>(a, c0, smem);
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
      const int c0 = c + sb + y * TreeNW<R>::value;
      if (c0 >= nk) return;
      const int L = op.ts ? mp : min(mp, c + sb);
      ApplyArgs<R> a = tree_args<R>(1, L, sb, sb, 0);
      a.C = Apk; a.c_cs = g.lda; a.ncols = nk;
      a.A1 = Aik + c; a.a_cs = g.lda;
      a.V = Apk + ix(0, c, g.lda); a.ldv = g.lda;
      a.T = g.ttile(g.T2, p, k) + ix(0, c, g.ldt); a.ldt = g.ldt;
      a.tt = op.ts ? -1 : c;
      apply_strip<R, TreeNW<R>::value>(a, c0, smem);
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
      apply_strip<R, TreeNW<R>::value>(a, c0, smem);
      return;
    }
    default:
      return;
  }
}

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS, 2) k_tree(const TreeGeom<R> g, const TreeOp op) {
  extern __shared__ __align__(16) unsigned char smem[];
  tree_task<R>(g, op, op.i0 + blockIdx.x * op.istep, blockIdx.y, smem);
}

template <typename R>
static cudaError_t tree_launch(const TreeGeom<R> &g, const TreeOp &op, int ntask, int ny, cudaStream_t st) {
  if (ntask <= 0 || ny <= 0) return cudaSuccess;
  k_tree<R><<<dim3(ntask, ny), TQR_THREADS, tree_smem<R>(), st>>>(g, op);
  count_launch();
  return cudaGetLastError();
}

template <typename R>
static int trail_strips(const TreeGeom<R> &g, int k, int a_cols) {
  constexpr int nw = TreeNW<R>::value;
  const int ca = a_cols ? std::max(0, g.n - (k + 1) * g.nb) : 0;
  return (ca + nw - 1) / nw + (g.nrhs + nw - 1) / nw;
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

// Leaders of panel k: tiles k, k + grp, ... below MTt; the last one takes
// the ragged tile.
static inline int tree_nlead(int k, int MTt, int grp) { return (MTt - k + grp - 1) / grp; }

template <typename R>
static cudaError_t tree_factor(const TreeGeom<R> &g, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_tree<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tree_smem<R>());
  if (e != cudaSuccess) return e;
  constexpr int nw = TreeNW<R>::value;
  const int ib = g.ib, G = g.grp;
  for (int k = 0; k < g.KT; ++k) {
    const int nk = g.cols(k);
    const bool rag = tree_ragged(g, k);
    const int MTt = rag ? g.MT - 1 : g.MT;
    const int nblk = (nk + ib - 1) / ib;
    const int nlead = tree_nlead(k, MTt, G);
    const int last = k + (nlead - 1) * G;
    TreeOp op{};
    op.k = k; op.i0 = k; op.istep = G; op.a_cols = 1;
    // reflectors of the shortest leader: its blocks end earliest, so its
    // strips reach furthest left (the other tiles skip the strips they do not need)
    const int kkmin = std::min(g.rows(last), nk);
    for (int b = 0; b < nblk; ++b) {
      op.b = b;
      op.type = OP_GE_PANEL;
      if ((e = tree_launch(g, op, nlead, 1, st)) != cudaSuccess) return e;
      const int rest = nk - std::min(nk, std::min(kkmin, (b + 1) * ib));
      op.type = OP_GE_APPLY;
      if ((e = tree_launch(g, op, nlead, (rest + nw - 1) / nw, st)) != cudaSuccess) return e;
    }
    op.type = OP_GE_TRAIL; op.trans = 0;
    if ((e = tree_launch(g, op, nlead, trail_strips(g, k, 1), st)) != cudaSuccess) return e;
    auto merge = [&](int i0, int s, int istep, int npair, int ts) -> cudaError_t {
      TreeOp q{};
      q.k = k; q.i0 = i0; q.istep = istep; q.s = s; q.ts = ts; q.a_cols = 1;
      const int kt = ts ? nk : std::min(g.rows(i0 + s), nk);
      const int nb2 = (kt + ib - 1) / ib;
      cudaError_t e2;
      for (int b = 0; b < nb2; ++b) {
        q.b = b;
        q.type = OP_PR_PANEL;
        if ((e2 = tree_launch(g, q, npair, 1, st)) != cudaSuccess) return e2;
        const int rest = nk - std::min(nk, std::min(kt, (b + 1) * ib));
        q.type = OP_PR_APPLY;
        if ((e2 = tree_launch(g, q, npair, (rest + nw - 1) / nw, st)) != cudaSuccess) return e2;
      }
      q.type = OP_PR_TRAIL; q.trans = 0;
      return tree_launch(g, q, npair, trail_strips(g, k, 1), st);
    };
    // flat reduction inside the groups (tile i + d into leader i), then the
    // ragged tile into the last leader
    for (int d = 1; d < G; ++d) {
      const int npair = (MTt - 1 - d - k) >= 0 ? (MTt - 1 - d - k) / G + 1 : 0;
      if (npair > 0 && (e = merge(k, d, G, npair, 1)) != cudaSuccess) return e;
    }
    if (rag && (e = merge(last, g.MT - 1 - last, 1, 1, 1)) != cudaSuccess) return e;
    for (int s = G; k + s < MTt; s *= 2)
      if ((e = merge(k, s, 2 * s, tree_pairs(k, MTt, s), 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// B := Q^T B (trans 0) or Q B (trans 1) through the stored tree factors.
template <typename R>
static cudaError_t tree_apply_q(const TreeGeom<R> &g, int trans, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_tree<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tree_smem<R>());
  if (e != cudaSuccess) return e;
  constexpr int nw = TreeNW<R>::value;
  const int ny = (g.nrhs + nw - 1) / nw, G = g.grp;
  for (int kx = 0; kx < g.KT; ++kx) {
    const int k = trans ? g.KT - 1 - kx : kx;
    const bool rag = tree_ragged(g, k);
    const int MTt = rag ? g.MT - 1 : g.MT;
    const int nlead = tree_nlead(k, MTt, G);
    const int last = k + (nlead - 1) * G;
    TreeOp ge{};
    ge.type = OP_GE_TRAIL; ge.k = k; ge.i0 = k; ge.istep = G; ge.trans = trans; ge.a_cols = 0;
    auto pair = [&](int i0, int s, int istep, int npair, int ts) {
      TreeOp q{};
      q.type = OP_PR_TRAIL; q.k = k; q.i0 = i0; q.istep = istep; q.s = s; q.ts = ts; q.trans = trans;
      q.a_cols = 0;
      return tree_launch(g, q, npair, ny, st);
    };
    auto group = [&](int d) {
      const int npair = (MTt - 1 - d - k) >= 0 ? (MTt - 1 - d - k) / G + 1 : 0;
      return npair > 0 ? pair(k, d, G, npair, 1) : cudaSuccess;
    };
    if (!trans) {
      if ((e = tree_launch(g, ge, nlead, ny, st)) != cudaSuccess) return e;
      for (int d = 1; d < G; ++d)
        if ((e = group(d)) != cudaSuccess) return e;
      if (rag && (e = pair(last, g.MT - 1 - last, 1, 1, 1)) != cudaSuccess) return e;
      for (int s = G; k + s < MTt; s *= 2)
        if ((e = pair(k, s, 2 * s, tree_pairs(k, MTt, s), 0)) != cudaSuccess) return e;
    } else {
      int smax = G;
      while (k + smax < MTt) smax *= 2;
      for (int s = smax / 2; s >= G; s /= 2)
        if ((e = pair(k, s, 2 * s, tree_pairs(k, MTt, s), 0)) != cudaSuccess) return e;
      if (rag && (e = pair(last, g.MT - 1 - last, 1, 1, 1)) != cudaSuccess) return e;
      for (int d = G - 1; d >= 1; --d)
        if ((e = group(d)) != cudaSuccess) return e;
      if ((e = tree_launch(g, ge, nlead, ny, st)) != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template <typename R>
static int tree_geom(int m, int n, int nrhs, int nb, int ib, R *A, int lda, R *B, int ldb, R *T, R *T2, int ldt,
                     R *tau, R *tau2, int ldtau, TreeGeom<R> *g, int grp = 1) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (nb <= 0 || nb > 256) return -3;
  if (ib <= 0 || ib > nb || ib > 32) return -4;
  g->m = m; g->n = n; g->nb = nb; g->ib = ib; g->nrhs = nrhs; g->grp = grp;
  g->MT = (m + nb - 1) / nb; g->NT = (n + nb - 1) / nb; g->KT = std::min(g->MT, g->NT);
  g->A = A; g->lda = lda; g->B = B; g->ldb = ldb;
  g->T = T; g->T2 = T2; g->ldt = ldt;
  g->tau = tau; g->tau2 = tau2; g->ldtau = ldtau;
  return 0;
}

template <typename R>
static int tree_geqrf_impl(int m, int n, int nb, int ib, R *A, int lda, R *T, R *T2, int ldt, R *tau, R *tau2,
                           int ldtau, int nrhs, R *B, int ldb, cudaStream_t st, int grp = 1) {
  if (grp <= 0) return -5;
  TreeGeom<R> g;
  int rc = tree_geom<R>(m, n, nrhs, nb, ib, A, lda, B, ldb, T, T2, ldt, tau, tau2, ldtau, &g, grp);
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
                           const R *T2, int ldt, R *B, int ldb, cudaStream_t st, int grp = 1) {
  if (trans != 'N' && trans != 'C' && trans != 'T') return -1;
  if (grp <= 0) return -7;
  TreeGeom<R> g;
  int rc = tree_geom<R>(m, n, nrhs, nb, ib, const_cast<R *>(A), lda, B, ldb, const_cast<R *>(T),
                        const_cast<R *>(T2), ldt, nullptr, nullptr, 1, &g, grp);
  if (rc) return rc == -1 ? -2 : rc == -2 ? -3 : rc == -3 ? -5 : -6;
  if (nrhs < 0) return -4;
  if (m == 0 || n == 0 || nrhs == 0) return 0;
  if (!A || lda < m) return -8;
  if (!T || !T2 || ldt < g.MT * ib) return -11;
  if (!B || ldb < m) return -13;
  cudaError_t e = tree_apply_q(g, trans == 'N' ? 1 : 0, st);
  return e == cudaSuccess ? 0 : (int)e;
}


// ---------------------------------------------------------------------------
// The same factorisation as one persistent launch over a task graph.
//
// Tasks are the steps above cut per tile / pair and per 16-column strip.  The
// host replays the stream driver's order and records, for every task, the
// regions it reads and writes (tile x strip x {upper triangle with diagonal,
// strictly lower part}, and the T blocks); a task depends on the last writer
// of each region it touches and, if it writes, on every reader since that
// writer.  Tasks are sorted by decreasing longest path to the end (a
// topological order); CTAs take them strictly in that order and wait on
// per-task done flags, so the lowest unfinished task always has its inputs
// done.  Every wait is bounded by a %globaltimer deadline that sets an error
// word and ends the launch.  All cross-CTA data is read through L2
// (ld.global.cg in the staged device routines) after an acquire load of the
// flag; writers publish with __syncthreads + __threadfence + a release store.
// ---------------------------------------------------------------------------
static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct TItem {
  uint8_t type;        // TreeOpType, | 0x80 for a tsqrt/tsmqr (whole-tile) merge
  uint8_t b;
  uint16_t k, i, p, y;
  uint16_t ndep;
  uint32_t dep;        // offset of this task's dependency list (task positions)
};
static_assert(sizeof(TItem) == 16, "TItem layout");

struct TDagHeader {
  int head;
  int error;           // 0 ok, 1 a wait timed out, 2 schedule / arguments mismatch
  int err_item;
  int nitems;
  long long key;
  int pad[58];
};
static_assert(sizeof(TDagHeader) == 256, "TDagHeader layout");

template <typename R>
struct TDagArgs {
  TreeGeom<R> g;
  TDagHeader *hdr;
  int *done;
  const TItem *items;
  const uint32_t *deps;
  int nitems;
  long long key;
  unsigned long long timeout_ns;
  // mixed form (FP32 matrix): FP64 diagonal R triangles of the panel steps,
  // ib x nb per (tile row i, panel k) at D + ((k MT + i) nb) ib, ld ib
  double *D = nullptr;
  // tensor-core tasks with tma: tensor maps of A (32 x 128 and 32 x 32
  // boxes); the kernel takes TDagArgs as a __grid_constant__ parameter
  CUtensorMap tmw, tmn;
  int tma = 0;
  // compact-WY chunk tasks (wy): tensor map of A with 16 x 128 boxes in the
  // 64-byte swizzle, and the slots (4 MT of tc::wy::kSlotBytes)
  CUtensorMap tmwy;
  unsigned char *slots = nullptr;
  int wy = 0;
  __device__ unsigned char *slot(int merge, int row, int k) const {
    return slots + (size_t)wy_slot(g.MT, merge, row, k) * tc::wy::kSlotBytes;
  }
  __device__ double *Dtri(int i, int k, int c) const {
    return D + ((size_t)k * g.MT + i) * (size_t)g.nb * g.ib + (size_t)c * g.ib;
  }
};

// Panel steps of the mixed form: geqrt blocks, tsqrt merges (into a group
// leader) and ttqrt merges (of two leaders) in FP64 with the leaders'
// diagonal triangles kept in D (panel_dev.cuh).
__device__ inline void tree_panel_f64(const TDagArgs<float> &a, const TreeOp &op, int i, unsigned char *smem) {
  const TreeGeom<float> &g = a.g;
  const int k = op.k, ib = g.ib, nk = g.cols(k), mi = g.rows(i), c = op.b * ib;
  float *Aik = g.tile(i, k);
  if (op.type == OP_GE_PANEL) {
    const int kk = min(mi, nk);
    if (c >= kk) return;
    const int sb = min(ib, kk - c);
    panel_qr_cta_f64(mi - c, sb, Aik + ix(c, c, g.lda), g.lda, g.tautile(g.tau, i, k) + c,
                     g.ttile(g.T, i, k) + ix(0, c, g.ldt), g.ldt, a.Dtri(i, k, c), ib, smem);
    return;
  }
  const int p = i + op.s, mp = g.rows(p);
  float *Apk = g.tile(p, k);
  const int kt = op.ts ? nk : min(mp, nk);
  if (c >= kt) return;
  const int sb = min(ib, kt - c);
  float *T2b = g.ttile(g.T2, p, k) + ix(0, c, g.ldt), *t2b = g.tautile(g.tau2, p, k) + c;
  if (op.ts)
    tsqrt_block_f64x(mp, sb, a.Dtri(i, k, c), ib, Aik + ix(c, c, g.lda), g.lda, Apk + ix(0, c, g.lda), g.lda, T2b,
                     g.ldt, t2b, smem);
  else
    ttqrt_block_cta_f64(mp, sb, c, a.Dtri(i, k, c), ib, Aik + ix(c, c, g.lda), g.lda, a.Dtri(p, k, c), ib,
                        Apk + ix(0, c, g.lda), g.lda, T2b, g.ldt, t2b, smem);
}

__device__ __forceinline__ int tdag_ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void tdag_st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long tdag_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// TC: this instantiation owns the SM's TMEM and runs the tensor-core chunk
// tasks (FP32, one CTA per SM); the other instantiations never meet one.
template <typename R, bool TC>
__global__ void __launch_bounds__(TQR_THREADS, TC ? 1 : 2) k_tree_dag(const __grid_constant__ TDagArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_it, s_err;
  __shared__ __align__(8) uint64_t s_bars[tc::kBars];
  // the compact-WY routines' mbarriers (loads, MMAs, A operands ready,
  // epilogue, teardown), used by the tensor-core instantiation only
  __shared__ __align__(8) uint64_t s_wybars[TC ? tc::wy::kBars : 1];
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x;
  if (tid == 0) s_err = (a.hdr->key != a.key || a.hdr->nitems != a.nitems) ? 2 : 0;
  __syncthreads();
  if (s_err) {
    if (tid == 0 && blockIdx.x == 0) atomicExch(&a.hdr->error, 2);
    return;
  }
  uint32_t phase[tc::kBars] = {0u, 0u, 0u, 0u};
  uint32_t wyph[tc::wy::kPh] = {};
  uint32_t tmem = 0;
  bool tc_failed = false;
  if constexpr (TC) {
    if (tid == 0) {
      for (int q = 0; q < tc::kBars; ++q)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::saddr(&s_bars[q])));
      for (int q = 0; q < tc::wy::kBars; ++q) {
        const int count = (q >= 2 * tc::wy::kRing && q < 3 * tc::wy::kRing) ? tc::wy::kWorkers : 1;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc::saddr(&s_wybars[q])), "r"(count));
      }
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
    tmem = s_tmem;
  }
  for (;;) {
    if (tid == 0) s_it = atomicAdd(&a.hdr->head, 1);
    __syncthreads();
    const int idx = s_it;
    if (idx >= a.nitems) break;
    const TItem it = a.items[idx];
    if (tid == 0) {
      int err = 0;
      const unsigned long long t0 = tdag_ns();
      for (int d = 0; d < (int)it.ndep && !err; ++d) {
        const int *f = a.done + a.deps[it.dep + d];
        while (tdag_ld_acquire(f) == 0) {
          if (tdag_ld_acquire(&a.hdr->error) != 0) { err = 1; break; }
          if (tdag_ns() - t0 > a.timeout_ns) {
            if (atomicCAS(&a.hdr->error, 0, 1) == 0) a.hdr->err_item = idx;
            err = 1;
            break;
          }
          __nanosleep(64);
        }
      }
      s_err = err;
    }
    __syncthreads();
    if (s_err) break;
    TreeOp op{};
    op.type = it.type & 0x7f;
    op.ts = (it.type & 0x80) ? 1 : 0;
    op.k = it.k; op.b = it.b;
    op.s = (int)it.p - (int)it.i;
    op.trans = 0; op.a_cols = 1;
    bool ok = true;
    if constexpr (std::is_same<R, float>::value) {
      if (op.type == OP_WY_BUILD) {
        if constexpr (TC) {
          // the slot of one reflector tile: geqrt!'s V (it.b == 0, unit
          // lower) or a merge's V (it.b == 1: tsqrt!'s whole tile, or
          // ttqrt!'s upper triangle)
          const TreeGeom<R> &g = a.g;
          const int k = it.k;
          unsigned char *al = smem + ((1024 - (tc::saddr(smem) & 1023)) & 1023);
          if (it.b == 0) {
            const int i = it.i;
            ok = tc::wy::wy_build(g.rows(i), min(g.rows(i), g.cols(k)), g.tile(i, k), g.lda, g.ttile(g.T, i, k),
                                  g.ldt, tc::kVUnitLower, a.slot(0, i, k), tmem, s_wybars, wyph, al);
          } else {
            const int p = it.p;
            ok = tc::wy::wy_build(g.rows(p), op.ts ? g.cols(k) : min(g.rows(p), g.cols(k)), g.tile(p, k), g.lda,
                                  g.ttile(g.T2, p, k), g.ldt, op.ts ? tc::kVFull : tc::kVUpper, a.slot(1, p, k),
                                  tmem, s_wybars, wyph, al);
          }
        } else {
          ok = false;   // never scheduled without the tensor-core instantiation
        }
      } else if ((op.type == OP_PR_TRAIL_TC || op.type == OP_GE_TRAIL_TC) && a.wy) {
        if constexpr (TC) {
          // one 128-column chunk through the tile's compact-WY slot
          const TreeGeom<R> &g = a.g;
          const int k = it.k;
          const int col = (k + 1) * g.nb + (int)it.y * tc::kChunk;
          const int j = col / g.nb, off = col % g.nb;
          unsigned char *al = smem + ((1024 - (tc::saddr(smem) & 1023)) & 1023);
          const int nb = g.nb, i = it.i;
          if (op.type == OP_GE_TRAIL_TC) {
            const tc::wy::WyMaps mp{&a.tmwy, &a.tmwy, 0, 0, i * nb, col};
            ok = tc::wy::wy_chunk(g.rows(i), min(g.rows(i), g.cols(k)), nullptr, g.lda,
                                  g.tile(i, j) + (size_t)off * g.lda, g.lda, a.slot(0, i, k), mp, tmem, s_wybars,
                                  wyph, al);
          } else {
            const int p = it.p;
            const tc::wy::WyMaps mp{&a.tmwy, &a.tmwy, i * nb, col, p * nb, col};
            ok = tc::wy::wy_chunk(g.rows(p), op.ts ? g.cols(k) : min(g.rows(p), g.cols(k)),
                                  g.tile(i, j) + (size_t)off * g.lda, g.lda, g.tile(p, j) + (size_t)off * g.lda,
                                  g.lda, a.slot(1, p, k), mp, tmem, s_wybars, wyph, al);
          }
        } else {
          ok = false;
        }
      } else if (op.type == OP_PR_TRAIL_TC || op.type == OP_GE_TRAIL_TC) {
        if constexpr (TC) {
          const TreeGeom<R> &g = a.g;
          const int k = it.k;
          const int col = (k + 1) * g.nb + (int)it.y * tc::kChunk;
          const int j = col / g.nb, off = col % g.nb;
          unsigned char *al = smem + ((1024 - (tc::saddr(smem) & 1023)) & 1023);
          const int nb = g.nb, i = it.i;
          if (op.type == OP_GE_TRAIL_TC) {
            // unmqr! of geqrt!'s factor of tile (i, k) on the chunk of tile (i, j)
            const tc::TcMaps mp{&a.tmw, &a.tmw, &a.tmn, 0, 0, i * nb, col, i * nb, k * nb};
            ok = tc::tsmqr_chunk(g.rows(i), min(g.rows(i), g.cols(k)), nullptr, g.lda,
                                 g.tile(i, j) + (size_t)off * g.lda, g.lda, g.tile(i, k), g.lda,
                                 g.ttile(g.T, i, k), g.ldt, tmem, s_bars, phase, al, tc::kVUnitLower,
                                 a.tma ? &mp : nullptr);
          } else {
            const int p = it.p;
            const tc::TcMaps mp{&a.tmw, &a.tmw, &a.tmn, i * nb, col, p * nb, col, p * nb, k * nb};
            ok = tc::tsmqr_chunk(g.rows(p), op.ts ? g.cols(k) : min(g.rows(p), g.cols(k)),
                                 g.tile(i, j) + (size_t)off * g.lda, g.lda, g.tile(p, j) + (size_t)off * g.lda,
                                 g.lda, g.tile(p, k), g.lda, g.ttile(g.T2, p, k), g.ldt, tmem, s_bars, phase, al,
                                 op.ts ? tc::kVFull : tc::kVUpper, a.tma ? &mp : nullptr);
          }
        } else {
          ok = false;   // never scheduled without the tensor-core instantiation
        }
      } else if (a.D && (op.type == OP_GE_PANEL || op.type == OP_PR_PANEL)) {
        tree_panel_f64(a, op, it.i, smem);
      } else {
        tree_task<R>(a.g, op, it.i, it.y, smem);
      }
    } else {
      tree_task<R>(a.g, op, it.i, it.y, smem);
    }
    if (!ok) {
      if (tid == 0 && atomicCAS(&a.hdr->error, 0, 3) == 0) a.hdr->err_item = idx;
      tc_failed = true;
      break;
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      tdag_st_release(a.done + idx, 1);
    }
  }
  if constexpr (TC) {
    // after a failed wait: one more commit (it arrives once every earlier MMA
    // has completed) and one bounded wait for it, then release TMEM
    if (tc_failed) {
      if (tid == 0) tc::commit(&s_bars[2]);
      tc::bar_wait(&s_bars[2], phase[2]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((tid >> 5) == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::kTmemCols));
  }
  (void)tc_failed;
}

// ---- host: task graph construction -----------------------------------------
struct TreeShape {
  int m, n, nb, ib, nrhs, MT, NT, KT;
  int grp = 1;
  int nw = kTreeNW; // strip width (TreeNW of the element type)
  int tc = 0;       // FP32: trailing updates of A as tensor-core chunk tasks
  int wy = 0;       // with tc: the chunk tasks in compact-WY form, one slot build per reflector tile
  int f64p = 0;     // FP32: panel steps in FP64 (the mixed form)
  int rows(int i) const { return std::min(nb, m - i * nb); }
  int cols(int k) const { return std::min(nb, n - k * nb); }
  int strips(int j) const { return j < NT ? (cols(j) + nw - 1) / nw : (nrhs + nw - 1) / nw; }
  bool ragged(int k) const { int p = MT - 1; return p > k && rows(p) < cols(k); }
};

struct TreePlan {
  TreeShape sh;
  long long key = 0;
  std::vector<TItem> items;
  std::vector<uint32_t> deps;
  unsigned char *pinned = nullptr;      // header + items + deps, page-locked
  std::vector<unsigned char> pageable;
  size_t off_items = 0, off_deps = 0, img_bytes = 0, done_bytes = 0, total_bytes = 0;
  const unsigned char *image() const { return pinned ? pinned : pageable.data(); }
  ~TreePlan() {
    if (pinned) cudaFreeHost(pinned);
  }
};

static double tree_cost(const TreeShape &sh, const TItem &it) {
  const double ib = sh.ib, w = sh.nw, nb = sh.nb;
  const int t = it.type & 0x7f;
  const bool ts = it.type & 0x80;
  const double lat = 64.0 * ib * 600;          // serial column steps of a panel
  switch (t) {
    case OP_GE_PANEL: return 3.0 * (sh.rows(it.i) - it.b * ib) * ib * ib + lat;
    case OP_GE_APPLY: return 4.0 * (sh.rows(it.i) - it.b * ib) * ib * w;
    case OP_GE_TRAIL: return 4.0 * sh.rows(it.i) * std::min(sh.rows(it.i), sh.cols(it.k)) * w;
    case OP_PR_PANEL: return 3.0 * (ts ? sh.rows(it.p) : (it.b + 1) * ib) * ib * ib + lat;
    case OP_PR_APPLY: return 4.0 * (ts ? sh.rows(it.p) : (it.b + 1) * ib) * ib * w;
    case OP_PR_TRAIL_TC: return 4.0 * sh.rows(it.p) * sh.cols(it.k) * tc::kChunk / 6.0;   // ~6x a SIMT strip
    case OP_GE_TRAIL_TC: return 4.0 * sh.rows(it.i) * sh.cols(it.k) * tc::kChunk / 6.0;
    case OP_WY_BUILD: return 4.0 * nb * sh.cols(it.k) * tc::kChunk / 6.0;
    default: return (ts ? 4.0 * sh.rows(it.p) : 2.0 * nb) * sh.cols(it.k) * w;
  }
}

// Builds the task list in program order with its dependencies, then sorts it.
static void tree_build(const TreeShape &sh, std::vector<TItem> &out_items, std::vector<uint32_t> &out_deps) {
  const int NS = std::max(sh.nb / sh.nw, (sh.nrhs + sh.nw - 1) / sh.nw);
  const int NJ = sh.NT + 1;                    // tile columns plus the right-hand sides
  const int nblk = (sh.nb + sh.ib - 1) / sh.ib;
  // regions: tile strips (upper / lower part), then T blocks of geqrt and of the merges
  const size_t nstrip = (size_t)sh.MT * NJ * NS * 2;
  auto rg = [&](int i, int j, int s, int lower) { return (((size_t)i * NJ + j) * NS + s) * 2 + lower; };
  auto rt = [&](int i, int k, int b, int merge) {
    return nstrip + (((size_t)i * sh.KT + k) * nblk + b) * 2 + merge;
  };
  // compact-WY slots (wy_slot), after the T blocks
  const size_t nslot_reg = nstrip + (size_t)sh.MT * sh.KT * nblk * 2;
  auto rs = [&](int merge, int row, int k) { return nslot_reg + (size_t)wy_slot(sh.MT, merge, row, k); };
  const size_t nreg = nslot_reg + (size_t)4 * sh.MT;
  std::vector<int> last(nreg, -1);
  std::vector<std::vector<int>> readers(nreg);
  std::vector<TItem> items;
  std::vector<std::vector<int>> preds;
  std::vector<int> cur;
  auto rd = [&](size_t r) {
    if (last[r] >= 0) cur.push_back(last[r]);
    readers[r].push_back((int)items.size());
  };
  auto wr = [&](size_t r) {
    if (last[r] >= 0) cur.push_back(last[r]);
    for (int x : readers[r]) cur.push_back(x);
    readers[r].clear();
    last[r] = (int)items.size();
  };
  auto emit = [&](int type, int k, int b, int i, int p, int y) {
    TItem it;
    it.type = (uint8_t)type; it.b = (uint8_t)b; it.k = (uint16_t)k; it.i = (uint16_t)i;
    it.p = (uint16_t)p; it.y = (uint16_t)y; it.ndep = 0; it.dep = 0;
    std::sort(cur.begin(), cur.end());
    cur.erase(std::unique(cur.begin(), cur.end()), cur.end());
    // a task that reads and writes disjoint columns of one region (a ragged
    // block) records itself; it never waits on itself
    cur.erase(std::remove(cur.begin(), cur.end(), (int)items.size()), cur.end());
    preds.push_back(cur);
    cur.clear();
    items.push_back(it);
  };
  // trailing strip y of panel k -> (tile column, strip)
  auto trail_js = [&](int k, int y, int &j, int &s) {
    const int ca = std::max(0, sh.n - (k + 1) * sh.nb);
    const int sa = (ca + sh.nw - 1) / sh.nw;
    if (y < sa) { const int c = y * sh.nw; j = k + 1 + c / sh.nb; s = (c % sh.nb) / sh.nw; }
    else { j = sh.NT; s = y - sa; }
  };
  auto ntrail = [&](int k) {
    const int ca = std::max(0, sh.n - (k + 1) * sh.nb);
    return (ca + sh.nw - 1) / sh.nw + (sh.nrhs + sh.nw - 1) / sh.nw;
  };
  const int G = sh.grp;
  for (int k = 0; k < sh.KT; ++k) {
    const int nk = sh.cols(k), NSk = sh.strips(k);   // NSk: strips of the panel's tile column
    const bool rag = sh.ragged(k);
    const int MTt = rag ? sh.MT - 1 : sh.MT;
    const int last = k + ((MTt - 1 - k) / G) * G;    // last group leader
    // geqrt of every group leader, block by block, then unmqr of its row
    for (int i = k; i < MTt; i += G) {
      const int kk = std::min(sh.rows(i), nk);
      for (int b = 0, c = 0; c < kk; ++b, c += sh.ib) {
        const int sb = std::min(sh.ib, kk - c);
        const int q0 = c / sh.nw, q1 = (c + sb + sh.nw - 1) / sh.nw;
        for (int q = q0; q < q1; ++q) { wr(rg(i, k, q, 0)); wr(rg(i, k, q, 1)); }
        wr(rt(i, k, b, 0));
        emit(OP_GE_PANEL, k, b, i, i, 0);
        // strip y covers columns [c + sb + 16 y, +16) clipped to nk (as in tree_task)
        for (int y = 0; c + sb + y * sh.nw < nk; ++y) {
          const int c0 = c + sb + y * sh.nw, c1 = std::min(nk, c0 + sh.nw);
          for (int v = q0; v < q1; ++v) rd(rg(i, k, v, 1));
          rd(rt(i, k, b, 0));
          for (int q = c0 / sh.nw; q <= (c1 - 1) / sh.nw; ++q) { wr(rg(i, k, q, 0)); wr(rg(i, k, q, 1)); }
          emit(OP_GE_APPLY, k, b, i, i, y);
        }
      }
      const int nbk = (kk + sh.ib - 1) / sh.ib;
      // tensor-core chunks of A's trailing columns for a full tile, then
      // strips for the rest (B's columns)
      int y0 = 0;
      const int ca = std::max(0, sh.n - (k + 1) * sh.nb);
      if (sh.tc && sh.rows(i) == sh.nb && kk == sh.nb && ca % tc::kChunk == 0) {
        if (sh.wy && ca > 0) {
          // the slot of geqrt!'s V and T for the chunks below
          for (int q = 0; q < NSk; ++q) rd(rg(i, k, q, 1));
          for (int b = 0; b < nbk; ++b) rd(rt(i, k, b, 0));
          wr(rs(0, i, k));
          emit(OP_WY_BUILD, k, 0, i, i, 0);
        }
        for (int ch = 0; ch < ca / tc::kChunk; ++ch) {
          if (sh.wy) {
            rd(rs(0, i, k));
          } else {
            for (int q = 0; q < NSk; ++q) rd(rg(i, k, q, 1));
            for (int b = 0; b < nbk; ++b) rd(rt(i, k, b, 0));
          }
          const int c0 = ch * tc::kChunk, j = k + 1 + c0 / sh.nb, s0 = (c0 % sh.nb) / sh.nw;
          for (int s = s0; s < s0 + tc::kChunk / sh.nw; ++s) { wr(rg(i, j, s, 0)); wr(rg(i, j, s, 1)); }
          emit(OP_GE_TRAIL_TC, k, 0, i, i, ch);
        }
        y0 = (ca + sh.nw - 1) / sh.nw;
      }
      for (int y = y0; y < ntrail(k); ++y) {
        int j, s;
        trail_js(k, y, j, s);
        for (int q = 0; q < NSk; ++q) rd(rg(i, k, q, 1));
        for (int b = 0; b < nbk; ++b) rd(rt(i, k, b, 0));
        wr(rg(i, j, s, 0)); wr(rg(i, j, s, 1));
        emit(OP_GE_TRAIL, k, 0, i, i, y);
      }
    }
    auto merge = [&](int i, int p, int ts) {
      const int kt = ts ? nk : std::min(sh.rows(p), nk);
      const int flag = ts ? 0x80 : 0;
      for (int b = 0, c = 0; c < kt; ++b, c += sh.ib) {
        const int sb = std::min(sh.ib, kt - c);
        const int q0 = c / sh.nw, q1 = (c + sb + sh.nw - 1) / sh.nw;
        for (int q = q0; q < q1; ++q) {
          wr(rg(i, k, q, 0));
          wr(rg(p, k, q, 0));
          if (ts) wr(rg(p, k, q, 1));
        }
        wr(rt(p, k, b, 1));
        emit(OP_PR_PANEL | flag, k, b, i, p, 0);
        for (int y = 0; c + sb + y * sh.nw < nk; ++y) {
          const int c0 = c + sb + y * sh.nw, c1 = std::min(nk, c0 + sh.nw);
          for (int v = q0; v < q1; ++v) {
            rd(rg(p, k, v, 0));
            if (ts) rd(rg(p, k, v, 1));
          }
          rd(rt(p, k, b, 1));
          for (int q = c0 / sh.nw; q <= (c1 - 1) / sh.nw; ++q) {
            wr(rg(i, k, q, 0));
            wr(rg(p, k, q, 0));
            if (ts) wr(rg(p, k, q, 1));
          }
          emit(OP_PR_APPLY | flag, k, b, i, p, y);
        }
      }
      const int nbk = (kt + sh.ib - 1) / sh.ib;
      // tensor-core chunks of A's trailing columns for a merge of full tiles,
      // then strips for the rest (B's columns)
      int y0 = 0;
      const int ca = std::max(0, sh.n - (k + 1) * sh.nb);
      if (sh.tc && sh.rows(p) == sh.nb && sh.rows(i) == sh.nb && kt == sh.nb && ca % tc::kChunk == 0) {
        if (sh.wy && ca > 0) {
          // the slot of the merge's V and T for the chunks below
          for (int q = 0; q < NSk; ++q) {
            rd(rg(p, k, q, 0));
            if (ts) rd(rg(p, k, q, 1));
          }
          for (int b = 0; b < nbk; ++b) rd(rt(p, k, b, 1));
          wr(rs(1, p, k));
          emit(OP_WY_BUILD | flag, k, 1, i, p, 0);
        }
        for (int ch = 0; ch < ca / tc::kChunk; ++ch) {
          if (sh.wy) {
            rd(rs(1, p, k));
          } else {
            for (int q = 0; q < NSk; ++q) {
              rd(rg(p, k, q, 0));
              if (ts) rd(rg(p, k, q, 1));
            }
            for (int b = 0; b < nbk; ++b) rd(rt(p, k, b, 1));
          }
          const int c0 = ch * tc::kChunk, j = k + 1 + c0 / sh.nb, s0 = (c0 % sh.nb) / sh.nw;
          for (int s = s0; s < s0 + tc::kChunk / sh.nw; ++s) {
            wr(rg(i, j, s, 0)); wr(rg(i, j, s, 1));
            wr(rg(p, j, s, 0)); wr(rg(p, j, s, 1));
          }
          emit(OP_PR_TRAIL_TC | flag, k, 0, i, p, ch);
        }
        y0 = (ca + sh.nw - 1) / sh.nw;
      }
      for (int y = y0; y < ntrail(k); ++y) {
        int j, s;
        trail_js(k, y, j, s);
        for (int q = 0; q < NSk; ++q) {
          rd(rg(p, k, q, 0));
          if (ts) rd(rg(p, k, q, 1));
        }
        for (int b = 0; b < nbk; ++b) rd(rt(p, k, b, 1));
        wr(rg(i, j, s, 0)); wr(rg(i, j, s, 1));
        wr(rg(p, j, s, 0)); wr(rg(p, j, s, 1));
        emit(OP_PR_TRAIL | flag, k, 0, i, p, y);
      }
    };
    for (int d = 1; d < G; ++d)
      for (int i = k; i + d < MTt; i += G) merge(i, i + d, 1);
    if (rag) merge(last, sh.MT - 1, 1);
    for (int s = G; k + s < MTt; s *= 2)
      for (int i = k; i + s < MTt; i += 2 * s) merge(i, i + s, 0);
  }
  // longest path to the end, then a stable sort by it
  const int N = (int)items.size();
  std::vector<double> rank(N, 0.0);
  for (int x = N - 1; x >= 0; --x) {
    rank[x] += tree_cost(sh, items[x]);
    for (int pr : preds[x]) rank[pr] = std::max(rank[pr], rank[x]);
  }
  std::vector<int> order(N), pos(N);
  for (int x = 0; x < N; ++x) order[x] = x;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rank[a] > rank[b]; });
  for (int x = 0; x < N; ++x) pos[order[x]] = x;
  out_items.resize(N);
  out_deps.clear();
  for (int q = 0; q < N; ++q) {
    const int x = order[q];
    TItem it = items[x];
    it.dep = (uint32_t)out_deps.size();
    it.ndep = (uint16_t)preds[x].size();
    for (int pr : preds[x]) out_deps.push_back((uint32_t)pos[pr]);
    out_items[q] = it;
  }
}

static long long tree_key(const TreeShape &sh) {
  long long h = 7809847782465536322LL;
  // f64p changes no task or dependency (only the device routines of the
  // panel tasks), so it shares the plan
  for (int v : {sh.m, sh.n, sh.nb, sh.ib, sh.nrhs, sh.grp, sh.tc, sh.wy, sh.nw == kTreeNW ? 0 : sh.nw, 0x7ee})
    h = (h ^ (long long)v) * 1099511628211LL;
  return h & 0x7fffffffffffffffLL;
}

static std::mutex g_tplan_mu;
static std::map<long long, std::shared_ptr<TreePlan>> g_tplans;

static bool tree_dag_shape(int m, int n, int nb, int ib, int nrhs, TreeShape *sh, int grp = 1, int nw = kTreeNW) {
  if (m <= 0 || n <= 0 || nb <= 0 || nb > 256 || nb % nw) return false;
  if (grp <= 0) return false;
  sh->grp = grp;
  sh->nw = nw;
  if (ib <= 0 || ib > 32 || ib % nw || nb % ib) return false;
  if (nrhs < 0 || nrhs > 256) return false;
  sh->m = m; sh->n = n; sh->nb = nb; sh->ib = ib; sh->nrhs = nrhs;
  sh->MT = (m + nb - 1) / nb; sh->NT = (n + nb - 1) / nb; sh->KT = std::min(sh->MT, sh->NT);
  if (sh->MT > 65535 || sh->NT > 65535) return false;
  return true;
}

static std::shared_ptr<TreePlan> tree_plan(const TreeShape &sh) {
  const long long key = tree_key(sh);
  std::lock_guard<std::mutex> l(g_tplan_mu);
  auto f = g_tplans.find(key);
  if (f != g_tplans.end()) return f->second;
  auto p = std::make_shared<TreePlan>();
  p->sh = sh;
  p->key = key;
  tree_build(sh, p->items, p->deps);
  const size_t N = p->items.size();
  p->off_items = 256;
  p->off_deps = align256(p->off_items + sizeof(TItem) * N);
  p->img_bytes = p->off_deps + sizeof(uint32_t) * p->deps.size();
  p->done_bytes = align256(sizeof(int) * N);
  p->total_bytes = align256(p->img_bytes) + p->done_bytes;
  unsigned char *dst = nullptr;
  if (cudaMallocHost((void **)&p->pinned, p->img_bytes) == cudaSuccess) {
    dst = p->pinned;
  } else {
    p->pinned = nullptr;
    cudaGetLastError();
    p->pageable.resize(p->img_bytes);
    dst = p->pageable.data();
  }
  std::memset(dst, 0, p->img_bytes);
  TDagHeader h;
  std::memset(&h, 0, sizeof(h));
  h.key = key;
  h.nitems = (int)N;
  std::memcpy(dst, &h, sizeof(h));
  std::memcpy(dst + p->off_items, p->items.data(), sizeof(TItem) * N);
  std::memcpy(dst + p->off_deps, p->deps.data(), sizeof(uint32_t) * p->deps.size());
  g_tplans[key] = p;
  return p;
}

// The tensor-core and FP64-panel options of an FP32 task graph: tensor-core
// chunks need full 256 x 256 tiles with ib = 32, a 16-byte aligned A and a
// leading dimension that keeps every column 16-byte aligned; the FP64 panels
// (mixed form) need full tiles and ib <= 32.
static bool tree_tc_ok(const TreeShape &sh, const void *A, int lda) {
  return sh.nb == 256 && sh.ib == tc::kIb && sh.m % sh.nb == 0 && sh.n % sh.nb == 0 && ((uintptr_t)A & 15) == 0 &&
         (lda & 3) == 0;
}
static bool tree_f64p_ok(const TreeShape &sh) { return sh.m % sh.nb == 0 && sh.n % sh.nb == 0 && sh.ib <= 32; }

// Bytes of the FP64 triangles of the mixed form (after the plan's bytes).
static size_t tree_d_bytes(const TreeShape &sh) {
  return align256(sizeof(double) * (size_t)sh.MT * sh.KT * sh.nb * sh.ib);
}

// Bytes of the compact-WY slots (after the FP64 triangles).
static size_t tree_wy_bytes(const TreeShape &sh) { return (size_t)4 * sh.MT * tc::wy::kSlotBytes; }

// Workspace covering the plain plan and, for FP32-eligible shapes, the
// tensor-core plans (other task lists), the FP64 triangles and the
// compact-WY slots.
static size_t tree_work_bytes(TreeShape sh) {
  size_t b = tree_plan(sh)->total_bytes;
  const size_t d = tree_f64p_ok(sh) ? tree_d_bytes(sh) : 0;
  b += d;
  if (sh.nb == 256 && sh.ib == tc::kIb && sh.m % sh.nb == 0 && sh.n % sh.nb == 0) {
    sh.tc = 1;
    b = std::max(b, tree_plan(sh)->total_bytes + d);
    sh.wy = 1;
    b = std::max(b, tree_plan(sh)->total_bytes + d + tree_wy_bytes(sh));
    sh.tc = 0;
    sh.wy = 0;
  }
  // ComplexF64 runs 8-column strips: another task list
  TreeShape sz = sh;
  if (tree_dag_shape(sh.m, sh.n, sh.nb, sh.ib, sh.nrhs, &sz, sh.grp, TreeNW<cx<double>>::value))
    b = std::max(b, tree_plan(sz)->total_bytes);
  return b;
}

template <typename R, bool TC>
static cudaError_t tree_dag_launch(const TDagArgs<R> &a, size_t sm, cudaStream_t st) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_tree_dag<R, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) !=
      cudaSuccess)
    return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tree_dag<R, TC>, TQR_THREADS, sm)) !=
      cudaSuccess)
    return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int grid = std::min(sms * per_sm, a.nitems);
  k_tree_dag<R, TC><<<grid, TQR_THREADS, sm, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

// mixed: FP32 only -- FP64 panel steps (and tensor-core updates where the
// shape allows), the factorisation of the mixed-precision solve.  Plain FP32
// graphs use the tensor cores too unless tqr_tile_dag_tensor_cores(0).
template <typename R>
static int tree_geqrf_dag_impl(int m, int n, int nb, int ib, R *A, int lda, R *T, R *T2, int ldt, R *tau,
                               R *tau2, int ldtau, int nrhs, R *B, int ldb, void *work, size_t lwork,
                               cudaStream_t st, int grp = 1, bool mixed = false) {
  if (grp <= 0) return -5;
  TreeGeom<R> g;
  int rc = tree_geom<R>(m, n, nrhs, nb, ib, A, lda, B, ldb, T, T2, ldt, tau, tau2, ldtau, &g, grp);
  if (rc) return rc;
  if (m == 0 || n == 0) return 0;
  if (!A || lda < m) return -6;
  if (!T || !T2 || ldt < g.MT * ib) return -9;
  if (!tau || !tau2 || ldtau < n) return -12;
  if (nrhs < 0) return -13;
  if (nrhs > 0 && (!B || ldb < m)) return -15;
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh, grp, TreeNW<R>::value)) return -3;
  if constexpr (std::is_same<R, float>::value) {
    if (tree_tc_ok(sh, A, lda) && (mixed || tile_tc_enabled())) sh.tc = 1;
    if (mixed) {
      if (!tree_f64p_ok(sh)) return -3;
      sh.f64p = 1;
    }
  } else {
    if (mixed) return -3;
  }
  TDagArgs<R> a;
  if constexpr (std::is_same<R, float>::value) {
    // compact-WY chunks need their tensor map of A (16 x 128 boxes)
    if (sh.tc && tc_wy_enabled() &&
        make_tmap_f32(&a.tmwy, A, m, n, lda, tc::wy::kKs, tc::kChunk, 64) == cudaSuccess)
      sh.wy = 1;
  }
  std::shared_ptr<TreePlan> p = tree_plan(sh);
  const size_t dbytes = sh.f64p ? tree_d_bytes(sh) : 0;
  const size_t sbytes = sh.wy ? tree_wy_bytes(sh) : 0;
  if (!work || ((uintptr_t)work & 255)) return -16;
  if (lwork < p->total_bytes + dbytes + sbytes) return -17;
  unsigned char *w = (unsigned char *)work;
  int *done = (int *)(w + align256(p->img_bytes));
  cudaError_t e;
  if ((e = cudaMemcpyAsync(w, p->image(), p->img_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) return (int)e;
  if ((e = cudaMemsetAsync(done, 0, sizeof(int) * p->items.size(), st)) != cudaSuccess) return (int)e;
  if ((e = cudaMemset2DAsync(T2, sizeof(R) * ldt, 0, sizeof(R) * g.MT * ib, n, st)) != cudaSuccess) return (int)e;
  a.g = g;
  a.hdr = (TDagHeader *)w;
  a.done = done;
  a.items = (const TItem *)(w + p->off_items);
  a.deps = (const uint32_t *)(w + p->off_deps);
  a.nitems = (int)p->items.size();
  a.key = p->key;
  a.timeout_ns = 20000000000ull;
  if (sh.f64p) a.D = (double *)(w + p->total_bytes);
  if (sh.wy) {
    a.wy = 1;
    a.slots = w + p->total_bytes + dbytes;
  }
  if constexpr (std::is_same<R, float>::value) {
    if (sh.tc && tc_tma_enabled())
      a.tma = make_tmap_f32(&a.tmw, A, m, n, lda, 32, tc::kChunk) == cudaSuccess &&
              make_tmap_f32(&a.tmn, A, m, n, lda, 32, tc::kIb) == cudaSuccess;
  }
  size_t sm = tree_smem<R>();
  if (sh.f64p)
    sm = std::max({sm, panel_f64_smem(nb, ib), tsqrt_f64x_smem(nb, ib), ttqrt_f64_smem(nb, ib)});
  if constexpr (std::is_same<R, float>::value) {
    if (sh.tc) {
      e = tree_dag_launch<R, true>(a, std::max({sm, tc::kSmem, tc::wy::kSmem}), st);
      return e == cudaSuccess ? 0 : (int)e;
    }
  }
  e = tree_dag_launch<R, false>(a, sm, st);
  return e == cudaSuccess ? 0 : (int)e;
}

int stile_gels_hqr_mixed(int m, int n, int nrhs, int nb, int ib, int grp, float *A, int lda, float *T, float *T2,
                         int ldt, float *tau, float *tau2, int ldtau, float *B, int ldb, void *work, size_t lwork,
                         cudaStream_t stream) {
  if (nrhs < 0) return -3;
  int rc = tree_geqrf_dag_impl<float>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, work, lwork,
                                      stream, grp, true);
  if (rc != 0) return rc;
  return nrhs > 0 ? tqr_strsm_lun(n, nrhs, A, lda, B, ldb, stream) : 0;
}

size_t tree_dag_work_bytes(int m, int n, int nb, int ib, int grp, int nrhs) {
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh, grp)) return 0;
  return tree_work_bytes(sh);
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

#define TQR_HQR(P, R)                                                                                          \
  int tqr_##P##tile_geqrf_hqr(int m, int n, int nb, int ib, int grp, R *A, int lda, R *T, R *T2, int ldt, R *tau, \
                              R *tau2, int ldtau, int nrhs, R *B, int ldb, cudaStream_t stream) {                \
    return tree_geqrf_impl<R>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, stream, grp);    \
  }                                                                                                              \
  int tqr_##P##tile_unmqr_hqr(char trans, int m, int n, int nrhs, int nb, int ib, int grp, const R *A, int lda,  \
                              const R *T, const R *T2, int ldt, R *B, int ldb, cudaStream_t stream) {            \
    return tree_unmqr_impl<R>(trans, m, n, nrhs, nb, ib, A, lda, T, T2, ldt, B, ldb, stream, grp);               \
  }                                                                                                              \
  int tqr_##P##tile_geqrf_hqr_dag(int m, int n, int nb, int ib, int grp, R *A, int lda, R *T, R *T2, int ldt,    \
                                  R *tau, R *tau2, int ldtau, int nrhs, R *B, int ldb, void *work, size_t lwork, \
                                  cudaStream_t stream) {                                                         \
    return tree_geqrf_dag_impl<R>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, work, lwork, \
                                  stream, grp);                                                                  \
  }
TQR_HQR(d, double)
TQR_HQR(s, float)
#undef TQR_HQR

// ComplexF64 (z) and ComplexF32 (c): the same drivers on cx<double> /
// cx<float> elements (Julia's Complex layout, real part first); the element
// pointers must be aligned to the element size.
#define TQR_TREE_CX(P, CT, E)                                                                                 \
  int tqr_##P##tile_geqrf_tree(int m, int n, int nb, int ib, CT *A, int lda, CT *T, CT *T2, int ldt, CT *tau,    \
                               CT *tau2, int ldtau, int nrhs, CT *B, int ldb, cudaStream_t stream) {            \
    if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)T2 | (uintptr_t)tau | (uintptr_t)tau2 | (uintptr_t)B) %      \
        alignof(E))                                                                                           \
      return -5;                                                                                              \
    return tree_geqrf_impl<E>(m, n, nb, ib, (E *)A, lda, (E *)T, (E *)T2, ldt, (E *)tau, (E *)tau2, ldtau,     \
                              nrhs, (E *)B, ldb, stream);                                                     \
  }                                                                                                           \
  int tqr_##P##tile_unmqr_tree(char trans, int m, int n, int nrhs, int nb, int ib, const CT *A, int lda,       \
                               const CT *T, const CT *T2, int ldt, CT *B, int ldb, cudaStream_t stream) {       \
    if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)T2 | (uintptr_t)B) % alignof(E)) return -7;                 \
    return tree_unmqr_impl<E>(trans, m, n, nrhs, nb, ib, (const E *)A, lda, (const E *)T, (const E *)T2, ldt, \
                              (E *)B, ldb, stream);                                                           \
  }                                                                                                           \
  int tqr_##P##tile_geqrf_hqr(int m, int n, int nb, int ib, int grp, CT *A, int lda, CT *T, CT *T2, int ldt,     \
                              CT *tau, CT *tau2, int ldtau, int nrhs, CT *B, int ldb, cudaStream_t stream) {     \
    if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)T2 | (uintptr_t)tau | (uintptr_t)tau2 | (uintptr_t)B) %      \
        alignof(E))                                                                                           \
      return -6;                                                                                              \
    return tree_geqrf_impl<E>(m, n, nb, ib, (E *)A, lda, (E *)T, (E *)T2, ldt, (E *)tau, (E *)tau2, ldtau,     \
                              nrhs, (E *)B, ldb, stream, grp);                                                \
  }                                                                                                           \
  int tqr_##P##tile_unmqr_hqr(char trans, int m, int n, int nrhs, int nb, int ib, int grp, const CT *A,       \
                              int lda, const CT *T, const CT *T2, int ldt, CT *B, int ldb, cudaStream_t stream) { \
    if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)T2 | (uintptr_t)B) % alignof(E)) return -8;                 \
    return tree_unmqr_impl<E>(trans, m, n, nrhs, nb, ib, (const E *)A, lda, (const E *)T, (const E *)T2, ldt, \
                              (E *)B, ldb, stream, grp);                                                      \
  }                                                                                                           \
  int tqr_##P##tile_geqrf_hqr_dag(int m, int n, int nb, int ib, int grp, CT *A, int lda, CT *T, CT *T2,        \
                                  int ldt, CT *tau, CT *tau2, int ldtau, int nrhs, CT *B, int ldb, void *work,    \
                                  size_t lwork, cudaStream_t stream) {                                        \
    if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)T2 | (uintptr_t)tau | (uintptr_t)tau2 | (uintptr_t)B) %      \
        alignof(E))                                                                                           \
      return -6;                                                                                              \
    return tree_geqrf_dag_impl<E>(m, n, nb, ib, (E *)A, lda, (E *)T, (E *)T2, ldt, (E *)tau, (E *)tau2, ldtau, \
                                  nrhs, (E *)B, ldb, work, lwork, stream, grp);                               \
  }                                                                                                           \
  int tqr_##P##tile_geqrf_tree_dag(int m, int n, int nb, int ib, CT *A, int lda, CT *T, CT *T2, int ldt,       \
                                   CT *tau, CT *tau2, int ldtau, int nrhs, CT *B, int ldb, void *work,          \
                                   size_t lwork, cudaStream_t stream) {                                       \
    if (((uintptr_t)A | (uintptr_t)T | (uintptr_t)T2 | (uintptr_t)tau | (uintptr_t)tau2 | (uintptr_t)B) %      \
        alignof(E))                                                                                           \
      return -5;                                                                                              \
    return tree_geqrf_dag_impl<E>(m, n, nb, ib, (E *)A, lda, (E *)T, (E *)T2, ldt, (E *)tau, (E *)tau2, ldtau, \
                                  nrhs, (E *)B, ldb, work, lwork, stream);                                    \
  }
TQR_TREE_CX(z, tqr_zcomplex, cx<double>)
TQR_TREE_CX(c, tqr_ccomplex, cx<float>)
#undef TQR_TREE_CX

int tqr_tile_hqr_dag_check_strips(int m, int n, int nb, int ib, int grp, int nrhs, int nw, long long *ntasks) {
  TreeShape sh;
  if (nw <= 0 || !tree_dag_shape(m, n, nb, ib, nrhs, &sh, grp, nw)) return -1;
  std::shared_ptr<TreePlan> p = tree_plan(sh);
  for (size_t q = 0; q < p->items.size(); ++q) {
    const TItem &it = p->items[q];
    for (int d = 0; d < (int)it.ndep; ++d)
      if (p->deps[it.dep + d] >= q) return 1;
  }
  if (ntasks) *ntasks = (long long)p->items.size();
  return 0;
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

extern "C" {

int tqr_tile_tree_dag_worksize(int m, int n, int nb, int ib, int nrhs, size_t *bytes) {
  if (!bytes) return -6;
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh)) return -1;
  *bytes = tree_work_bytes(sh);
  return 0;
}

int tqr_tile_tree_dag_check(int m, int n, int nb, int ib, int nrhs, long long *ntasks) {
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh)) return -1;
  std::shared_ptr<TreePlan> p = tree_plan(sh);
  // every dependency points to an earlier task of the sorted order
  for (size_t q = 0; q < p->items.size(); ++q) {
    const TItem &it = p->items[q];
    for (int d = 0; d < (int)it.ndep; ++d)
      if (p->deps[it.dep + d] >= q) return 1;
  }
  if (ntasks) *ntasks = (long long)p->items.size();
  return 0;
}

int tqr_tile_hqr_dag_worksize(int m, int n, int nb, int ib, int grp, int nrhs, size_t *bytes) {
  if (!bytes) return -7;
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh, grp)) return -1;
  *bytes = tree_work_bytes(sh);
  return 0;
}

int tqr_stile_geqrf_hqr_dag_f64p(int m, int n, int nb, int ib, int grp, float *A, int lda, float *T, float *T2,
                                 int ldt, float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb, void *work,
                                 size_t lwork, cudaStream_t stream) {
  return tree_geqrf_dag_impl<float>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, work, lwork,
                                    stream, grp, true);
}

int tqr_tile_hqr_dag_check_tc(int m, int n, int nb, int ib, int grp, int nrhs, long long *ntasks) {
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh, grp)) return -1;
  if (nb != 256 || ib != tc::kIb || m % nb || n % nb) return -1;
  sh.tc = 1;
  std::shared_ptr<TreePlan> p = tree_plan(sh);
  long long ntc = 0;
  for (size_t q = 0; q < p->items.size(); ++q) {
    const TItem &it = p->items[q];
    if ((it.type & 0x7f) == OP_PR_TRAIL_TC || (it.type & 0x7f) == OP_GE_TRAIL_TC) ++ntc;
    for (int d = 0; d < (int)it.ndep; ++d)
      if (p->deps[it.dep + d] >= q) return 1;
  }
  if (ntasks) *ntasks = ntc;
  return 0;
}

int tqr_tile_hqr_dag_check_wy(int m, int n, int nb, int ib, int grp, int nrhs, long long *nbuild,
                              long long *nchunk) {
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh, grp)) return -1;
  if (nb != 256 || ib != tc::kIb || m % nb || n % nb) return -1;
  sh.tc = 1;
  sh.wy = 1;
  std::shared_ptr<TreePlan> p = tree_plan(sh);
  const size_t N = p->items.size();
  auto slot_of = [&](const TItem &it) {
    const int t = it.type & 0x7f;
    const int merge = t == OP_WY_BUILD ? it.b : (t == OP_PR_TRAIL_TC ? 1 : 0);
    return wy_slot(sh.MT, merge, merge ? it.p : it.i, it.k);
  };
  // per slot: the position of its current build and the chunks that read it
  std::vector<long long> build_at((size_t)4 * sh.MT, -1);
  std::vector<std::vector<long long>> readers((size_t)4 * sh.MT);
  long long nb_ = 0, nc = 0;
  for (size_t q = 0; q < N; ++q) {
    const TItem &it = p->items[q];
    const uint32_t *d = p->deps.data() + it.dep;
    for (int x = 0; x < (int)it.ndep; ++x)
      if (d[x] >= q) return 1;   // not topological
    const int t = it.type & 0x7f;
    if (t != OP_WY_BUILD && t != OP_PR_TRAIL_TC && t != OP_GE_TRAIL_TC) continue;
    const int s = slot_of(it);
    auto has_dep = [&](long long on) {
      for (int x = 0; x < (int)it.ndep; ++x)
        if ((long long)d[x] == on) return true;
      return false;
    };
    if (t == OP_WY_BUILD) {
      // the rebuild waits for every chunk that read the slot's previous contents
      for (long long r : readers[s])
        if (!has_dep(r)) return 2;
      readers[s].clear();
      build_at[s] = (long long)q;
      ++nb_;
    } else {
      // a chunk reads the build of its own reflector tile (same panel)
      const long long b = build_at[s];
      if (b < 0 || p->items[b].k != it.k || !has_dep(b)) return 3;
      readers[s].push_back((long long)q);
      ++nc;
    }
  }
  if (nbuild) *nbuild = nb_;
  if (nchunk) *nchunk = nc;
  return 0;
}

int tqr_tile_hqr_dag_check(int m, int n, int nb, int ib, int grp, int nrhs, long long *ntasks) {
  TreeShape sh;
  if (!tree_dag_shape(m, n, nb, ib, nrhs, &sh, grp)) return -1;
  std::shared_ptr<TreePlan> p = tree_plan(sh);
  for (size_t q = 0; q < p->items.size(); ++q) {
    const TItem &it = p->items[q];
    for (int d = 0; d < (int)it.ndep; ++d)
      if (p->deps[it.dep + d] >= q) return 1;
  }
  if (ntasks) *ntasks = (long long)p->items.size();
  return 0;
}

int tqr_tile_tree_dag_status(const void *work, int *error, int *item, cudaStream_t stream) {
  if (!work || !error || !item) return -1;
  int h[3];
  cudaError_t e = cudaMemcpyAsync(h, work, sizeof(h), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return (int)e;
  *error = h[1];
  *item = h[2];
  return 0;
}

int tqr_dtile_geqrf_tree_dag(int m, int n, int nb, int ib, double *A, int lda, double *T, double *T2, int ldt,
                             double *tau, double *tau2, int ldtau, int nrhs, double *B, int ldb, void *work,
                             size_t lwork, cudaStream_t stream) {
  return tree_geqrf_dag_impl<double>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, work,
                                     lwork, stream);
}

int tqr_stile_geqrf_tree_dag(int m, int n, int nb, int ib, float *A, int lda, float *T, float *T2, int ldt,
                             float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb, void *work,
                             size_t lwork, cudaStream_t stream) {
  return tree_geqrf_dag_impl<float>(m, n, nb, ib, A, lda, T, T2, ldt, tau, tau2, ldtau, nrhs, B, ldb, work,
                                    lwork, stream);
}

}  // extern "C"
