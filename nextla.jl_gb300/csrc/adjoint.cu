// adjoint.cu -- batched thin QR with explicit Q and its adjoint (backward).
//
// NextLA has no derivative rules; this is the differentiable form of its tile
// QR for a batch of equal-shape problems (m-by-n, m >= n, n <= 256).  Each
// problem is factored by one CTA as a flat-tree tile QR over 256-row tiles:
// geqrt! on the top tile (src/geqrt.jl:22-68), then tsqrt! of the top triangle
// against every further tile (src/tsqrt.jl:46-126), each ib-block followed by
// its trailing update (unmqr!/tsmqr! arithmetic, src/unmqr.jl:52-149,
// src/tsmqr.jl:46-98).  The device routines are the same ones the persistent
// tile kernel runs.
//
// Forward:  F := packed factor (R on and above the diagonal of the top tile,
//           V below it and in the lower tiles), tau, Q (explicit, m-by-n) and
//           R (n-by-n, zero below the diagonal).  T factors live only in
//           per-CTA scratch while Q is formed.
// Backward: given the saved F and tau and cotangents Qbar, Rbar:
//           T of every block is recomputed from V and tau (the larft!
//           recursion, src/larft.jl:53-86), then the thin-QR adjoint
//             M    = R Rbar^T - Qbar^T Q
//             Abar = (Qbar + Q copyltu(M)) R^-T,   copyltu(M) = tril(M) + tril(M,-1)^T
//           (Walter & Lehmann 2018; Liao, Liu, Wang & Xiang 2019), with
//           Q^T Qbar and Q copyltu(M) applied through the block reflectors
//           and R^-T by an in-place triangular solve.  The formula holds for
//           any diagonal sign convention of R as long as Q and R agree.
// Complex elements (ComplexF64, ComplexF32), gradients in the convention
// Abar = dL/dRe(A) + i dL/dIm(A) for a real loss L (torch's): transposes
// become conjugate transposes, M = R Rbar^H - Qbar^H Q and
//             Abar = (Qbar + Q X) R^-H,   X = tril(M,-1) + tril(M,-1)^H + Re diag(M).
// The real part of M's diagonal alone enters because R's diagonal is real
// (the Householder beta): Q^H dQ is skew-Hermitian with the purely imaginary
// diagonal i Im diag(Q^H dA R^-1), which the Re-diagonal term is the adjoint
// of.  That needs a reflector below every column, m > n (for m == n the last
// column keeps tau = 0 and a complex R_nn, src/geqr2.jl:32-35); the complex
// backward rejects m == n.  Checked against central differences in the real
// and the imaginary direction of every entry.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

#include "apply_dev.cuh"
#include "panel_dev.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

constexpr int kAdjNb = 256;                 // tile rows
constexpr int kAdjNW = 16;                  // trailing-update strip width (8 for ComplexF64)
constexpr int kAdjMaxIb = 32;
constexpr size_t kAdjSmem = 110976;         // two CTAs per SM (ComplexF64: one, adj_smem)

template <typename R> struct AdjNW { static constexpr int value = kAdjNW; };
template <> struct AdjNW<cx<double>> { static constexpr int value = 8; };

// Dynamic shared memory of the forward and adjoint kernels for element type R:
// the staged panel, tsqrt block and strip apply at 256 rows, ib = 32.
template <typename R>
static size_t adj_smem() {
  return std::max({kAdjSmem, panel_smem<R>(256, 32, true, true), tsqrt_smem<R>(256, 32, true),
                   apply_smem_elems(256, 32, AdjNW<R>::value, true, true, true) * sizeof(R)});
}

struct AdjGeom {
  int m, n, ib, MT;
  __host__ __device__ int rows(int t) const { return min(kAdjNb, m - t * kAdjNb); }
};

struct AdjHeader {
  int next;
  int pad[63];
};
static_assert(sizeof(AdjHeader) == 256, "AdjHeader layout");

template <typename R>
__host__ __device__ inline size_t adj_scratch_elems(const AdjGeom &g) {
  // T of every tile (ib x n each) + an n x n matrix
  return (size_t)g.MT * kAdjMaxIb * g.n + (size_t)g.n * g.n;
}

template <typename R>
struct AdjArgs {
  AdjGeom g;
  int batch;
  R *F;             // packed factors, problem p at F + p m n (lda = m)
  R *tau;           // MT n per problem: tile t's tau at t n
  R *Q;             // m x n per problem
  R *Rout;          // n x n per problem
  const R *Qbar, *Rbar;
  R *Abar;          // m x n per problem
  AdjHeader *hdr;
  R *scratch;       // adj_scratch_elems per CTA
};

// Columns [c0, ncols) of an apply, strip by strip.
template <typename R>
__device__ void apply_cols(ApplyArgs<R> a, int c0, unsigned char *smem) {
  for (int c = c0; c < a.ncols; c += AdjNW<R>::value) {
    apply_strip<R, AdjNW<R>::value>(a, c, smem);
    __syncthreads();
  }
}

template <typename R>
__device__ ApplyArgs<R> base_args(int ib) {
  ApplyArgs<R> a;
  a.ib = ib; a.fwd = 1; a.transT = 1;
  a.c_rs = 1; a.a_rs = 1;
  a.nw = AdjNW<R>::value;
  a.stage_c = 1; a.stage_v = 1; a.stage_t = 1;
  a.A1 = nullptr; a.a_cs = 1;
  return a;
}

// C (m x n, ldc = m) := Q C (trans 0) or Q^T C (trans 1) with Q from the
// factor F (tile 0's reflectors, then tile t's for t = 1..MT-1) and T.
//
// ident (trans 0 only): C holds [I; 0] on entry, so the explicit thin Q is
// being formed (LAPACK's orgqr).  Blocks are applied last to first, and
// through every step column c of the top n rows is nonzero only above the
// end of its own ib-block, while tile rows not yet reached are zero.  A block
// of reflectors starting at column i0 > c then meets W = 0 on column c and
// leaves it as it is, so each strip [c0, c0 + NW) applies only the blocks
// starting before c0 + NW: the same values, about half the work of forming Q.
template <typename R>
__device__ void apply_q(const AdjGeom &g, const R *F, const R *Tw, int trans, R *C, unsigned char *smem,
                        bool ident = false) {
  const int m = g.m, n = g.n, ib = g.ib;
  auto run = [&](ApplyArgs<R> a) {
    if (!ident) {
      apply_cols<R>(a, 0, smem);
      return;
    }
    constexpr int NW = AdjNW<R>::value;
    for (int c = 0; c < a.ncols; c += NW) {
      a.k = min(n, ((c + NW + ib - 1) / ib) * ib);
      apply_strip<R, NW>(a, c, smem);
      __syncthreads();
    }
  };
  auto tile0 = [&]() {
    ApplyArgs<R> a = base_args<R>(ib);
    a.mode = 0; a.L = g.rows(0); a.k = n; a.fwd = trans; a.transT = trans;
    a.C = C; a.c_cs = m; a.ncols = n;
    a.V = F; a.ldv = m;
    a.T = Tw; a.ldt = ib;
    run(a);
  };
  auto pair = [&](int t) {
    ApplyArgs<R> a = base_args<R>(ib);
    a.mode = 1; a.L = g.rows(t); a.k = n; a.fwd = trans; a.transT = trans;
    a.C = C + (size_t)t * kAdjNb; a.c_cs = m; a.ncols = n;
    a.A1 = C; a.a_cs = m;
    a.V = F + (size_t)t * kAdjNb; a.ldv = m;
    a.T = Tw + (size_t)t * kAdjMaxIb * n; a.ldt = ib;
    run(a);
  };
  if (trans) {
    tile0();
    for (int t = 1; t < g.MT; ++t) pair(t);
  } else {
    for (int t = g.MT - 1; t >= 1; --t) pair(t);
    tile0();
  }
}

// Flat-tree tile QR of one problem in place; T blocks to Tw (tile t's at
// Tw + t * 32 * n, ld ib), tau to tau (tile t's at tau + t * n).
template <typename R>
__device__ void factor_one(const AdjGeom &g, R *A, R *tau, R *Tw, unsigned char *smem) {
  const int m = g.m, n = g.n, ib = g.ib, lda = m;
  const int L0 = g.rows(0);
  for (int i0 = 0; i0 < n; i0 += ib) {
    const int sb = min(ib, n - i0);
    panel_qr_cta<R>(L0 - i0, sb, A + ix(i0, i0, lda), lda, tau + i0, Tw + ix(0, i0, ib), ib, true, true, smem);
    ApplyArgs<R> a = base_args<R>(sb);
    a.mode = 0; a.L = L0 - i0; a.k = sb;
    a.C = A + i0; a.c_cs = lda; a.ncols = n;
    a.V = A + ix(i0, i0, lda); a.ldv = lda;
    a.T = Tw + ix(0, i0, ib); a.ldt = ib;
    apply_cols<R>(a, i0 + sb, smem);
  }
  for (int t = 1; t < g.MT; ++t) {
    R *At = A + (size_t)t * kAdjNb;
    R *Tt = Tw + (size_t)t * kAdjMaxIb * n;
    const int Lt = g.rows(t);
    // a reflector skipped for an exactly zero column leaves its T column as
    // it was, so start from zero
    for (int idx = threadIdx.x; idx < ib * n; idx += TQR_THREADS) Tt[(idx % ib) + (size_t)(idx / ib) * ib] = R(0);
    __syncthreads();
    for (int i0 = 0; i0 < n; i0 += ib) {
      const int sb = min(ib, n - i0);
      tsqrt_block_cta<R>(Lt, sb, A + ix(i0, i0, lda), lda, At + ix(0, i0, lda), lda, Tt + ix(0, i0, ib), ib,
                         tau + (size_t)t * n + i0, true, smem);
      ApplyArgs<R> a = base_args<R>(sb);
      a.mode = 1; a.L = Lt; a.k = sb;
      a.C = At; a.c_cs = lda; a.ncols = n;
      a.A1 = A + i0; a.a_cs = lda;
      a.V = At + ix(0, i0, lda); a.ldv = lda;
      a.T = Tt + ix(0, i0, ib); a.ldt = ib;
      apply_cols<R>(a, i0 + sb, smem);
    }
  }
}

// T (sb x sb, upper, ldt) of one block of reflectors from V and tau:
// T[j,j] = tau_j, T[0:j, j] = -tau_j T[0:j, 0:j] (V[:, 0:j]^T v_j).
// unit: V is unit lower trapezoidal (geqrt form, L rows); otherwise the
// reflectors are [e_j; V[:, j]] (tsqrt form) and only V's L rows enter.
template <typename R>
__device__ void larft_block(int L, int sb, const R *V, int ldv, const R *tau, bool unit, R *T, int ldt,
                            unsigned char *smem) {
  R *G = reinterpret_cast<R *>(smem);            // sb x sb, ld 33
  R *Ts = G + 33 * kAdjMaxIb;                    // sb x sb, ld 33
  const int tid = threadIdx.x;
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int p = idx % sb, j = idx / sb;
    R s = R(0);
    if (p < j) {   // G = V^H V (complex: the left factor conjugated, src/larft.jl:71-84)
      if (unit) {
        s = conj_(V[ix(j, p, ldv)]);
        for (int r = j + 1; r < L; ++r) s = madc(V[ix(r, p, ldv)], V[ix(r, j, ldv)], s);
      } else {
        for (int r = 0; r < L; ++r) s = madc(V[ix(r, p, ldv)], V[ix(r, j, ldv)], s);
      }
    }
    G[p + 33 * j] = s;
  }
  __syncthreads();
  for (int j = 0; j < sb; ++j) {
    const R tj = tau[j];
    if (tid < j) {
      R s = R(0);
      for (int q = tid; q < j; ++q) s = mad(Ts[tid + 33 * q], G[q + 33 * j], s);
      Ts[tid + 33 * j] = -tj * s;
    } else if (tid == j) {
      Ts[j + 33 * j] = tj;
    }
    __syncthreads();
  }
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int p = idx % sb, q = idx / sb;
    T[ix(p, q, ldt)] = (p <= q) ? Ts[p + 33 * q] : R(0);
  }
  __syncthreads();
}

template <typename R>
__device__ void recompute_t(const AdjGeom &g, const R *F, const R *tau, R *Tw, unsigned char *smem) {
  const int m = g.m, n = g.n, ib = g.ib;
  for (int t = 0; t < g.MT; ++t) {
    const R *Ft = F + (size_t)t * kAdjNb;
    R *Tt = Tw + (size_t)t * kAdjMaxIb * n;
    for (int i0 = 0; i0 < n; i0 += ib) {
      const int sb = min(ib, n - i0);
      if (t == 0)
        larft_block<R>(g.rows(0) - i0, sb, Ft + ix(i0, i0, m), m, tau + i0, true, Tt + ix(0, i0, ib), ib, smem);
      else
        larft_block<R>(g.rows(t), sb, Ft + ix(0, i0, m), m, tau + (size_t)t * n + i0, false, Tt + ix(0, i0, ib),
                       ib, smem);
    }
  }
}

// X R^T = Y (complex: X R^H = Y) in place for one row tile (X overwrites Y,
// rows x n, ldy), R n x n upper (ldr): column blocks of SolveBw from the
// right; each thread owns one row and keeps the block's entries in registers.
constexpr int kSolveBw = 32;
template <typename R> struct SolveBw { static constexpr int value = sizeof(R) == 16 ? 16 : kSolveBw; };

template <typename R>
__device__ void solve_rt(int rows, int n, const R *Rm, int ldr, R *Y, int ldy, unsigned char *smem) {
  constexpr int BW = SolveBw<R>::value;
  R *Rs = reinterpret_cast<R *>(smem);          // (n - j0) x BW: Rs[(k - j0) * BW + c] = R[j0 + c, k]
  R *rinv = Rs + (size_t)kAdjNb * BW;           // BW
  const int tid = threadIdx.x;
  for (int j0 = ((n - 1) / BW) * BW; j0 >= 0; j0 -= BW) {
    const int jb = min(BW, n - j0);
    const int kn = n - j0;
    // rows kk < BW are read by the in-block sweep even past kn (a partial
    // first block, jb < BW): zero them so 0 * (stale shared memory) never
    // turns into NaN
    for (int idx = tid; idx < max(kn, BW) * BW; idx += TQR_THREADS) {
      const int kk = idx / BW, c = idx % BW;
      Rs[idx] = (kk < kn && c < jb && c <= kk) ? conj_(Rm[ix(j0 + c, j0 + kk, ldr)]) : R(0);
    }
    for (int c = tid; c < BW; c += TQR_THREADS)
      rinv[c] = (c < jb) ? div_(R(1), conj_(Rm[ix(j0 + c, j0 + c, ldr)])) : R(0);
    __syncthreads();
    for (int r = tid; r < rows; r += TQR_THREADS) {
      R acc[BW];
#pragma unroll
      for (int c = 0; c < BW; ++c) acc[c] = (c < jb) ? Y[ix(r, j0 + c, ldy)] : R(0);
      for (int kk = jb; kk < kn; ++kk) {
        const R x = Y[ix(r, j0 + kk, ldy)];
        const R *rk = Rs + (size_t)kk * BW;
#pragma unroll
        for (int c = 0; c < BW; ++c) acc[c] = mad(-x, rk[c], acc[c]);
      }
#pragma unroll
      for (int c = BW - 1; c >= 0; --c) {
        const R xc = acc[c] * rinv[c];
        acc[c] = xc;
        const R *rc = Rs + (size_t)c * BW;
#pragma unroll
        for (int c2 = 0; c2 < c; ++c2) acc[c2] = mad(-xc, rc[c2], acc[c2]);
      }
#pragma unroll
      for (int c = 0; c < BW; ++c)
        if (c < jb) Y[ix(r, j0 + c, ldy)] = acc[c];
    }
    __syncthreads();
  }
}

// Abar := Y R^-T for row tile blockIdx.x of problem blockIdx.y.
template <typename R>
__global__ void __launch_bounds__(TQR_THREADS) k_solve_rt(AdjGeom g, const R *F, R *Abar) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = blockIdx.x, p = blockIdx.y;
  const size_t off = (size_t)p * g.m * g.n;
  solve_rt<R>(g.rows(t), g.n, F + off, g.m, Abar + off + (size_t)t * kAdjNb, g.m, smem_raw);
}

template <typename R>
__device__ void forward_one(const AdjArgs<R> &a, int p, R *Tw, unsigned char *smem) {
  const AdjGeom &g = a.g;
  const int m = g.m, n = g.n;
  R *A = a.F + (size_t)p * m * n;
  R *tau = a.tau + (size_t)p * g.MT * n;
  factor_one<R>(g, A, tau, Tw, smem);
  __syncthreads();
  R *Rp = a.Rout + (size_t)p * n * n;
  R *Qp = a.Q + (size_t)p * m * n;
  for (int idx = threadIdx.x; idx < n * n; idx += TQR_THREADS) {
    const int r = idx % n, c = idx / n;
    Rp[idx] = (r <= c) ? A[ix(r, c, m)] : R(0);
  }
  for (size_t idx = threadIdx.x; idx < (size_t)m * n; idx += TQR_THREADS) {
    const int r = (int)(idx % m), c = (int)(idx / m);
    Qp[idx] = (r == c) ? R(1) : R(0);
  }
  __syncthreads();
  apply_q<R>(g, A, Tw, 0, Qp, smem, true);
}

template <typename R>
__device__ void backward_one(const AdjArgs<R> &a, int p, R *Tw, R *Ms, unsigned char *smem) {
  const AdjGeom &g = a.g;
  const int m = g.m, n = g.n;
  const R *F = a.F + (size_t)p * m * n;
  const R *tau = a.tau + (size_t)p * g.MT * n;
  const R *Qb = a.Qbar + (size_t)p * m * n;
  const R *Rb = a.Rbar + (size_t)p * n * n;
  R *W = a.Abar + (size_t)p * m * n;
  const int tid = threadIdx.x;
  recompute_t<R>(g, F, tau, Tw, smem);
  // W := Q_full^T Qbar; its first n rows are Q^T Qbar
  for (size_t idx = tid; idx < (size_t)m * n; idx += TQR_THREADS) W[idx] = Qb[idx];
  __syncthreads();
  apply_q<R>(g, F, Tw, 1, W, smem);
  // Ms (lower) = R Rbar^H - (Q^H Qbar)^H
  for (int idx = tid; idx < n * n; idx += TQR_THREADS) {
    const int i = idx % n, j = idx / n;
    if (i >= j) {
      R s = R(0);
      for (int k = i; k < n; ++k) s = mad(F[ix(i, k, m)], conj_(Rb[ix(j, k, n)]), s);
      Ms[idx] = s - conj_(W[ix(j, i, m)]);
    }
  }
  __syncthreads();
  // W := [X; 0] with X = tril(M) + tril(M,-1)^H (complex: Re diag M), then W := Q W
  for (size_t idx = tid; idx < (size_t)m * n; idx += TQR_THREADS) {
    const int r = (int)(idx % m), c = (int)(idx / m);
    R v = R(0);
    if (r < n) {
      v = (r >= c) ? Ms[r + (size_t)c * n] : conj_(Ms[c + (size_t)r * n]);
      if constexpr (is_cx<R>) {
        if (r == c) v = R(v.x);
      }
    }
    W[idx] = v;
  }
  __syncthreads();
  apply_q<R>(g, F, Tw, 0, W, smem);
  // Y = Qbar + Q copyltu(M);  Abar = Y R^-T
  for (size_t idx = tid; idx < (size_t)m * n; idx += TQR_THREADS) W[idx] += Qb[idx];
  __syncthreads();
  // Abar = Y R^-T follows in k_solve_rt
}

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS, 2) k_qr_fwd(const AdjArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_p;
  R *Tw = a.scratch + (size_t)blockIdx.x * adj_scratch_elems<R>(a.g);
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(&a.hdr->next, 1);
    __syncthreads();
    const int p = s_p;
    __syncthreads();
    if (p >= a.batch) break;
    forward_one<R>(a, p, Tw, smem_raw);
    __syncthreads();
  }
}

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS, 2) k_qr_bwd(const AdjArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_p;
  R *Tw = a.scratch + (size_t)blockIdx.x * adj_scratch_elems<R>(a.g);
  R *Ms = Tw + (size_t)a.g.MT * kAdjMaxIb * a.g.n;
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(&a.hdr->next, 1);
    __syncthreads();
    const int p = s_p;
    __syncthreads();
    if (p >= a.batch) break;
    backward_one<R>(a, p, Tw, Ms, smem_raw);
    __syncthreads();
  }
}

__global__ void k_adj_reset(AdjHeader *h) {
  if (threadIdx.x == 0) h->next = 0;
}

static std::mutex g_adj_mu;
static int g_adj_grid[4][2][64];      // [element type][fwd/bwd][device]

template <typename R> constexpr int adj_slot() {
  return std::is_same<R, double>::value ? 0 : std::is_same<R, float>::value ? 1 : std::is_same<R, cx<double>>::value ? 2 : 3;
}

template <typename R, bool FWD>
static int adj_grid(int *grid) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev >= 64) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> l(g_adj_mu);
  int &gsz = g_adj_grid[adj_slot<R>()][FWD ? 0 : 1][dev];
  if (gsz == 0) {
    int sms = 0, per = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return (int)e;
    auto kern = FWD ? k_qr_fwd<R> : k_qr_bwd<R>;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_smem<R>())) !=
        cudaSuccess)
      return (int)e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, TQR_THREADS, adj_smem<R>())) != cudaSuccess)
      return (int)e;
    gsz = sms * std::max(per, 1);
  }
  *grid = gsz;
  return 0;
}

static bool adj_geom(int m, int n, int ib, AdjGeom *g) {
  if (n < 1 || n > kAdjNb || m < n || ib < 1 || ib > kAdjMaxIb) return false;
  g->m = m; g->n = n; g->ib = ib;
  g->MT = (m + kAdjNb - 1) / kAdjNb;
  return true;
}

template <typename R>
static int adj_worksize(int m, int n, int ib, size_t *bytes, int *grid_out) {
  AdjGeom g;
  if (!adj_geom(m, n, ib, &g)) return -1;
  int gf = 0, gb = 0, rc;
  if ((rc = adj_grid<R, true>(&gf)) != 0) return rc;
  if ((rc = adj_grid<R, false>(&gb)) != 0) return rc;
  const int grid = std::max(gf, gb);
  *bytes = sizeof(AdjHeader) + sizeof(R) * adj_scratch_elems<R>(g) * (size_t)grid;
  if (grid_out) *grid_out = grid;
  return 0;
}

template <typename R, bool FWD>
static int adj_launch(int batch, int m, int n, int ib, R *F, R *tau, R *Q, R *Rout, const R *Qbar,
                      const R *Rbar, R *Abar, void *work, size_t lwork, cudaStream_t st) {
  if (batch < 0) return -1;
  AdjGeom g;
  if (n < 1 || n > kAdjNb) return -3;
  if (m < n) return -2;
  // complex adjoint: every diagonal entry of R must be real, which needs a
  // reflector below every column (m > n; with m == n the last column has one
  // row, gets tau = 0 as in src/geqr2.jl:32-35, and keeps a complex R_nn)
  if (!FWD && is_cx<R> && m == n) return -2;
  if (ib < 1 || ib > kAdjMaxIb) return -4;
  adj_geom(m, n, ib, &g);
  if (batch == 0) return 0;
  if (!F || !tau) return -5;
  if (FWD && (!Q || !Rout)) return -6;
  if (!FWD && (!Qbar || !Rbar || !Abar)) return -6;
  if (!work || ((uintptr_t)work & 255)) return -7;
  size_t need = 0;
  int grid = 0;
  int rc = adj_worksize<R>(m, n, ib, &need, &grid);
  if (rc != 0) return rc;
  if (lwork < need) return -8;
  AdjArgs<R> a;
  a.g = g; a.batch = batch; a.F = F; a.tau = tau; a.Q = Q; a.Rout = Rout;
  a.Qbar = Qbar; a.Rbar = Rbar; a.Abar = Abar;
  a.hdr = (AdjHeader *)work;
  a.scratch = (R *)((unsigned char *)work + sizeof(AdjHeader));
  k_adj_reset<<<1, 32, 0, st>>>(a.hdr);
  count_launch();
  const int gl = std::min(grid, batch);
  if (FWD) {
    k_qr_fwd<R><<<gl, TQR_THREADS, adj_smem<R>(), st>>>(a);
    count_launch();
  } else {
    k_qr_bwd<R><<<gl, TQR_THREADS, adj_smem<R>(), st>>>(a);
    count_launch();
    const size_t sm = sizeof(R) * ((size_t)kAdjNb * SolveBw<R>::value + SolveBw<R>::value);
    cudaError_t e = cudaSuccess;
    if (sm > 48 * 1024)
      e = cudaFuncSetAttribute(k_solve_rt<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return (int)e;
    k_solve_rt<R><<<dim3(g.MT, batch), TQR_THREADS, sm, st>>>(g, F, Abar);
    count_launch();
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace tqr

using namespace tqr;

extern "C" {

int tqr_qr_batched_worksize(int dtype_bytes, int m, int n, int ib, size_t *bytes) {
  if (!bytes) return -5;
  if (dtype_bytes == 8) {   // FP64 and ComplexF32 (8-byte elements)
    size_t bd = 0, bc = 0;
    int rc = adj_worksize<double>(m, n, ib, &bd, nullptr);
    if (rc == 0) rc = adj_worksize<cx<float>>(m, n, ib, &bc, nullptr);
    if (rc == 0) *bytes = std::max(bd, bc);
    return rc;
  }
  if (dtype_bytes == 4) return adj_worksize<float>(m, n, ib, bytes, nullptr);
  if (dtype_bytes == 16) return adj_worksize<cx<double>>(m, n, ib, bytes, nullptr);
  return -9;
}

#define TQR_ADJ_CX(P, CT, E)                                                                                  \
  int tqr_##P##qr_batched_fwd(int batch, int m, int n, int ib, CT *F, CT *tau, CT *Q, CT *R, void *work,       \
                              size_t lwork, cudaStream_t stream) {                                          \
    if (((uintptr_t)F | (uintptr_t)tau | (uintptr_t)Q | (uintptr_t)R) % alignof(E)) return -5;             \
    return adj_launch<E, true>(batch, m, n, ib, (E *)F, (E *)tau, (E *)Q, (E *)R, nullptr, nullptr, nullptr,  \
                               work, lwork, stream);                                                        \
  }                                                                                                         \
  int tqr_##P##qr_batched_bwd(int batch, int m, int n, int ib, const CT *F, const CT *tau, const CT *Qbar,    \
                              const CT *Rbar, CT *Abar, void *work, size_t lwork, cudaStream_t stream) {      \
    if (((uintptr_t)F | (uintptr_t)tau | (uintptr_t)Qbar | (uintptr_t)Rbar | (uintptr_t)Abar) % alignof(E))  \
      return -5;                                                                                            \
    return adj_launch<E, false>(batch, m, n, ib, (E *)F, (E *)tau, nullptr, nullptr, (const E *)Qbar,       \
                                (const E *)Rbar, (E *)Abar, work, lwork, stream);                          \
  }
TQR_ADJ_CX(z, tqr_zcomplex, cx<double>)
TQR_ADJ_CX(c, tqr_ccomplex, cx<float>)
#undef TQR_ADJ_CX

int tqr_dqr_batched_fwd(int batch, int m, int n, int ib, double *F, double *tau, double *Q, double *R,
                        void *work, size_t lwork, cudaStream_t stream) {
  return adj_launch<double, true>(batch, m, n, ib, F, tau, Q, R, nullptr, nullptr, nullptr, work, lwork, stream);
}

int tqr_sqr_batched_fwd(int batch, int m, int n, int ib, float *F, float *tau, float *Q, float *R,
                        void *work, size_t lwork, cudaStream_t stream) {
  return adj_launch<float, true>(batch, m, n, ib, F, tau, Q, R, nullptr, nullptr, nullptr, work, lwork, stream);
}

int tqr_dqr_batched_bwd(int batch, int m, int n, int ib, const double *F, const double *tau, const double *Qbar,
                        const double *Rbar, double *Abar, void *work, size_t lwork, cudaStream_t stream) {
  return adj_launch<double, false>(batch, m, n, ib, const_cast<double *>(F), const_cast<double *>(tau), nullptr,
                                   nullptr, Qbar, Rbar, Abar, work, lwork, stream);
}

int tqr_sqr_batched_bwd(int batch, int m, int n, int ib, const float *F, const float *tau, const float *Qbar,
                        const float *Rbar, float *Abar, void *work, size_t lwork, cudaStream_t stream) {
  return adj_launch<float, false>(batch, m, n, ib, const_cast<float *>(F), const_cast<float *>(tau), nullptr,
                                  nullptr, Qbar, Rbar, Abar, work, lwork, stream);
}

}  // extern "C"
