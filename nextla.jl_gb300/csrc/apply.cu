// apply.cu -- block-reflector application: the FP64/FP32 trailing update.
//
// One kernel covers NextLA's larfb!, unmqr! (src/larfb.jl:37-142,
// src/unmqr.jl:52-149) and tsmqr!/parfb!/pamm! with l = 0
// (src/tsmqr.jl:47-146, src/parfb.jl:121-189, src/pamm.jl:104-128,306-325):
//
//   mode 0 (larfb/unmqr): the reflectors live in C's own rows; block b at row
//          i uses V1 = unit-lower V[i:i+kb, i:i+kb] over C rows [i, i+kb) and
//          V2 = V[i+kb:L, i:i+kb] over C rows [i+kb, L).
//   mode 1 (tsmqr): V1 = I over a separate A1 (rows [i, i+kb)), V2 = V[0:L, i:i+kb]
//          over all L rows of A2.
//
// For every block, in the reference's order:  W = A1/C1 rows + V^T C2,
// W = op(T) W, A1/C1 rows -= W, C2 -= V W.  Right-side applies run the same
// code on the transposed view (row stride ld, column stride 1): C op(Q) is
// (op(Q)^T C^T)^T, which only swaps strides and whether T is transposed.
//
// GB300 mapping: FP64 throughput is ~7.9 GFLOP/s per SM (SIMT DFMA; the FP64
// MMA path is slower on sm_103a), so the kernel keeps every operand in shared
// memory (one C strip per CTA for the whole call, V and T per block) and gives
// each thread independent FMA chains; loads and index arithmetic hide in the
// issue slots between DFMAs.  A CTA owns an NW-wide strip of columns (rows for
// side R), so strips never interact and a call needs no global scratch.
#include "common.cuh"
#include "tileqr_internal.h"

namespace tqr {

template <typename R>
struct ApplyArgs {
  int mode;      // 0: larfb/unmqr, 1: tsmqr
  int L;         // rows of the region (C rows for mode 0, A2 rows for mode 1), transposed view
  int ncols;     // extent split into strips (columns of the transposed view)
  int k, ib, fwd, transT;
  R *C;          // element (r, c) at C[r * c_rs + c * c_cs]
  int c_rs, c_cs;
  R *A1;         // mode 1: element (r, c) at A1[r * a_rs + c * a_cs]
  int a_rs, a_cs;
  const R *V;    // column-major, ldv
  int ldv;
  const R *T;    // column-major, ldt; block at columns [i, i+kb)
  int ldt;
  int nw;        // strip width
  int stage_c, stage_v, stage_t;
};

template <typename R>
__global__ void __launch_bounds__(TQR_THREADS)
k_apply(const ApplyArgs<R> a)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  const int nw = a.nw;
  const int c0 = blockIdx.x * nw;
  const int nwl = min(nw, a.ncols - c0);
  if (nwl <= 0) return;
  const int L = a.L, ib = a.ib;
  const int ldw = ib;
  const int ldcs = odd_ld(L), ldvs = odd_ld(L);

  R *Ws = reinterpret_cast<R *>(smem_raw);                 // ib x nw
  R *W2 = Ws + (size_t)ib * nw;                            // ib x nw
  R *Ts = W2 + (size_t)ib * nw;                            // ib x ib (if staged)
  R *Cs = Ts + (a.stage_t ? (size_t)ib * ib : 0);          // ldcs x nw (if staged)
  R *Vs = Cs + (a.stage_c ? (size_t)ldcs * nw : 0);        // ldvs x ib (if staged)

  // C strip: element (r, c) of the strip at Cp[r * crs + c * ccs]
  R *const Cg = a.C + (size_t)c0 * a.c_cs;
  R *Cp;
  int crs, ccs;
  if (a.stage_c) {
    Cp = Cs; crs = 1; ccs = ldcs;
    if (a.c_rs == 1) {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int r = idx % L, c = idx / L;
        Cs[r + (size_t)c * ldcs] = Cg[(size_t)r + (size_t)c * a.c_cs];
      }
    } else {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int c = idx % nwl, r = idx / nwl;
        Cs[r + (size_t)c * ldcs] = Cg[(size_t)r * a.c_rs + c];
      }
    }
  } else {
    Cp = Cg; crs = a.c_rs; ccs = a.c_cs;
  }
  R *const A1g = (a.mode == 1) ? a.A1 + (size_t)c0 * a.a_cs : nullptr;

  const int nblk = (a.k + ib - 1) / ib;
  for (int b = 0; b < nblk; ++b) {
    const int i = a.fwd ? b * ib : (nblk - 1 - b) * ib;
    const int kb = min(ib, a.k - i);
    const int r0 = (a.mode == 0) ? i : 0;       // first region row this block touches
    const int Lr = L - r0;
    // V block: element (rr, p) = reflector i+p at region row r0+rr
    const R *Vp;
    int ldvp;
    if (a.stage_v) {
      __syncthreads();                            // previous block done with Vs
      for (int idx = tid; idx < Lr * kb; idx += TQR_THREADS) {
        int rr = idx % Lr, p = idx / Lr;
        R v;
        if (a.mode == 0)
          v = (rr < p) ? R(0) : (rr == p ? R(1) : a.V[ix(r0 + rr, i + p, a.ldv)]);
        else
          v = a.V[ix(rr, i + p, a.ldv)];
        Vs[rr + (size_t)p * ldvs] = v;
      }
      Vp = Vs; ldvp = ldvs;
    } else {
      Vp = a.V + ix(r0, i, a.ldv); ldvp = a.ldv;
    }
    const R *Tp;
    int ldtp;
    if (a.stage_t) {
      for (int idx = tid; idx < kb * kb; idx += TQR_THREADS) {
        int p = idx % kb, q = idx / kb;
        Ts[p + q * ib] = (p <= q) ? a.T[ix(p, i + q, a.ldt)] : R(0);
      }
      Tp = Ts; ldtp = ib;
    } else {
      Tp = a.T + ix(0, i, a.ldt); ldtp = a.ldt;
    }
    __syncthreads();

    // Phase 1: W[p, c] = (A1 or C1 row) + sum_rr V[rr, p] * C[r0 + rr, c]
    // (mode 0 needs the unit-lower test only when V is read from global).
    const bool vtri = (a.mode == 0) && !a.stage_v;
    for (int e = tid; e < kb * nwl; e += TQR_THREADS) {
      const int p = e % kb, c = e / kb;
      R acc0 = 0, acc1 = 0;
      const R *vcol = Vp + (size_t)p * ldvp;
      const R *ccol = Cp + (size_t)r0 * crs + (size_t)c * ccs;
      int rr = vtri ? p : 0;
      if (vtri) { acc0 = ccol[(size_t)p * crs]; ++rr; }
      for (; rr + 1 < Lr; rr += 2) {
        acc0 += vcol[rr] * ccol[(size_t)rr * crs];
        acc1 += vcol[rr + 1] * ccol[(size_t)(rr + 1) * crs];
      }
      if (rr < Lr) acc0 += vcol[rr] * ccol[(size_t)rr * crs];
      R w = acc0 + acc1;
      if (a.mode == 1) w += A1g[(size_t)(i + p) * a.a_rs + (size_t)c * a.a_cs];
      Ws[p + c * ldw] = w;
    }
    __syncthreads();
    // Phase 2: W := op(T) W, T upper triangular kb-by-kb
    for (int e = tid; e < kb * nwl; e += TQR_THREADS) {
      const int p = e % kb, c = e / kb;
      R acc = 0;
      if (a.transT) {
        for (int q = 0; q <= p; ++q) acc += Tp[q + (size_t)p * ldtp] * Ws[q + c * ldw];
      } else {
        for (int q = p; q < kb; ++q) acc += Tp[p + (size_t)q * ldtp] * Ws[q + c * ldw];
      }
      W2[p + c * ldw] = acc;
    }
    __syncthreads();
    // Phase 3: C[r0 + rr, c] -= sum_p V[rr, p] W[p, c];  mode 1: A1 rows -= W
    if (a.mode == 1) {
      for (int e = tid; e < kb * nwl; e += TQR_THREADS) {
        const int p = e % kb, c = e / kb;
        A1g[(size_t)(i + p) * a.a_rs + (size_t)c * a.a_cs] -= W2[p + c * ldw];
      }
    }
    for (int rr = tid; rr < Lr; rr += TQR_THREADS) {
      R acc[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) acc[c] = 0;
      const int pmax = vtri ? min(kb, rr + 1) : kb;
      for (int p = 0; p < pmax; ++p) {
        R v = Vp[rr + (size_t)p * ldvp];
        if (vtri && p == rr) v = R(1);
        const R *wrow = W2 + p;
#pragma unroll
        for (int c = 0; c < 16; ++c)
          if (c < nwl) acc[c] += v * wrow[c * ldw];
      }
      R *crow = Cp + (size_t)(r0 + rr) * crs;
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c < nwl) crow[(size_t)c * ccs] -= acc[c];
    }
    __syncthreads();
  }
  if (a.stage_c) {
    if (a.c_rs == 1) {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int r = idx % L, c = idx / L;
        Cg[(size_t)r + (size_t)c * a.c_cs] = Cs[r + (size_t)c * ldcs];
      }
    } else {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int c = idx % nwl, r = idx / nwl;
        Cg[(size_t)r * a.c_rs + c] = Cs[r + (size_t)c * ldcs];
      }
    }
  }
}

template <typename R>
static size_t apply_smem(int L, int ib, int nw, bool sc, bool sv, bool stt) {
  size_t s = 2 * (size_t)ib * nw;
  if (stt) s += (size_t)ib * ib;
  if (sc) s += (size_t)odd_ld(L) * nw;
  if (sv) s += (size_t)odd_ld(L) * ib;
  return s * sizeof(R);
}

// side: 'L' or 'R'; trans: 'N' or not.  For mode 0, C is the m-by-n matrix the
// reflectors of V (rows = order of Q) act on; for mode 1, C is A2 and A1 is
// the separate triangular/rectangular part.
template <typename R>
cudaError_t launch_apply(int mode, char side, char trans, int m, int n, int k, int ib,
                         R *C, int ldc, R *A1, int lda1, const R *V, int ldv,
                         const R *T, int ldt, cudaStream_t st)
{
  ApplyArgs<R> a;
  const bool left = (side == 'L');
  a.mode = mode;
  a.k = k;
  a.ib = ib;
  a.fwd = (left && trans != 'N') || (!left && trans == 'N');
  a.transT = left ? (trans != 'N') : (trans == 'N');
  a.C = C;
  a.A1 = A1;
  a.V = V; a.ldv = ldv;
  a.T = T; a.ldt = ldt;
  if (left) { a.L = m; a.ncols = n; a.c_rs = 1; a.c_cs = ldc; a.a_rs = 1; a.a_cs = lda1; }
  else      { a.L = n; a.ncols = m; a.c_rs = ldc; a.c_cs = 1; a.a_rs = lda1; a.a_cs = 1; }
  if (a.L <= 0 || a.ncols <= 0 || k <= 0) return cudaSuccess;
  // Strip width and staging: prefer everything in shared memory with two
  // CTAs per SM, then one CTA per SM, then read V / C from global.
  const size_t half = (size_t)TQR_SMEM_MAX / 2 - 1024;
  int nw = 16;
  bool sc = true, sv = true, stt = (ib <= 64);
  size_t sm = apply_smem<R>(a.L, ib, nw, sc, sv, stt);
  if (sm > half) {
    if (apply_smem<R>(a.L, ib, 8, sc, sv, stt) <= half) nw = 8;
  }
  sm = apply_smem<R>(a.L, ib, nw, sc, sv, stt);
  if (sm > (size_t)TQR_SMEM_MAX) { sv = false; sm = apply_smem<R>(a.L, ib, nw, sc, sv, stt); }
  if (sm > (size_t)TQR_SMEM_MAX) { sc = false; sm = apply_smem<R>(a.L, ib, nw, sc, sv, stt); }
  while (sm > (size_t)TQR_SMEM_MAX && nw > 1) { nw >>= 1; sm = apply_smem<R>(a.L, ib, nw, sc, sv, stt); }
  if (sm > (size_t)TQR_SMEM_MAX) return cudaErrorInvalidValue;
  a.nw = nw;
  a.stage_c = sc; a.stage_v = sv; a.stage_t = stt;
  cudaError_t e = cudaFuncSetAttribute(k_apply<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TQR_SMEM_MAX);
  if (e != cudaSuccess) return e;
  const int grid = (a.ncols + nw - 1) / nw;
  k_apply<R><<<grid, TQR_THREADS, sm, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

template cudaError_t launch_apply<double>(int, char, char, int, int, int, int, double *, int, double *, int,
                                          const double *, int, const double *, int, cudaStream_t);
template cudaError_t launch_apply<float>(int, char, char, int, int, int, int, float *, int, float *, int,
                                         const float *, int, const float *, int, cudaStream_t);

}  // namespace tqr
