// apply_dev.cuh -- one CTA applies a block reflector to one strip.
//
// Shared by the stand-alone apply kernel (apply.cu) and the persistent tile
// DAG kernel (dag.cu).  Covers NextLA's larfb!, unmqr! (src/larfb.jl:37-142,
// src/unmqr.jl:52-149) and tsmqr!/parfb!/pamm! with l = 0
// (src/tsmqr.jl:47-146, src/parfb.jl:121-189, src/pamm.jl:104-128,306-325):
//
//   mode 0 (larfb/unmqr): the reflectors live in C's own rows; block b at row
//          i uses V1 = unit-lower V[i:i+kb, i:i+kb] over C rows [i, i+kb) and
//          V2 = V[i+kb:L, i:i+kb] over C rows [i+kb, L).
//   mode 1 (tsmqr): V1 = I over a separate A1 (rows [i, i+kb)), V2 = V[0:L, i:i+kb]
//          over all L rows of A2.
//
// For every block, in the reference's order:  W = A1/C1 rows + V^H C2,
// W = op(T) W, A1/C1 rows -= W, C2 -= V W.  Right-side applies run the same
// code on the conjugate-transposed view (row stride ld, column stride 1):
// C op(Q) is (op(Q)^H C^H)^H, which swaps the strides and whether T is
// conjugate-transposed and, for complex elements, conjugates C (and A1) on
// the way in and out (conj_c).  Element types as in panel_dev.cuh; for
// complex ones op(T) is T or T^H and 'T' means 'C' (src/tsmqr.jl:20).
//
// GB300 mapping: FP64 runs at ~7.9 GFLOP/s per SM through the SIMT DFMA pipe
// (the FP64 MMA path is slower on sm_103a) and every FP64 warp instruction
// occupies an SM sub-partition's pipe for ~64 cycles, whatever its active or
// predicated lanes.  So the strip width NW is a compile-time constant (no
// predicated-off FMAs in the inner loops), the strip, V block and T block sit
// in shared memory, and each thread carries independent FMA chains; loads and
// index arithmetic hide between DFMAs.  Global reads go through L2
// (ld.global.cg): in the persistent kernel other SMs write the same tiles
// between tasks, and L1 is not coherent with them.
#pragma once
#include <type_traits>

#include "common.cuh"

namespace tqr {

template <typename R>
struct ApplyArgs {
  int conj_c = 0;  // complex elements, right side: the view holds conj(C), conj(A1)
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
  int nw;        // strip width (the template argument of apply_strip)
  int stage_c, stage_v, stage_t;
  int tt = -1;   // mode 1 only, >= 0: reflector q of V (q = 0..k-1) holds rows
                 // [0, tt + q] only (ttmqr!/parfb! with a triangular part,
                 // src/ttmqr.jl:60-90, src/pamm.jl:104-127); rows below are
                 // never read and region rows past tt + q are not touched
};

// Phase 2 keeps op(T) W in registers (up to kW2Regs entries per thread) and
// only needs a second W buffer beyond that.
constexpr int kW2Regs = 4;

__host__ __device__ inline bool apply_w2_buffer(int ib, int nw) { return ib * nw > kW2Regs * TQR_THREADS; }

__host__ __device__ inline size_t apply_smem_elems(int L, int ib, int nw, bool sc, bool sv, bool stt) {
  size_t s = (size_t)ib * nw;
  if (apply_w2_buffer(ib, nw)) s += (size_t)ib * nw;
  if (stt) s += (size_t)ib * ib;
  if (sc) s += (size_t)odd_ld(L) * nw;
  if (sv) s += (size_t)odd_ld(L) * ib;
  return s;
}

// acc[c] += v * w[c], c < NW, reading w (16-byte aligned) in 16-byte pieces
// for FP64 / FP32 elements; the FMAs are the scalar loop's, in its order.
template <typename R, int NW>
__device__ __forceinline__ void wrow_mad(R v, const R *w, R (&acc)[NW]) {
  if constexpr (std::is_same<R, double>::value && NW % 2 == 0) {
#pragma unroll
    for (int c = 0; c < NW; c += 2) {
      const double2 x = *reinterpret_cast<const double2 *>(w + c);
      acc[c] = mad(v, x.x, acc[c]);
      acc[c + 1] = mad(v, x.y, acc[c + 1]);
    }
  } else if constexpr (std::is_same<R, float>::value && NW % 4 == 0) {
#pragma unroll
    for (int c = 0; c < NW; c += 4) {
      const float4 x = *reinterpret_cast<const float4 *>(w + c);
      acc[c] = mad(v, x.x, acc[c]);
      acc[c + 1] = mad(v, x.y, acc[c + 1]);
      acc[c + 2] = mad(v, x.z, acc[c + 2]);
      acc[c + 3] = mad(v, x.w, acc[c + 3]);
    }
  } else {
#pragma unroll
    for (int c = 0; c < NW; ++c) acc[c] = mad(v, w[c], acc[c]);
  }
}

// Phase 1 of a full FP32 block (256 staged rows, 32 reflectors, 16 columns)
// with register blocking: warp g takes rows [32 g, 32 g + 32), lane t a 4 x 4
// block of W (reflectors 4 (t % 8) .., columns 4 (t / 8) ..), so each shared
// load feeds four FMAs; part[g * 512 + p + 32 c] receives the row group's sum.
// Used by the tensor-core instantiation, whose one CTA per SM leaves phase 1
// bound by shared-memory load throughput.
__device__ __forceinline__ void phase1_blocked_f32(const float *Vp, int ldvp, const float *Cp, int ccs, float *part) {
  const int g = threadIdx.x >> 5, t = threadIdx.x & 31;
  const int p0 = 4 * (t & 7), c0 = 4 * (t >> 3);
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int w = 0; w < 4; ++w) acc[u][w] = 0.0f;
  const float *v0 = Vp + (size_t)p0 * ldvp, *cp0 = Cp + (size_t)c0 * ccs;
#pragma unroll 4
  for (int rr = 32 * g; rr < 32 * g + 32; ++rr) {
    float v[4], c[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      v[u] = v0[rr + (size_t)u * ldvp];
      c[u] = cp0[rr + (size_t)u * ccs];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int w = 0; w < 4; ++w) acc[u][w] = fmaf(v[u], c[w], acc[u][w]);
  }
  float *pg = part + (size_t)g * 512;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int w = 0; w < 4; ++w) pg[(p0 + u) + 32 * (c0 + w)] = acc[u][w];
}

// Apply to the strip of columns [c0, c0 + NW) (clamped to ncols).  VEC:
// 16-byte staging of C and V for FP32 elements (kernels with registers to
// spare: the tensor-core tile kernel runs one CTA per SM).
template <typename R, int NW, bool VEC = false>
__device__ void apply_strip(const ApplyArgs<R> &a, int c0, unsigned char *smem_raw)
{
  const int tid = threadIdx.x;
  const int nwl = min(NW, a.ncols - c0);
  if (nwl <= 0) return;
  const int L = a.L, ib = a.ib;
  const int ldw = ib;
  const int ldcs = odd_ld(L), ldvs = odd_ld(L);
  const bool w2buf = apply_w2_buffer(ib, NW);

  R *Ws = reinterpret_cast<R *>(smem_raw);                 // ib x NW
  R *W2 = Ws + (w2buf ? (size_t)ib * NW : 0);              // ib x NW (only if w2buf)
  R *Ts = W2 + (size_t)ib * NW;                            // ib x ib (if staged)
  if (!w2buf) Ts = Ws + (size_t)ib * NW;
  R *Cs = Ts + (a.stage_t ? (size_t)ib * ib : 0);          // ldcs x NW (if staged)
  R *Vs = Cs + (a.stage_c ? (size_t)ldcs * NW : 0);        // ldvs x ib (if staged)

  // C strip: element (r, c) of the strip at Cp[r * crs + c * ccs]
  R *const Cg = a.C + (size_t)c0 * a.c_cs;
  R *Cp;
  int crs, ccs;
  const bool cjc = a.conj_c != 0;
  if (a.stage_c) {
    Cp = Cs; crs = 1; ccs = ldcs;
    if (VEC && a.c_rs == 1 && cols16_ok(Cg, (size_t)a.c_cs, L)) {
      stage_cols16_f32(Cg, (size_t)a.c_cs, L, nwl, Cs, ldcs, cjc);
    } else if (a.c_rs == 1) {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int r = idx % L, c = idx / L;
        Cs[r + (size_t)c * ldcs] = conj_if(ldg_cg(Cg + (size_t)r + (size_t)c * a.c_cs), cjc);
      }
    } else {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int c = idx % nwl, r = idx / nwl;
        Cs[r + (size_t)c * ldcs] = conj_if(ldg_cg(Cg + (size_t)r * a.c_rs + c), cjc);
      }
    }
  } else {
    Cp = Cg; crs = a.c_rs; ccs = a.c_cs;
  }
  R *const A1g = (a.mode == 1) ? a.A1 + (size_t)c0 * a.a_cs : nullptr;
  const bool cjg = cjc && !a.stage_c;          // C read and written in global memory

  const int nblk = (a.k + ib - 1) / ib;
  for (int b = 0; b < nblk; ++b) {
    const int i = a.fwd ? b * ib : (nblk - 1 - b) * ib;
    const int kb = min(ib, a.k - i);
    const int r0 = (a.mode == 0) ? i : 0;       // first region row this block touches
    const bool ttb = (a.mode == 1 && a.tt >= 0);
    const int Lr = ttb ? min(L, a.tt + i + kb) : L - r0;
    auto vrows = [&](int p) { return ttb ? min(Lr, a.tt + i + p + 1) : Lr; };   // valid rows of column p
    // V block: element (rr, p) = reflector i+p at region row r0+rr
    const R *Vp;
    int ldvp;
    if (VEC && a.stage_v && a.mode == 1 && !ttb && cols16_ok(a.V + ix(0, i, a.ldv), (size_t)a.ldv, Lr)) {
      // every row of every reflector is stored: a plain column-block copy
      stage_cols16_f32(a.V + ix(0, i, a.ldv), (size_t)a.ldv, Lr, kb, Vs, ldvs, false);
      Vp = Vs; ldvp = ldvs;
    } else if (a.stage_v) {
      for (int idx = tid; idx < Lr * kb; idx += TQR_THREADS) {
        int rr = idx % Lr, p = idx / Lr;
        R v;
        if (a.mode == 0)
          v = (rr < p) ? R(0) : (rr == p ? R(1) : ldg_cg(a.V + ix(r0 + rr, i + p, a.ldv)));
        else
          v = (rr < vrows(p)) ? ldg_cg(a.V + ix(rr, i + p, a.ldv)) : R(0);
        Vs[rr + (size_t)p * ldvs] = v;
      }
      Vp = Vs; ldvp = ldvs;
    } else {
      Vp = a.V + ix(r0, i, a.ldv); ldvp = a.ldv;
    }
    const R *Tp;
    int ldtp;
    // Staged T is column-major for op(T) = T and row-major for op(T) = T^H:
    // phase 2 then reads, for fixed q, entries that are consecutive across the
    // lanes (p), free of shared-memory bank conflicts.
    if (a.stage_t) {
      for (int idx = tid; idx < kb * kb; idx += TQR_THREADS) {
        int p = idx % kb, q = idx / kb;
        const R t = (p <= q) ? ldg_cg(a.T + ix(p, i + q, a.ldt)) : R(0);
        if (a.transT) Ts[q + p * ib] = t;
        else Ts[p + q * ib] = t;
      }
      Tp = Ts; ldtp = ib;
    } else {
      Tp = a.T + ix(0, i, a.ldt); ldtp = a.ldt;
    }
    __syncthreads();

    // Phase 1: W[p, c] = (A1 or C1 row) + sum_rr conj(V[rr, p]) * C[r0 + rr, c]
    // (mode 0 needs the unit-lower test only when V is read from global).
    // Entries e and e + TQR_THREADS have the same p when kb divides
    // TQR_THREADS: one pass computes both, reading V's column once and
    // running four independent FMA chains; each entry keeps its own two-chain
    // summation order, so the result does not depend on the pairing.
    const bool vtri = (a.mode == 0) && !a.stage_v;
    const bool vtt = ttb && !a.stage_v;          // unstaged TT V: bound each column's rows
    const int ne1 = kb * nwl;
    const bool pair = (TQR_THREADS % kb) == 0;
    auto finish_w = [&](int p, int c, R w) {
      if (a.mode == 1) w += conj_if(ldg_cg(A1g + (size_t)(i + p) * a.a_rs + (size_t)c * a.a_cs), cjc);
      Ws[p + c * ldw] = w;
    };
    bool blocked = false;
    if constexpr (VEC && std::is_same<R, float>::value && NW == 16) {
      // tensor-core instantiation: 16 x 32 W of a full 256-row block through
      // 4 x 4 register blocks; the eight row-group sums are added in order
      if (a.mode == 1 && !ttb && kb == 32 && nwl == 16 && Lr == 256 && a.stage_v && a.stage_c && !cjg) {
        float *part = Vs + (size_t)ldvs * ib;     // 8 x 512 partial sums after the staged V
        phase1_blocked_f32(Vp, ldvp, Cp, ccs, part);
        __syncthreads();
        for (int e = tid; e < 512; e += TQR_THREADS) {
          float w = 0.0f;
#pragma unroll
          for (int g = 0; g < 8; ++g) w += part[g * 512 + e];
          finish_w(e % 32, e / 32, w);
        }
        blocked = true;
      }
    }
    for (int e = blocked ? ne1 : tid; e < ne1; e += (pair ? 2 : 1) * TQR_THREADS) {
      const int p = e % kb, c = e / kb;
      const R *vcol = Vp + (size_t)p * ldvp;
      const R *ccol = Cp + (size_t)r0 * crs + (size_t)c * ccs;
      const int Lp = vtt ? vrows(p) : Lr;
      int rr = vtri ? p : 0;
      if (pair && e + TQR_THREADS < ne1) {
        const int c2 = (e + TQR_THREADS) / kb;
        const R *ccol2 = Cp + (size_t)r0 * crs + (size_t)c2 * ccs;
        R acc0 = 0, acc1 = 0, bcc0 = 0, bcc1 = 0;
        if (vtri) {
          acc0 = conj_if(ccol[(size_t)p * crs], cjg);
          bcc0 = conj_if(ccol2[(size_t)p * crs], cjg);
          ++rr;
        }
        for (; rr + 1 < Lp; rr += 2) {
          const R v0 = vcol[rr], v1 = vcol[rr + 1];
          acc0 = madc(v0, conj_if(ccol[(size_t)rr * crs], cjg), acc0);
          acc1 = madc(v1, conj_if(ccol[(size_t)(rr + 1) * crs], cjg), acc1);
          bcc0 = madc(v0, conj_if(ccol2[(size_t)rr * crs], cjg), bcc0);
          bcc1 = madc(v1, conj_if(ccol2[(size_t)(rr + 1) * crs], cjg), bcc1);
        }
        if (rr < Lp) {
          const R v0 = vcol[rr];
          acc0 = madc(v0, conj_if(ccol[(size_t)rr * crs], cjg), acc0);
          bcc0 = madc(v0, conj_if(ccol2[(size_t)rr * crs], cjg), bcc0);
        }
        finish_w(p, c, acc0 + acc1);
        finish_w(p, c2, bcc0 + bcc1);
      } else {
        R acc0 = 0, acc1 = 0;
        if (vtri) { acc0 = conj_if(ccol[(size_t)p * crs], cjg); ++rr; }
        for (; rr + 1 < Lp; rr += 2) {
          acc0 = madc(vcol[rr], conj_if(ccol[(size_t)rr * crs], cjg), acc0);
          acc1 = madc(vcol[rr + 1], conj_if(ccol[(size_t)(rr + 1) * crs], cjg), acc1);
        }
        if (rr < Lp) acc0 = madc(vcol[rr], conj_if(ccol[(size_t)rr * crs], cjg), acc0);
        finish_w(p, c, acc0 + acc1);
      }
    }
    __syncthreads();
    // Phase 2: W := op(T) W, T upper triangular kb-by-kb, op(T) = T^H when
    // transT (two partial sums per entry to halve the dependent FMA chain)
    auto t_entry = [&](int e) -> R {
      const int p = e % kb, c = e / kb;
      const R *wc = Ws + c * ldw;
      R s0 = 0, s1 = 0;
      if (a.transT) {
        // T(q, p): row-major when staged, column-major in global memory
        const size_t rs = a.stage_t ? (size_t)ib : 1, cs = a.stage_t ? 1 : (size_t)ldtp;
        int q = 0;
        for (; q + 1 <= p; q += 2) {
          s0 = madc(Tp[q * rs + p * cs], wc[q], s0);
          s1 = madc(Tp[(q + 1) * rs + p * cs], wc[q + 1], s1);
        }
        if (q <= p) s0 = madc(Tp[q * rs + p * cs], wc[q], s0);
      } else {
        int q = p;
        for (; q + 1 < kb; q += 2) {
          s0 = mad(Tp[p + (size_t)q * ldtp], wc[q], s0);
          s1 = mad(Tp[p + (size_t)(q + 1) * ldtp], wc[q + 1], s1);
        }
        if (q < kb) s0 = mad(Tp[p + (size_t)q * ldtp], wc[q], s0);
      }
      return s0 + s1;
    };
    // op(T) W is written back transposed, W^T[c, p] at c + p * NW, so that
    // phase 3 reads the NW entries of one p contiguously
    const int ne = kb * nwl;
    if (w2buf) {
      for (int e = tid; e < ne; e += TQR_THREADS) W2[(e / kb) + (e % kb) * NW] = t_entry(e);
      __syncthreads();
    } else {
      R reg[kW2Regs];
#pragma unroll
      for (int u = 0; u < kW2Regs; ++u) {
        const int e = tid + u * TQR_THREADS;
        if (e < ne) reg[u] = t_entry(e);
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < kW2Regs; ++u) {
        const int e = tid + u * TQR_THREADS;
        if (e < ne) Ws[(e / kb) + (e % kb) * NW] = reg[u];
      }
      __syncthreads();
    }
    const R *Wf = w2buf ? W2 : Ws;     // W^T: entry (p, c) at c + p * NW
    // Phase 3: C[r0 + rr, c] -= sum_p V[rr, p] W[p, c];  mode 1: A1 rows -= W
    // (through the conjugated view when conj_c)
    if (a.mode == 1) {
      for (int e = tid; e < ne; e += TQR_THREADS) {
        const int p = e % kb, c = e / kb;
        R *dst = A1g + (size_t)(i + p) * a.a_rs + (size_t)c * a.a_cs;
        *dst = ldg_cg(dst) - conj_if(Wf[c + p * NW], cjc);
      }
    }
    if (nwl == NW) {
      // 16-byte loads of W^T rows where the element type and alignment allow
      const bool wvec = ((uintptr_t)Wf & 15) == 0;
      for (int rr = tid; rr < Lr; rr += TQR_THREADS) {
        R acc[NW];
#pragma unroll
        for (int c = 0; c < NW; ++c) acc[c] = 0;
        const int pmax = vtri ? min(kb, rr + 1) : kb;
        const int pmin = vtt ? max(0, rr - a.tt - i) : 0;
        for (int p = pmin; p < pmax; ++p) {
          R v = Vp[rr + (size_t)p * ldvp];
          if (vtri && p == rr) v = R(1);
          const R *wrow = Wf + (size_t)p * NW;
          if (wvec) {
            wrow_mad<R, NW>(v, wrow, acc);
          } else {
#pragma unroll
            for (int c = 0; c < NW; ++c) acc[c] = mad(v, wrow[c], acc[c]);
          }
        }
        R *crow = Cp + (size_t)(r0 + rr) * crs;
#pragma unroll
        for (int c = 0; c < NW; ++c) crow[(size_t)c * ccs] -= conj_if(acc[c], cjg);
      }
    } else {
      for (int rr = tid; rr < Lr; rr += TQR_THREADS) {
        R acc[NW];
#pragma unroll
        for (int c = 0; c < NW; ++c) acc[c] = 0;
        const int pmax = vtri ? min(kb, rr + 1) : kb;
        const int pmin = vtt ? max(0, rr - a.tt - i) : 0;
        for (int p = pmin; p < pmax; ++p) {
          R v = Vp[rr + (size_t)p * ldvp];
          if (vtri && p == rr) v = R(1);
          const R *wrow = Wf + (size_t)p * NW;
#pragma unroll
          for (int c = 0; c < NW; ++c)
            if (c < nwl) acc[c] = mad(v, wrow[c], acc[c]);
        }
        R *crow = Cp + (size_t)(r0 + rr) * crs;
#pragma unroll
        for (int c = 0; c < NW; ++c)
          if (c < nwl) crow[(size_t)c * ccs] -= conj_if(acc[c], cjg);
      }
    }
    __syncthreads();
  }
  if (a.stage_c) {
    if (VEC && a.c_rs == 1 && cols16_ok(Cg, (size_t)a.c_cs, L)) {
      unstage_cols16_f32(Cs, ldcs, L, nwl, Cg, (size_t)a.c_cs, cjc);
    } else if (a.c_rs == 1) {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int r = idx % L, c = idx / L;
        Cg[(size_t)r + (size_t)c * a.c_cs] = conj_if(Cs[r + (size_t)c * ldcs], cjc);
      }
    } else {
      for (int idx = tid; idx < L * nwl; idx += TQR_THREADS) {
        int c = idx % nwl, r = idx / nwl;
        Cg[(size_t)r * a.c_rs + c] = conj_if(Cs[r + (size_t)c * ldcs], cjc);
      }
    }
  }
}

}  // namespace tqr
