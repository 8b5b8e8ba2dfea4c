// panel_cluster.cuh -- one Householder panel factorised by a thread-block
// cluster: geqr2 with its T (NextLA src/geqr2.jl:23-105, src/larft.jl:53-124)
// or one tsqrt / ttqrt block (src/tsqrt.jl:46-126, src/ttqrt.jl:1-80).
//
// A panel's work is two passes over its rows per column (the V^H P products
// and the rank-1 update), and on GB300 one SM does FP64 at ~8 GFLOP/s: a
// 256-row panel held by one CTA is bound by that one SM.  Here C CTAs
// (C = 2, 4 or 8, one cluster) each own a contiguous slice of the rows, kept
// in their own shared memory, and combine per column through distributed
// shared memory:
//
//   (a) each CTA: partial |x|^2 of its rows (one value per warp)
//   (b) cluster barrier
//   (c) each CTA, redundantly and in the same order: sum of the C x 8
//       partials, alpha read from the CTA that owns the pivot, the
//       Householder scalars (identical in every CTA)
//   (d) x *= scale on own rows
//   (e) partial S_j = x^H P[:, j] over own rows, plus the pivot row's term
//       by the CTA that holds it
//   (f) cluster barrier
//   (g) each CTA: d_j from the C partials (fixed order, identical everywhere)
//   (h) rank-1 update of own rows; the pivot's owner updates the pivot row;
//       CTA 0 extends T
//
// Every remote read of step i happens between two cluster barriers that its
// writer cannot pass before the reader does, so one buffer of each kind is
// enough; a last cluster barrier keeps every CTA resident until no other one
// can still read its shared memory.  Both barriers run on every column,
// whatever the data, so all CTAs always execute the same barrier sequence.
// The element type E is real or complex as in panel_dev.cuh.
#pragma once
#include "panel_dev.cuh"

namespace tqr {
namespace cl {

__device__ __forceinline__ uint32_t rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// address of the same shared-memory location in CTA `r` of the cluster
__device__ __forceinline__ uint32_t map(const void *p, uint32_t r) {
  uint32_t o;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(o) : "r"(saddr(p)), "r"(r));
  return o;
}

template <typename E> __device__ __forceinline__ E ld(uint32_t a);
template <> __device__ __forceinline__ double ld<double>(uint32_t a) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
  return v;
}
template <> __device__ __forceinline__ float ld<float>(uint32_t a) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
template <> __device__ __forceinline__ cx<double> ld<cx<double>>(uint32_t a) {
  double x, y;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "r"(a) : "memory");
  return cx<double>(x, y);
}
template <> __device__ __forceinline__ cx<float> ld<cx<float>>(uint32_t a) {
  float x, y;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(x), "=f"(y) : "r"(a) : "memory");
  return cx<float>(x, y);
}

}  // namespace cl

template <typename E>
struct ClusterPanelArgs {
  int form;        // 0: geqr2 (+T) of the m-by-nc panel A; 1: one tsqrt / ttqrt block
  int m, nc;       // rows of A (the x region for form 1), columns
  E *A; int lda;   // form 0: the panel; form 1: A2's block columns
  E *A1; int lda1; // form 1: the nc-by-nc upper triangle of A1 (pivot rows)
  E *T; int ldt;   // form 0: T (nc-by-nc upper) or nullptr; form 1: the T block
  E *tau;
  int tt;          // form 1, >= 0: ttqrt block, column c of A2 holds rows [0, tt + c]
};

// Rows of A each CTA holds for a cluster of C.
__host__ __device__ inline int cluster_rows(int m, int C) { return (m + C - 1) / C; }

template <typename E>
__host__ __device__ inline size_t cluster_panel_smem(int m, int nc, int C) {
  const int rc = cluster_rows(m, C);
  size_t s = rnd16(sizeof(E) * (size_t)odd_ld(rc) * nc);          // own rows
  s += rnd16(sizeof(real_t<E>) * TQR_WARPS);                       // |x|^2 partials
  s += rnd16(sizeof(E) * TQR_THREADS);                             // row-group partials
  s += 2 * rnd16(sizeof(E) * nc);                                  // pd, d
  s += rnd16(sizeof(E) * 4);                                       // scalars
  s += 2 * rnd16(sizeof(E) * (size_t)odd_ld(nc) * nc);             // T, A1 triangle (CTA 0)
  return s;
}

template <typename E>
__device__ void cluster_panel(const ClusterPanelArgs<E> &a, int C, unsigned char *smem_raw) {
  using S = real_t<E>;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cr = (int)cl::rank();
  const int m = a.m, nc = a.nc, form = a.form, tt = a.tt;
  const bool tri = form == 1 && tt >= 0;
  const int mrow = tri ? min(m, tt + nc) : m;                      // rows the panel touches
  const int rc = cluster_rows(mrow, C);
  const int r0 = min(mrow, cr * rc), r1 = min(mrow, r0 + rc);      // own rows [r0, r1)
  const int ldp = odd_ld(rc), ldn = odd_ld(nc);
  unsigned char *sp = smem_raw;
  E *P = carve<E>(sp, (size_t)ldp * nc);
  S *wpart = carve<S>(sp, TQR_WARPS);
  E *gpart = carve<E>(sp, TQR_THREADS);
  E *pd = carve<E>(sp, nc);
  E *d = carve<E>(sp, nc);
  E *scal = carve<E>(sp, 4);
  E *Ts = carve<E>(sp, (size_t)ldn * nc);
  E *B = carve<E>(sp, (size_t)ldn * nc);
  const bool buildT = form == 1 || a.T != nullptr;
  auto in_tri = [&](int r, int c) { return !tri || r <= tt + c; };
  // stage own rows, CTA 0 also the pivot triangle and the T block
  for (int idx = tid; idx < (r1 - r0) * nc; idx += TQR_THREADS) {
    const int rr = idx % (r1 - r0), c = idx / (r1 - r0);
    P[rr + (size_t)c * ldp] = in_tri(r0 + rr, c) ? ldg_cg(a.A + ix(r0 + rr, c, a.lda)) : E(0);
  }
  if (cr == 0 && form == 1) {
    for (int idx = tid; idx < nc * nc; idx += TQR_THREADS) {
      const int r = idx % nc, c = idx / nc;
      if (r <= c) {
        B[r + (size_t)c * ldn] = ldg_cg(a.A1 + ix(r, c, a.lda1));
        Ts[r + (size_t)c * ldn] = ldg_cg(a.T + ix(r, c, a.ldt));    // skipped columns keep T
      }
    }
  }
  __syncthreads();
  const int kcols = form == 0 ? min(m, nc) : nc;
  for (int i = 0; i < kcols; ++i) {
    // x rows of column i: [xlo, xhi); the pivot is row i of the panel (form 0,
    // held by CTA `own`) or row i of the A1 triangle (form 1, CTA 0)
    const int xlo = form == 0 ? i + 1 : 0;
    const int xhi = form == 0 ? m : (tri ? min(m, tt + i + 1) : m);
    const int own = form == 0 ? i / rc : 0;
    const int lo = max(xlo, r0), hi = min(xhi, r1);
    // (a)
    S s = 0;
    for (int r = lo + tid; r < hi; r += TQR_THREADS) s = abs2_add(P[(r - r0) + (size_t)i * ldp], s);
    s = warp_sum(s);
    if (lane == 0) wpart[warp] = s;
    cl::sync();                                                       // (b)
    // (c)
    if (warp == 0) {
      S t = 0;
      for (int q = lane; q < C * TQR_WARPS; q += 32) t += cl::ld<S>(cl::map(&wpart[q % TQR_WARPS], q / TQR_WARPS));
      t = warp_sum(t);
      if (lane == 0) {
        const E alpha = form == 0 ? cl::ld<E>(cl::map(&P[(i - own * rc) + (size_t)i * ldp], own))
                                  : cl::ld<E>(cl::map(&B[i + (size_t)i * ldn], 0));
        E beta, tv, sc;
        const bool ok = !(form == 0 && m - i <= 1) && householder(alpha, t, beta, tv, sc);   // geqr2.jl:32-35
        if (ok) {
          scal[0] = beta; scal[1] = tv; scal[2] = sc; scal[3] = E(1);
        } else {
          scal[3] = E(0);
        }
      }
    }
    __syncthreads();
    const bool skip = scal[3] == E(0);
    const E tv = scal[1];
    const int jlo = buildT ? 0 : i + 1;
    const int nj = nc - jlo;
    if (!skip) {
      // (d)
      const E sc = scal[2];
      for (int r = lo + tid; r < hi; r += TQR_THREADS) P[(r - r0) + (size_t)i * ldp] *= sc;
      __syncthreads();
      // (e) partial S_j over own x rows (ttqrt: column j < i holds rows <= tt + j)
      if (nj > 0) {
        const int G = TQR_THREADS / nj;
        const int j = jlo + tid % nj, g = tid / nj;
        if (g < G) {
          E acc0 = 0, acc1 = 0;
          if (j != i) {
            const int hij = (tri && j < i) ? min(hi, tt + j + 1) : hi;
            const E *pc = P + (size_t)j * ldp;
            const E *xc = P + (size_t)i * ldp;
            int r = lo + g;
            for (; r + G < hij; r += 2 * G) {
              acc0 = madc(xc[r - r0], pc[r - r0], acc0);
              acc1 = madc(xc[r + G - r0], pc[r + G - r0], acc1);
            }
            if (r < hij) acc0 = madc(xc[r - r0], pc[r - r0], acc0);
          }
          gpart[g * nj + (j - jlo)] = acc0 + acc1;
        }
        __syncthreads();
        if (tid < nj) {
          const int jj = jlo + tid;
          E acc = 0;
          for (int gg = 0; gg < G; ++gg) acc += gpart[gg * nj + tid];
          // the pivot row's term (v_i = 1 there): geqr2 keeps it for j < i too
          // (row i of column j < i is part of v_j), tsqrt only for j > i
          if (cr == own && (jj > i || (form == 0 && jj < i)))
            acc += form == 0 ? P[(i - r0) + (size_t)jj * ldp] : B[i + (size_t)jj * ldn];
          pd[jj] = acc;
        }
      }
    }
    cl::sync();                                                       // (f)
    if (!skip) {
      // (g) d_j = -conj(tau) S_j (j > i), -tau conj(S_j) (j < i)
      if (tid < nj) {
        const int jj = jlo + tid;
        if (jj != i) {
          E acc = 0;
          for (int c = 0; c < C; ++c) acc += cl::ld<E>(cl::map(&pd[jj], c));
          d[jj] = jj > i ? -(conj_(tv) * acc) : -(tv * conj_(acc));
        }
      }
      __syncthreads();
      // (h)
      const int ncol = nc - i - 1, rows = hi - lo;
      if (rows > 0)
        for (int idx = tid; idx < ncol * rows; idx += TQR_THREADS) {
          const int rr = lo - r0 + idx % rows, j = i + 1 + idx / rows;
          P[rr + (size_t)j * ldp] = mad(P[rr + (size_t)i * ldp], d[j], P[rr + (size_t)j * ldp]);
        }
      if (cr == own) {
        E *row = form == 0 ? P + (i - r0) : B + i;
        const int rs = form == 0 ? ldp : ldn;
        for (int j = i + 1 + tid; j < nc; j += TQR_THREADS) row[(size_t)j * rs] += d[j];
        if (tid == 0) row[(size_t)i * rs] = scal[0];
      }
      if (cr == 0) {
        if (buildT) {
          for (int p = tid; p < i; p += TQR_THREADS) {
            E acc = 0;
            for (int q = p; q < i; ++q) acc = mad(Ts[p + (size_t)q * ldn], d[q], acc);
            Ts[p + (size_t)i * ldn] = acc;
          }
          if (tid == 0) Ts[i + (size_t)i * ldn] = tv;
        }
        if (tid == 0) a.tau[i] = tv;
      }
    } else if (cr == 0) {
      if (tid == 0) a.tau[i] = E(0);
      if (form == 0 && buildT)                                      // larft: a tau = 0 column of T is zero
        for (int p = tid; p <= i; p += TQR_THREADS) Ts[p + (size_t)i * ldn] = E(0);
    }
    __syncthreads();
  }
  cl::sync();   // no CTA may leave while another can still read its shared memory
  for (int idx = tid; idx < (r1 - r0) * nc; idx += TQR_THREADS) {
    const int rr = idx % (r1 - r0), c = idx / (r1 - r0);
    if (in_tri(r0 + rr, c)) a.A[ix(r0 + rr, c, a.lda)] = P[rr + (size_t)c * ldp];
  }
  if (cr == 0) {
    const int kt = form == 0 ? kcols : nc;
    for (int idx = tid; idx < kt * kt; idx += TQR_THREADS) {
      const int p = idx % kt, q = idx / kt;
      if (p <= q) {
        if (buildT) a.T[ix(p, q, a.ldt)] = Ts[p + (size_t)q * ldn];
        if (form == 1) a.A1[ix(p, q, a.lda1)] = B[p + (size_t)q * ldn];
      }
    }
  }
}

}  // namespace tqr
