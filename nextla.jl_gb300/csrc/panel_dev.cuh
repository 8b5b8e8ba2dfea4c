// panel_dev.cuh -- Householder panel factorisation by one CTA.
//
//  panel_qr_cta     geqr2 with the larft T build fused in (NextLA src/geqr2.jl:23-105
//                   and src/larft.jl:53-86,112-124 for direct 'F', storev 'C').
//  tsqrt_block_cta  one ib-block of tsqrt: reflectors of [A1 (upper); A2] and the
//                   T block (NextLA src/tsqrt.jl:46-126).
//
// Shared by the stand-alone panel kernels (panel.cu) and the persistent tile
// DAG kernel (dag.cu).  The reference runs each as a single work-item; here
// the CTA works on every column together.  Both share one column step:
//
//   geqr2 at column i:  alpha = P[i,i], x = P[i+1:m, i], "row" = P[i, :]
//   tsqrt at column i:  alpha = A1[i,i], x = A2[0:m, i], "row" = A1[i, :]
//
//   xnorm^2 = sum |x|^2; beta, tau, scale (one thread, broadcast); x *= scale;
//   S_j = row[j] + x^H P[x rows, j] for every other column j;
//   j > i: d_j = -conj(tau) S_j, the update of H^H = I - conj(tau) v v^H
//          (row[j] += d_j, P[x rows, j] += x d_j);
//   j < i: d_j = -tau conj(S_j) = -tau v_j^H v_i, the T column's V^H v
//          (geqr2 keeps the row term there because row i of column j < i is
//          part of v_j; tsqrt drops it because the A1 part of v_j is e_j);
//   T[0:i, i] = T[0:i, 0:i] d[0:i].
// For real elements conj is the identity and both d's are -tau S_j.  The
// element type E is double, float, cx<double> or cx<float> (common.cuh); the
// complex forms follow the reference's complex branches (src/geqr2.jl:38-99,
// src/tsqrt.jl:52-122, src/larft.jl:71-84).
//
// On GB300 every FP64 warp instruction holds an SM sub-partition's FP64 pipe
// for ~64 cycles whatever its active-lane count, and sqrt/div cost ~600 cycles.
// So the step minimises dependent FP64 instructions: the dot products use one
// thread per (column, row group) combined by a single add per group (no
// shuffle trees), the Householder scalars are computed once, and the panel
// and T live in shared memory.
#pragma once
#include "common.cuh"

namespace tqr {

template <typename E>
struct ColumnStep {
  E *P;       // x region rows live here (geqr2: the panel; tsqrt: A2)
  int ldp;
  E *row;     // row i of the factored matrix: row[j * rs]
  int rs;
  E *Ts;      // T (nc-by-nc upper), ld = ldts, or nullptr
  int ldts;
  E *part;    // TQR_THREADS partial sums
  E *d;       // nc: d_j above
  E *scal;    // 4
  int tt = -1;  // >= 0: triangle-on-triangle form, column j of P holds rows
                // [0, tt + j] only (NextLA src/ttqrt.jl:9); its rows below
                // are never read
  bool round32 = false;   // FP64 panels of an FP32 matrix: each reflector and
                          // its tau are rounded to FP32 as soon as they are
                          // formed, so every later use -- the rest of the
                          // block, the T build, the FP32 updates -- applies
                          // the reflector that is stored
};

// One column step.  x rows are [x0, m) of P, column i.  Returns false when
// the reflector is the identity (tau = 0).  Contains the syncs it needs; all
// threads call it with identical arguments.
template <typename E>
__device__ bool column_step(const ColumnStep<E> &c, int i, int x0, int m, int nc, bool tsqrt_form,
                            E *tau_out, bool zero_t_on_skip)
{
  using S = real_t<E>;
  const int tid = threadIdx.x;
  E *xcol = c.P + (size_t)i * c.ldp;
  // ---- norm of x ----
  S s = 0;
  for (int r = x0 + tid; r < m; r += TQR_THREADS) s = abs2_add(xcol[r], s);
  s = warp_sum(s);
  S *rpart = reinterpret_cast<S *>(c.part);
  if ((tid & 31) == 0) rpart[tid >> 5] = s;
  __syncthreads();
  if (tid == 0) {
    S t = 0;
#pragma unroll
    for (int w = 0; w < TQR_WARPS; ++w) t += rpart[w];
    E beta, tv, sc;
    if (householder(c.row[(size_t)i * c.rs], t, beta, tv, sc)) {
      if constexpr (std::is_same<E, double>::value) {
        if (c.round32) tv = (double)(float)tv;
      }
      c.scal[0] = beta; c.scal[1] = tv; c.scal[2] = sc; c.scal[3] = E(1);
    } else {
      c.scal[3] = E(0);
    }
  }
  __syncthreads();
  if (c.scal[3] == E(0)) {
    if (tid == 0) *tau_out = E(0);
    if (zero_t_on_skip && c.Ts)
      for (int p = tid; p <= i; p += TQR_THREADS) c.Ts[p + (size_t)i * c.ldts] = E(0);
    __syncthreads();
    return false;
  }
  const E beta = c.scal[0], tv = c.scal[1], sc = c.scal[2];
  // d_j = -conj(tau) S_j (j > i), -tau conj(S_j) (j < i)
  auto dval = [&](int j, E acc) -> E { return j > i ? -(conj_(tv) * acc) : -(tv * conj_(acc)); };
  if constexpr (std::is_same<E, double>::value) {
    if (c.round32) {
      for (int r = x0 + tid; r < m; r += TQR_THREADS) xcol[r] = (double)(float)(xcol[r] * sc);
    } else {
      for (int r = x0 + tid; r < m; r += TQR_THREADS) xcol[r] *= sc;
    }
  } else {
    for (int r = x0 + tid; r < m; r += TQR_THREADS) xcol[r] *= sc;
  }
  __syncthreads();
  // ---- d_j for all j != i (j < i only when T is built) ----
  const int jlo = c.Ts ? 0 : i + 1;
  const int nj = nc - jlo;
  if (nj > 0 && sizeof(S) == 4) {
    // single precision: a warp per four columns, lanes over rows (stride 32),
    // one shuffle reduction per column -- no shared-memory partials and one
    // barrier less; the FP32 pipe makes the reduction's adds cheap
    const int lane = tid & 31, warp = tid >> 5;
    for (int jb = jlo + 4 * warp; jb < nc; jb += 4 * TQR_WARPS) {
      E a[4];
      const E *pcs[4];
      int mjs[4];
      int mmax = x0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = jb + u;
        a[u] = E(0);
        pcs[u] = c.P + (size_t)j * c.ldp;
        mjs[u] = (j < nc && j != i) ? ((c.tt >= 0 && j < i) ? min(m, c.tt + j + 1) : m) : x0;
        mmax = max(mmax, mjs[u]);
      }
      for (int r = x0 + lane; r < mmax; r += 32) {
        const E xv = xcol[r];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (r < mjs[u]) a[u] = madc(xv, pcs[u][r], a[u]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = warp_sum(a[u]);
      if (lane == 0) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = jb + u;
          if (j >= nc || j == i) continue;
          E acc = a[u];
          if (j > i || (!tsqrt_form && j < i)) acc += c.row[(size_t)j * c.rs];
          c.d[j] = dval(j, acc);
        }
      }
    }
  } else if (nj > 0) {
    if (nj <= TQR_THREADS) {
      const int G = TQR_THREADS / nj;          // row groups
      const int j = jlo + tid % nj, g = tid / nj;
      if (g < G) {
        E a0 = 0, a1 = 0;
        if (j != i) {
          const E *pc = c.P + (size_t)j * c.ldp;
          const int mj = (c.tt >= 0 && j < i) ? min(m, c.tt + j + 1) : m;
          int r = x0 + g;
          for (; r + G < mj; r += 2 * G) {
            a0 = madc(xcol[r], pc[r], a0);
            a1 = madc(xcol[r + G], pc[r + G], a1);
          }
          if (r < mj) a0 = madc(xcol[r], pc[r], a0);
        }
        c.part[g * nj + (j - jlo)] = a0 + a1;
      }
      __syncthreads();
      if (tid < nj) {
        const int jj = jlo + tid;
        E acc = 0;
        for (int gg = 0; gg < G; ++gg) acc += c.part[gg * nj + tid];
        if (jj > i || (!tsqrt_form && jj < i)) acc += c.row[(size_t)jj * c.rs];
        c.d[jj] = dval(jj, acc);
      }
    } else {
      const int lane = tid & 31, warp = tid >> 5;
      for (int j = jlo + warp; j < nc; j += TQR_WARPS) {
        if (j == i) continue;
        const E *pc = c.P + (size_t)j * c.ldp;
        const int mj = (c.tt >= 0 && j < i) ? min(m, c.tt + j + 1) : m;
        E a = 0;
        for (int r = x0 + lane; r < mj; r += 32) a = madc(xcol[r], pc[r], a);
        a = warp_sum(a);
        if (lane == 0) {
          if (j > i || (!tsqrt_form && j < i)) a += c.row[(size_t)j * c.rs];
          c.d[j] = dval(j, a);
        }
      }
    }
  }
  __syncthreads();
  // ---- rank-1 update of the columns right of i: one row per thread, its x
  //      entry held in a register, the columns in order (no index division) ----
  {
    const int rows = m - x0;
    for (int j = i + 1 + tid; j < nc; j += TQR_THREADS) c.row[(size_t)j * c.rs] += c.d[j];
    for (int rr = tid; rr < rows; rr += TQR_THREADS) {
      const E xv = xcol[x0 + rr];
      E *pr = c.P + x0 + rr;
#pragma unroll 4
      for (int j = i + 1; j < nc; ++j) pr[(size_t)j * c.ldp] = mad(xv, c.d[j], pr[(size_t)j * c.ldp]);
    }
  }
  // ---- T column i: T[p, i] = sum_{q = p}^{i-1} T[p, q] d[q], four partial
  //      sums over q (mod 4) to shorten the dependent chain ----
  if (c.Ts) {
    for (int p = tid; p < i; p += TQR_THREADS) {
      E a0 = 0, a1 = 0, a2 = 0, a3 = 0;
      const E *tp = c.Ts + p;
      int q = p;
      for (; q + 3 < i; q += 4) {
        a0 = mad(tp[(size_t)q * c.ldts], c.d[q], a0);
        a1 = mad(tp[(size_t)(q + 1) * c.ldts], c.d[q + 1], a1);
        a2 = mad(tp[(size_t)(q + 2) * c.ldts], c.d[q + 2], a2);
        a3 = mad(tp[(size_t)(q + 3) * c.ldts], c.d[q + 3], a3);
      }
      for (; q < i; ++q) a0 = mad(tp[(size_t)q * c.ldts], c.d[q], a0);
      c.Ts[p + (size_t)i * c.ldts] = (a0 + a1) + (a2 + a3);
    }
    if (tid == 0) c.Ts[i + (size_t)i * c.ldts] = tv;
  }
  if (tid == 0) {
    c.row[(size_t)i * c.rs] = beta;
    *tau_out = tv;
  }
  __syncthreads();
  return true;
}

// The column loop of a staged FP64 panel (T built in shared memory, 256
// threads) with nothing waiting on the serial parts of a column.  FORM 0:
// geqr2 (x rows [i + 1, m) of column i, row i of the panel is P's row i);
// 1: tsqrt (x rows [0, m), row i of the triangle in rowb); 2: ttqrt (x rows
// [0, min(m, tt + i + 1)), column j of P holds rows [0, tt + j]).  The same
// arithmetic as column_step, column by column, except the grouping of the T
// column's sums; per column i:
//   S  x *= scale (rounded to FP32 with round32);
//   A  d_j = -tau (row_j [j > i, or any j != i for geqr2] + x^T P_j), j != i,
//      laid out as (column j = tid / 8, row group tid % 8), three shuffles;
//   B  column i + 1 updated first and the squares of its next x region summed;
//   C  warp 0 forms column i + 1's Householder scalars (a square root and two
//      divisions, ~30 dependent FP64 instructions) while warps 1..7 update
//      columns i + 2 .. nc - 1 over all x rows, add d to row i and form the T
//      column's partial sums (seven per row p < i); warp 0 collects those on
//      a named barrier and adds them in fixed order.
// part[] holds 256 values: [0, 8) the norm partials, [32, 256) the T partials.
template <int FORM>
__device__ void columns_la_f64(double *P, int ldp, double *rowb, int rs, double *Ts, int ldts, double *d,
                               double *part, double *scal, int m, int k, int nc, int tt, bool round32,
                               bool zero_t_on_skip, double *tau)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double *tpart = part + 32;
  auto x0 = [&](int i) { return FORM == 0 ? i + 1 : 0; };
  auto mx = [&](int i) { return FORM == 2 ? min(m, tt + i + 1) : m; };
  auto scalars = [&](int col) {   // warp 0
    double t = lane < TQR_WARPS ? part[lane] : 0.0;
    t += __shfl_xor_sync(0xffffffffu, t, 4);
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    if (lane == 0) {
      double beta, tv, sc;
      if (householder(rowb[(size_t)col + (size_t)col * rs], t, beta, tv, sc)) {
        if (round32) tv = (double)(float)tv;
        scal[0] = beta; scal[1] = tv; scal[2] = sc; scal[3] = 1.0;
      } else {
        scal[3] = 0.0;
      }
    }
  };
  auto norm_partials = [&](int col) {
    const double *xc = P + (size_t)col * ldp;
    double s = 0.0;
    for (int r = x0(col) + tid; r < mx(col); r += TQR_THREADS) s = fma(xc[r], xc[r], s);
    s = warp_sum(s);
    if (lane == 0) part[warp] = s;
  };
  if (k <= 0) return;
  norm_partials(0);
  __syncthreads();
  if (warp == 0) scalars(0);
  __syncthreads();
  const int jd = tid >> 3, gd = tid & 7;
  for (int i = 0; i < k; ++i) {
    double *xi = P + (size_t)i * ldp;
    const double beta = scal[0], tv = scal[1], sc = scal[2];
    const bool has = scal[3] != 0.0;
    const int lo = x0(i), hi = mx(i);
    if (!has) {
      if (tid == 0) tau[i] = 0.0;
      if (zero_t_on_skip)
        for (int p = tid; p <= i; p += TQR_THREADS) Ts[p + (size_t)i * ldts] = 0.0;
      if (i + 1 < k) {
        norm_partials(i + 1);
        __syncthreads();
        if (warp == 0) scalars(i + 1);
      }
      __syncthreads();
      continue;
    }
    // ---- S ----
    if (round32) {
      for (int r = lo + tid; r < hi; r += TQR_THREADS) xi[r] = (double)(float)(xi[r] * sc);
    } else {
      for (int r = lo + tid; r < hi; r += TQR_THREADS) xi[r] *= sc;
    }
    __syncthreads();
    // ---- A ----
    {
      double a0 = 0.0, a1 = 0.0;
      if (jd < nc && jd != i) {
        const double *pj = P + (size_t)jd * ldp;
        const int hj = (FORM == 2 && jd < i) ? min(m, tt + jd + 1) : hi;
        int r = lo + gd;
        for (; r + 8 < hj; r += 16) {
          a0 = fma(xi[r], pj[r], a0);
          a1 = fma(xi[r + 8], pj[r + 8], a1);
        }
        if (r < hj) a0 = fma(xi[r], pj[r], a0);
      }
      double a = a0 + a1;
      a += __shfl_xor_sync(0xffffffffu, a, 4);
      a += __shfl_xor_sync(0xffffffffu, a, 2);
      a += __shfl_xor_sync(0xffffffffu, a, 1);
      if (gd == 0 && jd < nc && jd != i) {
        if (jd > i || (FORM == 0 && jd < i)) a += rowb[(size_t)i + (size_t)jd * rs];
        d[jd] = -(tv * a);
      }
    }
    __syncthreads();
    // ---- B: column i + 1 first, the squares of its x region ----
    if (i + 1 < nc) {
      double *pn = P + (size_t)(i + 1) * ldp;
      const double dn = d[i + 1];
      const bool nrm = i + 1 < k;
      const int nlo = nrm ? x0(i + 1) : hi, nhi = nrm ? mx(i + 1) : hi;
      double s = 0.0;
      for (int r = min(lo, nlo) + tid; r < max(hi, nhi); r += TQR_THREADS) {
        double v = pn[r];
        if (r >= lo && r < hi) {
          v = fma(xi[r], dn, v);
          pn[r] = v;
        }
        if (r >= nlo && r < nhi) s = fma(v, v, s);
      }
      if (tid == 0) rowb[(size_t)i + (size_t)(i + 1) * rs] += dn;
      s = warp_sum(s);
      if (lane == 0) part[warp] = s;
      __syncthreads();
    }
    // ---- C ----
    if (warp == 0) {
      if (i + 1 < k) scalars(i + 1);
      asm volatile("bar.sync 1, %0;" ::"r"(TQR_THREADS) : "memory");
      if (lane < i) {
        double v = tpart[lane];
#pragma unroll
        for (int w = 1; w < 7; ++w) v += tpart[w * 32 + lane];
        Ts[lane + (size_t)i * ldts] = v;
      }
    } else {
      const int w7 = warp - 1;
      {
        double v = 0.0;
        for (int q = lane + w7; q < i; q += 7) v = fma(Ts[lane + (size_t)q * ldts], d[q], v);
        tpart[w7 * 32 + lane] = v;
      }
      asm volatile("bar.arrive 1, %0;" ::"r"(TQR_THREADS) : "memory");
      // columns i + 2 .. nc - 1 over the x rows, spread over the 224 threads
      const int rows = hi - lo;
      if (rows > 0) {
        int r = tid - 32, j = i + 2;
        if (r >= rows) { j += r / rows; r %= rows; }
        while (j < nc) {
          double *pr = P + lo + r + (size_t)j * ldp;
          *pr = fma(xi[lo + r], d[j], *pr);
          r += TQR_THREADS - 32;
          if (r >= rows) { j += r / rows; r %= rows; }
        }
      }
      if (warp == 1)
        for (int j2 = i + 2 + lane; j2 < nc; j2 += 32) rowb[(size_t)i + (size_t)j2 * rs] += d[j2];
      if (tid == 32) {
        Ts[i + (size_t)i * ldts] = tv;
        rowb[(size_t)i + (size_t)i * rs] = beta;
        tau[i] = tv;
      }
    }
    __syncthreads();
  }
}

template <typename R>
__device__ inline R *carve(unsigned char *&p, size_t n) {
  R *r = reinterpret_cast<R *>(p);
  p += ((n * sizeof(R) + 15) / 16) * 16;
  return r;
}

__host__ __device__ inline size_t rnd16(size_t b) { return ((b + 15) / 16) * 16; }

template <typename R>
__host__ __device__ inline size_t panel_smem(int m, int nc, bool staged, bool stage_t) {
  size_t s = rnd16(sizeof(R) * TQR_THREADS) + rnd16(sizeof(R) * nc) + rnd16(sizeof(R) * 4);
  if (stage_t) s += rnd16(sizeof(R) * (size_t)odd_ld(nc) * nc);
  if (staged) s += rnd16(sizeof(R) * (size_t)odd_ld(m) * nc);
  return s;
}

// (for the ttqrt form pass m = min(m, ii + sb), the rows the block touches)
template <typename R>
__host__ __device__ inline size_t tsqrt_smem(int m, int sb, bool staged) {
  size_t s = rnd16(sizeof(R) * TQR_THREADS) + rnd16(sizeof(R) * sb) + rnd16(sizeof(R) * 4) +
             2 * rnd16(sizeof(R) * (size_t)odd_ld(sb) * sb);
  if (staged) s += rnd16(sizeof(R) * (size_t)odd_ld(m) * sb);
  return s;
}

// geqr2 (+ T) on the m-by-nc panel A; T (nc-by-nc, ldt) may be nullptr.
// VEC: 16-byte staging for FP32 elements (as apply_strip).
template <typename R, bool VEC = false>
__device__ void panel_qr_cta(int m, int nc, R *A, int lda, R *tau, R *T, int ldt, bool staged,
                             bool stage_t, unsigned char *smem_raw)
{
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x;
  ColumnStep<R> c;
  c.part = carve<R>(sp, TQR_THREADS);
  c.d = carve<R>(sp, nc);
  c.scal = carve<R>(sp, 4);
  if (T && stage_t) {
    c.ldts = odd_ld(nc);
    c.Ts = carve<R>(sp, (size_t)c.ldts * nc);
  } else {
    c.Ts = T;
    c.ldts = ldt;
  }
  if (staged) {
    c.ldp = odd_ld(m);
    c.P = carve<R>(sp, (size_t)c.ldp * nc);
    if (VEC && cols16_ok(A, (size_t)lda, m)) {
      stage_cols16_f32(A, (size_t)lda, m, nc, c.P, c.ldp, false);
    } else {
      for (int idx = tid; idx < m * nc; idx += TQR_THREADS) {
        int r = idx % m, cc = idx / m;
        c.P[ix(r, cc, c.ldp)] = ldg_cg(A + ix(r, cc, lda));
      }
    }
  } else {
    c.P = A;
    c.ldp = lda;
  }
  __syncthreads();
  const int k = min(m, nc);
  bool done = false;
  if constexpr (std::is_same<R, double>::value) {
    // staged FP64 panel with T in shared memory: the latency-hiding column
    // loop (a one-row column, geqr2.jl:32-35, is its empty-norm case)
    if (staged && T && stage_t && nc <= 32) {
      columns_la_f64<0>(c.P, c.ldp, c.P, c.ldp, c.Ts, c.ldts, c.d, c.part, c.scal, m, k, nc, -1, false, true,
                        tau);
      done = true;
    }
  }
  for (int i = 0; i < k && !done; ++i) {
    c.row = c.P + i;
    c.rs = c.ldp;
    if (m - i <= 1) {                                  // geqr2.jl:32-35
      if (tid == 0) tau[i] = R(0);
      if (c.Ts)
        for (int p = tid; p <= i; p += TQR_THREADS) c.Ts[p + (size_t)i * c.ldts] = R(0);
      __syncthreads();
      continue;
    }
    column_step<R>(c, i, i + 1, m, nc, false, tau + i, true);
  }
  if (staged) {
    if (VEC && cols16_ok(A, (size_t)lda, m)) {
      unstage_cols16_f32(c.P, c.ldp, m, nc, A, (size_t)lda, false);
    } else {
      for (int idx = tid; idx < m * nc; idx += TQR_THREADS) {
        int r = idx % m, cc = idx / m;
        A[ix(r, cc, lda)] = c.P[ix(r, cc, c.ldp)];
      }
    }
  }
  if (T && stage_t) {
    for (int idx = tid; idx < k * k; idx += TQR_THREADS) {
      int p = idx % k, q = idx / k;
      if (p <= q) T[ix(p, q, ldt)] = c.Ts[p + (size_t)q * c.ldts];
    }
  }
  __syncthreads();
}

// One ib-block of tsqrt.  A1 points at A1[ii, ii] (sb-by-sb diagonal block,
// only its upper triangle is read or written), A2 at A2[0, ii] (m-by-sb),
// T at T[0, ii], tau at tau[ii].  A column whose A2 part is exactly zero gets
// tau = 0 and leaves its T column untouched, as the reference does
// (tsqrt.jl:61-64).
// tt >= 0 gives the block of ttqrt instead (src/ttqrt.jl:1-80): A2 is upper
// triangular, block column i holds rows [0, tt + i] of A2 (tt = ii), so
// column i's reflector uses rows [0, min(tt + i + 1, m)) and nothing below
// the diagonal is read or written.
template <typename R, bool VEC = false>
__device__ void tsqrt_block_cta(int m, int sb, R *A1, int lda1, R *A2, int lda2, R *T, int ldt,
                                R *tau, bool staged, unsigned char *smem_raw, int tt = -1)
{
  const int mrow = tt >= 0 ? min(m, tt + sb) : m;     // rows of A2 the block touches
  auto in_tri = [&](int r, int cc) { return tt < 0 || r <= tt + cc; };
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x;
  ColumnStep<R> c;
  c.part = carve<R>(sp, TQR_THREADS);
  c.d = carve<R>(sp, sb);
  c.scal = carve<R>(sp, 4);
  const int ldb = odd_ld(sb);
  R *B = carve<R>(sp, (size_t)ldb * sb);
  c.ldts = odd_ld(sb);
  c.Ts = carve<R>(sp, (size_t)c.ldts * sb);
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      B[ix(r, cc, ldb)] = ldg_cg(A1 + ix(r, cc, lda1));
      c.Ts[r + (size_t)cc * c.ldts] = ldg_cg(T + ix(r, cc, ldt));   // skipped columns keep T
    }
  }
  if (staged) {
    c.ldp = odd_ld(mrow);
    c.P = carve<R>(sp, (size_t)c.ldp * sb);
    if (VEC && tt < 0 && cols16_ok(A2, (size_t)lda2, mrow)) {
      stage_cols16_f32(A2, (size_t)lda2, mrow, sb, c.P, c.ldp, false);
    } else {
      for (int idx = tid; idx < mrow * sb; idx += TQR_THREADS) {
        int r = idx % mrow, cc = idx / mrow;
        c.P[ix(r, cc, c.ldp)] = in_tri(r, cc) ? ldg_cg(A2 + ix(r, cc, lda2)) : R(0);
      }
    }
  } else {
    c.P = A2;
    c.ldp = lda2;
  }
  c.tt = tt;
  __syncthreads();
  c.rs = ldb;
  bool done = false;
  if constexpr (std::is_same<R, double>::value) {
    if (staged && sb <= 32) {
      if (tt >= 0)
        columns_la_f64<2>(c.P, c.ldp, B, ldb, c.Ts, c.ldts, c.d, c.part, c.scal, m, sb, sb, tt, false, false, tau);
      else
        columns_la_f64<1>(c.P, c.ldp, B, ldb, c.Ts, c.ldts, c.d, c.part, c.scal, m, sb, sb, -1, false, false, tau);
      done = true;
    }
  }
  for (int i = 0; i < sb && !done; ++i) {
    c.row = B + i;
    column_step<R>(c, i, 0, tt >= 0 ? min(m, tt + i + 1) : m, sb, true, tau + i, false);
  }
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      A1[ix(r, cc, lda1)] = B[ix(r, cc, ldb)];
      T[ix(r, cc, ldt)] = c.Ts[r + (size_t)cc * c.ldts];
    }
  }
  if (staged) {
    if (VEC && tt < 0 && cols16_ok(A2, (size_t)lda2, mrow)) {
      unstage_cols16_f32(c.P, c.ldp, mrow, sb, A2, (size_t)lda2, false);
    } else {
      for (int idx = tid; idx < mrow * sb; idx += TQR_THREADS) {
        int r = idx % mrow, cc = idx / mrow;
        if (in_tri(r, cc)) A2[ix(r, cc, lda2)] = c.P[ix(r, cc, c.ldp)];
      }
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Panels of an FP32 matrix computed in FP64 (the mixed-precision tile QR).
// The block is widened into shared memory as doubles (exact), the Householder
// norms and scalars, the in-block updates and the T build run in FP64
// (column_step<double>).  Each reflector v and its tau are rounded to FP32
// the moment they are formed (ColumnStep::round32), so the rest of the block,
// the FP64 T build and the FP32 trailing updates all apply the reflector that
// is stored; T is rounded once, on the way out.  The R triangle on
// the panel's diagonal -- geqrt's ib x ib block, which every tsqrt block of
// the panel then updates as its A1 -- also goes to an FP64 copy D; the tsqrt
// blocks read and write D instead of the rounded A1, so the chain of tsqrt
// blocks down a panel never rounds it (A1 receives each result rounded, and
// holds the final R after the last one).
// ---------------------------------------------------------------------------
__host__ __device__ inline size_t panel_f64_smem(int m, int nc) {
  return panel_smem<double>(m, nc, true, true) + rnd16(sizeof(double) * nc);
}
__host__ __device__ inline size_t tsqrt_f64_smem(int m, int sb) {
  return tsqrt_smem<double>(m, sb, true) + rnd16(sizeof(double) * sb);
}

// geqr2 + T of the m-by-nc FP32 panel A in FP64.  D (ldd) receives the upper
// triangle of the first min(m, nc) rows in FP64.
__device__ inline void panel_qr_cta_f64(int m, int nc, float *A, int lda, float *tau, float *T, int ldt,
                                        double *D, int ldd, unsigned char *smem_raw)
{
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x;
  ColumnStep<double> c;
  c.round32 = true;
  c.part = carve<double>(sp, TQR_THREADS);
  c.d = carve<double>(sp, nc);
  c.scal = carve<double>(sp, 4);
  c.ldts = odd_ld(nc);
  c.Ts = carve<double>(sp, (size_t)c.ldts * nc);
  c.ldp = odd_ld(m);
  c.P = carve<double>(sp, (size_t)c.ldp * nc);
  double *taus = carve<double>(sp, nc);
  for (int idx = tid; idx < m * nc; idx += TQR_THREADS) {
    const int r = idx % m, cc = idx / m;
    c.P[ix(r, cc, c.ldp)] = (double)ldg_cg(A + ix(r, cc, lda));
  }
  __syncthreads();
  const int k = min(m, nc);
  if (nc <= 32) {
    columns_la_f64<0>(c.P, c.ldp, c.P, c.ldp, c.Ts, c.ldts, c.d, c.part, c.scal, m, k, nc, -1, true, true, taus);
  } else {
    for (int i = 0; i < k; ++i) {
      c.row = c.P + i;
      c.rs = c.ldp;
      if (m - i <= 1) {                                  // geqr2.jl:32-35
        if (tid == 0) taus[i] = 0.0;
        for (int p = tid; p <= i; p += TQR_THREADS) c.Ts[p + (size_t)i * c.ldts] = 0.0;
        __syncthreads();
        continue;
      }
      column_step<double>(c, i, i + 1, m, nc, false, taus + i, true);
    }
  }
  for (int idx = tid; idx < m * nc; idx += TQR_THREADS) {
    const int r = idx % m, cc = idx / m;
    const double v = c.P[ix(r, cc, c.ldp)];
    A[ix(r, cc, lda)] = (float)v;
    if (r <= cc && r < k) D[ix(r, cc, ldd)] = v;
  }
  for (int idx = tid; idx < k * k; idx += TQR_THREADS) {
    const int p = idx % k, q = idx / k;
    if (p <= q) T[ix(p, q, ldt)] = (float)c.Ts[p + (size_t)q * c.ldts];
  }
  for (int i = tid; i < k; i += TQR_THREADS) tau[i] = (float)taus[i];
  __syncthreads();
}

// One ib-block of tsqrt on an FP32 A2 (m-by-sb) in FP64; its A1 triangle is
// read from and written to the FP64 copy D (ldd), and written rounded to A1.
__device__ inline void tsqrt_block_cta_f64(int m, int sb, double *D, int ldd, float *A1, int lda1, float *A2,
                                           int lda2, float *T, int ldt, float *tau, unsigned char *smem_raw)
{
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x;
  ColumnStep<double> c;
  c.round32 = true;
  c.part = carve<double>(sp, TQR_THREADS);
  c.d = carve<double>(sp, sb);
  c.scal = carve<double>(sp, 4);
  const int ldb = odd_ld(sb);
  double *B = carve<double>(sp, (size_t)ldb * sb);
  c.ldts = odd_ld(sb);
  c.Ts = carve<double>(sp, (size_t)c.ldts * sb);
  c.ldp = odd_ld(m);
  c.P = carve<double>(sp, (size_t)c.ldp * sb);
  double *taus = carve<double>(sp, sb);
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      B[ix(r, cc, ldb)] = ldg_cg(D + ix(r, cc, ldd));
      c.Ts[r + (size_t)cc * c.ldts] = (double)ldg_cg(T + ix(r, cc, ldt));   // skipped columns keep T
    }
  }
  for (int idx = tid; idx < m * sb; idx += TQR_THREADS) {
    const int r = idx % m, cc = idx / m;
    c.P[ix(r, cc, c.ldp)] = (double)ldg_cg(A2 + ix(r, cc, lda2));
  }
  __syncthreads();
  c.rs = ldb;
  if (sb <= 32) {
    columns_la_f64<1>(c.P, c.ldp, B, ldb, c.Ts, c.ldts, c.d, c.part, c.scal, m, sb, sb, -1, true, false, taus);
  } else {
    for (int i = 0; i < sb; ++i) {
      c.row = B + i;
      column_step<double>(c, i, 0, m, sb, true, taus + i, false);
    }
  }
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      const double v = B[ix(r, cc, ldb)];
      D[ix(r, cc, ldd)] = v;
      A1[ix(r, cc, lda1)] = (float)v;
      T[ix(r, cc, ldt)] = (float)c.Ts[r + (size_t)cc * c.ldts];
    }
  }
  for (int idx = tid; idx < m * sb; idx += TQR_THREADS) {
    const int r = idx % m, cc = idx / m;
    A2[ix(r, cc, lda2)] = (float)c.P[ix(r, cc, c.ldp)];
  }
  for (int i = tid; i < sb; i += TQR_THREADS) tau[i] = (float)taus[i];
  __syncthreads();
}

// One ib-block of ttqrt (src/ttqrt.jl:1-80) in FP64 for the mixed form of the
// hierarchical tree: A1's triangle is read from and written to its FP64 copy
// D1 (ldd1) and written rounded to A1; A2 holds the block's columns of the
// upper-triangular partner R, rows [0, tt + sb): rows [0, tt) come from the
// FP32 A2, the partner's diagonal triangle (rows [tt, tt + sb)) from its FP64
// copy D2 (ldd2).  Reflector q uses rows [0, tt + q] (the tt form of
// column_step).  The merge reflectors go back to A2 rounded; D2 is consumed.
__host__ __device__ inline size_t ttqrt_f64_smem(int m, int sb) {
  return tsqrt_smem<double>(m, sb, true) + rnd16(sizeof(double) * sb);
}

__device__ inline void ttqrt_block_cta_f64(int m, int sb, int tt, double *D1, int ldd1, float *A1, int lda1,
                                           const double *D2, int ldd2, float *A2, int lda2, float *T, int ldt,
                                           float *tau, unsigned char *smem_raw)
{
  const int mrow = min(m, tt + sb);
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x;
  ColumnStep<double> c;
  c.round32 = true;
  c.part = carve<double>(sp, TQR_THREADS);
  c.d = carve<double>(sp, sb);
  c.scal = carve<double>(sp, 4);
  const int ldb = odd_ld(sb);
  double *B = carve<double>(sp, (size_t)ldb * sb);
  c.ldts = odd_ld(sb);
  c.Ts = carve<double>(sp, (size_t)c.ldts * sb);
  c.ldp = odd_ld(mrow);
  c.P = carve<double>(sp, (size_t)c.ldp * sb);
  double *taus = carve<double>(sp, sb);
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      B[ix(r, cc, ldb)] = ldg_cg(D1 + ix(r, cc, ldd1));
      c.Ts[r + (size_t)cc * c.ldts] = (double)ldg_cg(T + ix(r, cc, ldt));   // skipped columns keep T
    }
  }
  for (int idx = tid; idx < mrow * sb; idx += TQR_THREADS) {
    const int r = idx % mrow, cc = idx / mrow;
    double v = 0.0;
    if (r <= tt + cc) v = r < tt ? (double)ldg_cg(A2 + ix(r, cc, lda2)) : ldg_cg(D2 + ix(r - tt, cc, ldd2));
    c.P[ix(r, cc, c.ldp)] = v;
  }
  c.tt = tt;
  __syncthreads();
  c.rs = ldb;
  if (sb <= 32) {
    columns_la_f64<2>(c.P, c.ldp, B, ldb, c.Ts, c.ldts, c.d, c.part, c.scal, m, sb, sb, tt, true, false, taus);
  } else {
    for (int i = 0; i < sb; ++i) {
      c.row = B + i;
      column_step<double>(c, i, 0, min(m, tt + i + 1), sb, true, taus + i, false);
    }
  }
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      const double v = B[ix(r, cc, ldb)];
      D1[ix(r, cc, ldd1)] = v;
      A1[ix(r, cc, lda1)] = (float)v;
      T[ix(r, cc, ldt)] = (float)c.Ts[r + (size_t)cc * c.ldts];
    }
  }
  for (int idx = tid; idx < mrow * sb; idx += TQR_THREADS) {
    const int r = idx % mrow, cc = idx / mrow;
    if (r <= tt + cc) A2[ix(r, cc, lda2)] = (float)c.P[ix(r, cc, c.ldp)];
  }
  for (int i = tid; i < sb; i += TQR_THREADS) tau[i] = (float)taus[i];
  __syncthreads();
}

// The tsqrt block of the mixed form laid out for latency (sb <= 32, m <= 256,
// 256 threads).  Same arithmetic as tsqrt_block_cta_f64 (column_step<double>
// with round32 in the tsqrt form) except the order of some sums, reorganised
// because a dependent FP64 instruction costs ~64 cycles on GB300 and the
// block runs on the serial tsqrt chain of a panel.  Columns with a zero A2
// part are skipped as in the reference (tau = 0, T column untouched,
// src/tsqrt.jl:61-64).  Nothing waits on the serial parts of a column (the
// next column's Householder scalars: a square root and two divisions, ~30
// dependent FP64 instructions; the T column's sums) with the whole block
// idle.  Per column i:
//   S  x_i *= scale, rounded to the stored FP32 reflector;
//   A  d_j = -tau (row_j [j > i] + x^T P_j), j != i;
//   B  column i + 1 updated first, its squares summed (the next norm);
//   C  warp 0 forms column i + 1's scalars from those sums while warps 1..7
//      update columns i + 2 .. sb - 1 (all rows, spread evenly), add d to row
//      i of the triangle and form the T column's partial sums (seven per
//      row p < i, over q = p + w, p + w + 7, ...); warp 0 then waits for the
//      partials on a named barrier and adds them in fixed order.
// The dot products S_j = x^T P_j are laid out as (column j = tid / 8, row
// group g = tid % 8), so each column's eight partial sums meet in eight
// consecutive lanes and reduce by three shuffles.  Four block barriers per
// column.  On one SM: 194 us per 256 x 32 block against 238 us with the
// scalars and the T column on warp 0 between barriers.
__host__ __device__ inline size_t tsqrt_f64x_smem(int m, int sb) {
  return rnd16(sizeof(double) * (size_t)odd_ld(m) * sb) + 2 * rnd16(sizeof(double) * (size_t)odd_ld(sb) * sb) +
         rnd16(sizeof(double) * 32) + rnd16(sizeof(double) * TQR_WARPS) + rnd16(sizeof(double) * 4) +
         rnd16(sizeof(double) * 32) + rnd16(sizeof(double) * 7 * 32);
}

__device__ inline void tsqrt_block_f64x(int m, int sb, double *D, int ldd, float *A1, int lda1, float *A2, int lda2,
                                        float *T, int ldt, float *tau, unsigned char *smem_raw)
{
  unsigned char *sp = smem_raw;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ldp = odd_ld(m), ldb = odd_ld(sb), ldts = odd_ld(sb);
  double *P = carve<double>(sp, (size_t)ldp * sb);
  double *B = carve<double>(sp, (size_t)ldb * sb);
  double *Ts = carve<double>(sp, (size_t)ldts * sb);
  double *d = carve<double>(sp, 32);
  double *part = carve<double>(sp, TQR_WARPS);
  double *scal = carve<double>(sp, 4);
  double *taus = carve<double>(sp, 32);
  double *tpart = carve<double>(sp, 7 * 32);
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      B[ix(r, cc, ldb)] = ldg_cg(D + ix(r, cc, ldd));
      Ts[r + (size_t)cc * ldts] = (double)ldg_cg(T + ix(r, cc, ldt));   // skipped columns keep T
    }
  }
  for (int idx = tid; idx < m * sb; idx += TQR_THREADS) {
    const int r = idx % m, cc = idx / m;
    P[ix(r, cc, ldp)] = (double)ldg_cg(A2 + ix(r, cc, lda2));
  }
  __syncthreads();
  // Householder scalars of column c from the norm partials in part[] (warp 0)
  auto scalars = [&](int c) {
    double t = lane < TQR_WARPS ? part[lane] : 0.0;
    t += __shfl_xor_sync(0xffffffffu, t, 4);
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    if (lane == 0) {
      double beta, tv, sc;
      if (householder(B[ix(c, c, ldb)], t, beta, tv, sc)) {
        scal[0] = beta; scal[1] = (double)(float)tv; scal[2] = sc; scal[3] = 1.0;
      } else {
        scal[3] = 0.0;
      }
    }
  };
  // norm partials of column c (rows split over the block)
  auto norm_partials = [&](int c) {
    const double *xc = P + (size_t)c * ldp;
    double s = 0.0;
    for (int r = tid; r < m; r += TQR_THREADS) s = fma(xc[r], xc[r], s);
    s = warp_sum(s);
    if (lane == 0) part[warp] = s;
  };
  norm_partials(0);
  __syncthreads();
  if (warp == 0) scalars(0);
  __syncthreads();
  const int jd = tid >> 3, gd = tid & 7;
  for (int i = 0; i < sb; ++i) {
    double *xi = P + (size_t)i * ldp;
    const double beta = scal[0], tv = scal[1], sc = scal[2];
    const bool has = scal[3] != 0.0;
    if (!has) {
      // no reflector: tau = 0, T column and the block's columns untouched
      if (tid == 0) taus[i] = 0.0;
      if (i + 1 < sb) {
        norm_partials(i + 1);
        __syncthreads();
        if (warp == 0) scalars(i + 1);
      }
      __syncthreads();
      continue;
    }
    // ---- S: x *= scale, rounded to the stored FP32 reflector ----
    for (int r = tid; r < m; r += TQR_THREADS) xi[r] = (double)(float)(xi[r] * sc);
    __syncthreads();
    // ---- A: d_j = -tau (row_j [j > i] + x^T P_j), j != i ----
    {
      double a0 = 0.0, a1 = 0.0;
      if (jd < sb && jd != i) {
        const double *pj = P + (size_t)jd * ldp;
        int r = gd;
        for (; r + 8 < m; r += 16) {
          a0 = fma(xi[r], pj[r], a0);
          a1 = fma(xi[r + 8], pj[r + 8], a1);
        }
        if (r < m) a0 = fma(xi[r], pj[r], a0);
      }
      double a = a0 + a1;
      a += __shfl_xor_sync(0xffffffffu, a, 4);
      a += __shfl_xor_sync(0xffffffffu, a, 2);
      a += __shfl_xor_sync(0xffffffffu, a, 1);
      if (gd == 0 && jd < sb && jd != i) {
        if (jd > i) a += B[ix(i, jd, ldb)];
        d[jd] = -(tv * a);
      }
    }
    __syncthreads();
    // ---- B: column i + 1 first, and the squares of its new entries ----
    if (i + 1 < sb) {
      double *pn = P + (size_t)(i + 1) * ldp;
      const double dn = d[i + 1];
      double s = 0.0;
      for (int r = tid; r < m; r += TQR_THREADS) {
        const double v = fma(xi[r], dn, pn[r]);
        pn[r] = v;
        s = fma(v, v, s);
      }
      s = warp_sum(s);
      if (lane == 0) part[warp] = s;
      __syncthreads();
    }
    // ---- C ----
    if (warp == 0) {
      if (i + 1 < sb) scalars(i + 1);
      asm volatile("bar.sync 1, %0;" ::"r"(TQR_THREADS) : "memory");
      if (lane < i) {
        double v = tpart[lane];
#pragma unroll
        for (int w = 1; w < 7; ++w) v += tpart[w * 32 + lane];
        Ts[lane + (size_t)i * ldts] = v;
      }
    } else {
      const int w7 = warp - 1;
      {
        double v = 0.0;
        for (int q = lane + w7; q < i; q += 7) v = fma(Ts[lane + (size_t)q * ldts], d[q], v);
        tpart[w7 * 32 + lane] = v;
      }
      asm volatile("bar.arrive 1, %0;" ::"r"(TQR_THREADS) : "memory");
      // columns i + 2 .. sb - 1, all rows, spread over the 224 threads
      const int t7 = tid - 32;
      int r = t7, j = i + 2;
      while (r >= m) { r -= m; ++j; }
      while (j < sb) {
        double *pr = P + r + (size_t)j * ldp;
        *pr = fma(xi[r], d[j], *pr);
        r += TQR_THREADS - 32;
        while (r >= m) { r -= m; ++j; }
      }
      if (warp == 1)
        for (int j2 = i + 1 + lane; j2 < sb; j2 += 32) B[ix(i, j2, ldb)] += d[j2];
      if (tid == 32) {
        Ts[i + (size_t)i * ldts] = tv;
        B[ix(i, i, ldb)] = beta;
        taus[i] = tv;
      }
    }
    __syncthreads();
  }
  for (int idx = tid; idx < sb * sb; idx += TQR_THREADS) {
    const int r = idx % sb, cc = idx / sb;
    if (r <= cc) {
      const double v = B[ix(r, cc, ldb)];
      D[ix(r, cc, ldd)] = v;
      A1[ix(r, cc, lda1)] = (float)v;
      T[ix(r, cc, ldt)] = (float)Ts[r + (size_t)cc * ldts];
    }
  }
  for (int idx = tid; idx < m * sb; idx += TQR_THREADS) {
    const int r = idx % m, cc = idx / m;
    A2[ix(r, cc, lda2)] = (float)P[ix(r, cc, ldp)];
  }
  for (int i = tid; i < sb; i += TQR_THREADS) tau[i] = (float)taus[i];
  __syncthreads();
}

}  // namespace tqr
