// pamm.cu -- NextLA's pamm! (src/pamm.jl:49-473) as a stand-alone entry
// point, every op / side / storev / direct form, real and complex.
//
// The reflector block in its canonical orientation Ve (mv x k, mv = m for side
// 'L', n for 'R') is V (storev 'C') or V^T ('R'); its trapezoid of order l
// holds, for direct 'F', only the upper triangle of the last l rows of the
// first l columns (pamm.jl:104-127) and, for 'B', only the lower triangle of
// the first l rows of the last l columns (pamm.jl:197-222); entries outside
// it are never read.
//   op 'W': W = A1 + f(Ve)^T A2 (side 'L') or A1 + A2 f(Ve) ('R'), f = conj
//           for (L, C) and (R, R);
//   op 'A': A2 -= g(Ve) W (L) or W g(Ve)^T (R), g = conj for (L, R) and
//           (R, C); W's first ('F') or last ('B') l rows (L) / columns (R)
//           then hold the trapezoid's triangle times W, as the reference's
//           in-place triangular product leaves them.
// Inside parfb! / tsmqr! the same two products run fused in apply_strip; this
// entry point is for callers of pamm! itself.  One thread per output element
// (the reduction runs over the reflector length or k); the 'A' op is two
// launches in stream order -- A2 from the incoming W, then W's triangle block
// in place, one thread per W column (row) walking the block in the order that
// only reads entries it has not yet overwritten.
#include "common.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

struct PammForm {
  int left, colmajor, fwd;
  int m, n, k, l, mv;
  int cjw, cja;
};

__device__ __forceinline__ bool pamm_valid(const PammForm &f, int r, int p) {
  if (f.fwd) return !(p < f.l && r >= f.mv - f.l && r - (f.mv - f.l) > p);
  return !(p >= f.k - f.l && r < f.l && r < p - (f.k - f.l));
}

template <typename E>
__device__ __forceinline__ E pamm_ve(const PammForm &f, const E *V, int ldv, int r, int p) {
  return f.colmajor ? V[ix(r, p, ldv)] : V[ix(p, r, ldv)];
}

template <typename E>
__global__ void __launch_bounds__(TQR_THREADS)
k_pamm_w(const PammForm f, const E *__restrict__ A1, int lda1, const E *__restrict__ A2, int lda2,
         const E *__restrict__ V, int ldv, E *__restrict__ W, int ldw)
{
  const long long id = (long long)blockIdx.x * TQR_THREADS + threadIdx.x;
  if (f.left) {                                        // W (k x n): element (p, c)
    if (id >= (long long)f.k * f.n) return;
    const int p = (int)(id % f.k), c = (int)(id / f.k);
    E acc = 0;
    for (int r = 0; r < f.m; ++r)
      if (pamm_valid(f, r, p)) acc = mad(conj_if(pamm_ve(f, V, ldv, r, p), f.cjw != 0), A2[ix(r, c, lda2)], acc);
    W[ix(p, c, ldw)] = A1[ix(p, c, lda1)] + acc;
  } else {                                             // W (m x k): element (i, p)
    if (id >= (long long)f.m * f.k) return;
    const int i = (int)(id % f.m), p = (int)(id / f.m);
    E acc = 0;
    for (int c = 0; c < f.n; ++c)
      if (pamm_valid(f, c, p)) acc = mad(A2[ix(i, c, lda2)], conj_if(pamm_ve(f, V, ldv, c, p), f.cjw != 0), acc);
    W[ix(i, p, ldw)] = A1[ix(i, p, lda1)] + acc;
  }
}

template <typename E>
__global__ void __launch_bounds__(TQR_THREADS)
k_pamm_a(const PammForm f, E *__restrict__ A2, int lda2, const E *__restrict__ V, int ldv,
         const E *__restrict__ W, int ldw)
{
  const long long id = (long long)blockIdx.x * TQR_THREADS + threadIdx.x;
  if (id >= (long long)f.m * f.n) return;
  const int i = (int)(id % f.m), c = (int)(id / f.m);
  E acc = 0;
  if (f.left) {
    for (int p = 0; p < f.k; ++p)
      if (pamm_valid(f, i, p)) acc = mad(conj_if(pamm_ve(f, V, ldv, i, p), f.cja != 0), W[ix(p, c, ldw)], acc);
  } else {
    for (int p = 0; p < f.k; ++p)
      if (pamm_valid(f, c, p)) acc = mad(W[ix(i, p, ldw)], conj_if(pamm_ve(f, V, ldv, c, p), f.cja != 0), acc);
  }
  A2[ix(i, c, lda2)] = A2[ix(i, c, lda2)] - acc;
}

// W's triangle block in place: triangle row t (A2 row/column rt) times the
// block.  'F': row t reads block entries p >= t (upper), so t ascends; 'B':
// p <= t (lower), so t descends.
template <typename E>
__global__ void __launch_bounds__(TQR_THREADS)
k_pamm_wtri(const PammForm f, const E *__restrict__ V, int ldv, E *__restrict__ W, int ldw)
{
  const int x = blockIdx.x * TQR_THREADS + threadIdx.x;
  const int cnt = f.left ? f.n : f.m;
  if (x >= cnt) return;
  const int b0 = f.fwd ? 0 : f.k - f.l;
  auto w = [&](int p) -> E & { return f.left ? W[ix(p, x, ldw)] : W[ix(x, p, ldw)]; };
  for (int s = 0; s < f.l; ++s) {
    const int t = f.fwd ? s : f.l - 1 - s;
    const int rt = f.fwd ? f.mv - f.l + t : t;
    E acc = 0;
    for (int p = b0; p < b0 + f.l; ++p)
      if (pamm_valid(f, rt, p)) {
        const E v = conj_if(pamm_ve(f, V, ldv, rt, p), f.cja != 0);
        acc = f.left ? mad(v, w(p), acc) : mad(w(p), v, acc);
      }
    w(b0 + t) = acc;
  }
}

template <typename E>
int pamm_impl(char op, char side, char storev, char direct, int m, int n, int k, int l, const E *A1, int lda1,
              E *A2, int lda2, const E *V, int ldv, E *W, int ldw, cudaStream_t st) {
  if (op != 'W' && op != 'A') return -1;               // src/pamm.jl:51-78
  if (side != 'L' && side != 'R') return -2;
  if (storev != 'C' && storev != 'R') return -3;
  if (direct != 'F' && direct != 'B') return -4;
  if (m < 0) return -5;
  if (n < 0) return -6;
  if (k < 0) return -7;
  if (l < 0) return -8;
  if (m == 0 || n == 0 || k == 0) return 0;            // src/pamm.jl:81-83
  PammForm f;
  f.left = side == 'L'; f.colmajor = storev == 'C'; f.fwd = direct == 'F';
  f.m = m; f.n = n; f.k = k; f.l = l; f.mv = f.left ? m : n;
  f.cjw = (f.left && f.colmajor) || (!f.left && !f.colmajor);
  f.cja = (f.left && !f.colmajor) || (!f.left && f.colmajor);
  if (l > k || l > f.mv) return -8;
  const int wrows = f.left ? k : m, wcols = f.left ? n : k;
  if (!A2 || lda2 < m) return -12;
  if (!V || ldv < (f.colmajor ? f.mv : k)) return -14;
  if (!W || ldw < wrows) return -16;
  cudaError_t e;
  if (op == 'W') {
    if (!A1 || lda1 < wrows) return -10;
    const long long nt = (long long)wrows * wcols;
    k_pamm_w<E><<<(unsigned)((nt + TQR_THREADS - 1) / TQR_THREADS), TQR_THREADS, 0, st>>>(f, A1, lda1, A2, lda2, V,
                                                                                         ldv, W, ldw);
    count_launch();
    e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
  }
  const long long na = (long long)m * n;
  k_pamm_a<E><<<(unsigned)((na + TQR_THREADS - 1) / TQR_THREADS), TQR_THREADS, 0, st>>>(f, A2, lda2, V, ldv, W, ldw);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
  if (l > 0) {
    const int cnt = f.left ? n : m;
    k_pamm_wtri<E><<<(cnt + TQR_THREADS - 1) / TQR_THREADS, TQR_THREADS, 0, st>>>(f, V, ldv, W, ldw);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
  }
  return 0;
}

// W := M W (side L, W k x cnt) or W M (side R, W cnt x k), M = tfun(T's upper
// ('F') or lower ('B') triangle), in place: one thread per W column (row),
// walking the outputs in the order that reads only entries not yet rewritten.
template <typename E>
__global__ void __launch_bounds__(TQR_THREADS)
k_parfb_tmul(int left, int upper, int adj, int k, int cnt, const E *__restrict__ T, int ldt, E *__restrict__ W,
             int ldw)
{
  const int x = blockIdx.x * TQR_THREADS + threadIdx.x;
  if (x >= cnt) return;
  auto m = [&](int i, int j) -> E {            // M[i, j]
    const int r = adj ? j : i, c = adj ? i : j;
    if (upper ? r > c : r < c) return E(0);
    return conj_if(T[ix(r, c, ldt)], adj != 0);
  };
  auto w = [&](int i) -> E & { return left ? W[ix(i, x, ldw)] : W[ix(x, i, ldw)]; };
  // effective triangle of M: upper when (upper, no adjoint) or (lower, adjoint)
  const bool mup = (upper != 0) != (adj != 0);
  // left: out[i] = sum_j M[i,j] w[j]; M upper -> reads j >= i -> ascending i.
  // right: out[j] = sum_i w[i] M[i,j]; M upper -> reads i <= j -> descending j.
  const bool ascend = left ? mup : !mup;
  for (int s = 0; s < k; ++s) {
    const int i = ascend ? s : k - 1 - s;
    // only the triangle's entries: the rest of w is already rewritten
    const bool hi = left ? mup : !mup;          // the nonzero j lie at or above i
    const int j0 = hi ? i : 0, j1 = hi ? k : i + 1;
    E acc = 0;
    if (left) {
      for (int j = j0; j < j1; ++j) acc = mad(m(i, j), w(j), acc);
    } else {
      for (int j = j0; j < j1; ++j) acc = mad(w(j), m(j, i), acc);
    }
    w(i) = acc;
  }
}

template <typename E>
__global__ void __launch_bounds__(TQR_THREADS)
k_sub_block(int rows, int cols, E *__restrict__ A, int lda, const E *__restrict__ W, int ldw)
{
  const long long id = (long long)blockIdx.x * TQR_THREADS + threadIdx.x;
  if (id >= (long long)rows * cols) return;
  const int r = (int)(id % rows), c = (int)(id / rows);
  A[ix(r, c, lda)] = A[ix(r, c, lda)] - W[ix(r, c, ldw)];
}

template <typename E>
int parfb_general(char side, char trans, char direct, char storev, int m2, int n2, int k, int l, E *A1, int lda1,
                  E *A2, int lda2, const E *V, int ldv, const E *T, int ldt, E *W, int ldw, cudaStream_t st) {
  const bool left = side == 'L';
  int rc = pamm_impl<E>('W', side, storev, direct, m2, n2, k, l, A1, lda1, A2, lda2, V, ldv, W, ldw, st);
  if (rc) return rc;
  const int cnt = left ? n2 : m2;
  k_parfb_tmul<E><<<(cnt + TQR_THREADS - 1) / TQR_THREADS, TQR_THREADS, 0, st>>>(
      left ? 1 : 0, direct == 'F' ? 1 : 0, trans != 'N' ? 1 : 0, k, cnt, T, ldt, W, ldw);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  const int rows = left ? k : m2, cols = left ? n2 : k;
  const long long nt = (long long)rows * cols;
  k_sub_block<E><<<(unsigned)((nt + TQR_THREADS - 1) / TQR_THREADS), TQR_THREADS, 0, st>>>(rows, cols, A1, lda1, W,
                                                                                          ldw);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
  return pamm_impl<E>('A', side, storev, direct, m2, n2, k, l, A1, lda1, A2, lda2, V, ldv, W, ldw, st);
}

#define TQR_PARFB_INST(E)                                                                                     \
  template int parfb_general<E>(char, char, char, char, int, int, int, int, E *, int, E *, int, const E *, int, \
                                const E *, int, E *, int, cudaStream_t);
TQR_PARFB_INST(double)
TQR_PARFB_INST(float)
TQR_PARFB_INST(cx<double>)
TQR_PARFB_INST(cx<float>)
#undef TQR_PARFB_INST

}  // namespace tqr

using namespace tqr;

extern "C" {

#define TQR_PAMM(P, CT, E)                                                                                     \
  int tqr_##P##pamm(char op, char side, char storev, char direct, int m, int n, int k, int l, const CT *A1,    \
                    int lda1, CT *A2, int lda2, const CT *V, int ldv, CT *W, int ldw, cudaStream_t stream) {    \
    if (((uintptr_t)A1 | (uintptr_t)A2 | (uintptr_t)V | (uintptr_t)W) % alignof(E)) return -9;                \
    return pamm_impl<E>(op, side, storev, direct, m, n, k, l, (const E *)A1, lda1, (E *)A2, lda2,              \
                        (const E *)V, ldv, (E *)W, ldw, stream);                                               \
  }
TQR_PAMM(d, double, double)
TQR_PAMM(s, float, float)
TQR_PAMM(z, tqr_zcomplex, cx<double>)
TQR_PAMM(c, tqr_ccomplex, cx<float>)
#undef TQR_PAMM

}  // extern "C"
