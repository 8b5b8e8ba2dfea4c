// ls.cu -- least squares on top of the tile QR: the mixed-precision solve.
//
// Not a NextLA routine: NextLA ships the tile kernels, and its poster lists a
// mixed-precision solver as future work.  min ||A X - B||_2 for a Float32-stored
// A (m >= n) and Float64 right-hand sides:
//
//   1. copy A into the factor workspace F and tile-QR it (the same persistent
//      kernel as the FP64 form, float instantiation): the trailing tsmqr
//      updates in FP32 (TF32x3 on the tensor cores), the panel tasks -- the
//      larfg norm and reflector scaling, the larft T build and the tsqrt
//      blocks with their diagonal R triangles -- in FP64 on a widened copy of
//      the panel block, V / T / tau rounded to FP32 once for the updates;
//   2. X0 = R^-1 (Q^T B)[0:n] in FP32 (tile Q application + triangular solve);
//   3. refine with CGLS on the right-preconditioned problem
//      min || (A R^-1) Y - B ||, X = R^-1 Y, with FP64 iterates: every product
//      with A uses the FP32 entries of A exactly and sums in double-float
//      (~2^-48 relative per 32 terms, FP64 beyond), every solve with R runs in
//      FP64 on R's FP32 entries.  A R^-1 is within O(kappa(A) u_32) of
//      orthonormal, so CGLS converges in a few iterations to the FP64 least-
//      squares solution; no product with Q is needed.
//
// On GB300 the FP32 pipe is ~55x the FP64 pipe, so steps 1-2 cost a small part
// of the FP64 factorisation and what is left is a handful of A*x and A^T*r
// products (4 m n k flops per iteration) and triangular solves.
//
// Kernels here (FP32 matrix entries, FP64 operands and results):
//   k_gemm_sd_n   Y = alpha A X + beta Y          (A m-by-n FP32, X n-by-k;
//                 double-float sums on the FP32 pipe, flushed to FP64)
//   k_gemm_sd_t   Z += alpha A^T R               (split over row blocks, FP64 atomics;
//                 the same double-float sums)
//   k_trinv_diag / k_blk_solve  triangular solves through inverted diagonal blocks
//   small column kernels for the CGLS recurrences (dots, axpys)
#include <algorithm>
#include <vector>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

constexpr int kLsMaxRhs = 16;

// Exact float -> double widening with integer instructions: every FP64 warp
// instruction occupies the SM sub-partition's FP64 pipe for ~64 cycles on
// GB300, and a conversion is one of them; for normal numbers the IEEE fields
// move directly (exponent rebias +896, mantissa shifted left 29).  Zeros,
// subnormals, infinities and NaNs take the ordinary conversion.
__device__ __forceinline__ double widen(float a) {
  const uint32_t u = __float_as_uint(a);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)a;
  const unsigned long long bits = ((unsigned long long)(u & 0x80000000u) << 32) |
                                  ((unsigned long long)(e + 896u) << 52) |
                                  ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// The products with A (FP32 entries) and an FP64 operand run in double-float
// arithmetic on the FP32 pipe, which is ~55x the FP64 pipe on GB300: the FP64
// operand x is split into floats x = xh + xl (|xl| <= 2^-24 |x|); a * xh is
// formed exactly as p + e (product and its FMA-recovered error) and added to
// the float pair (sh, sl) by Knuth's TwoSum, a * xl joins the low part, and
// the pair is renormalised (Fast2Sum) after every term so that sl stays below
// half an ulp of sh.  The pair is flushed into an FP64 accumulator every
// kDfFlush terms: a sum's rounding is ~2^-48 relative within a flushed group
// and FP64 across groups.  The _rn intrinsics keep the compiler from
// contracting the steps (a contracted TwoSum is no longer error-free).
// Measured at 32768 x 4096, 4 right-hand sides: CGLS reaches the same 1e-13
// relative gradient in one more iteration than with FP64 products, at ~55 %
// of their time per iteration.
constexpr int kDfFlush = 32;

__device__ __forceinline__ void df_mad(float a, float xh, float xl, float &sh, float &sl) {
  const float p = __fmul_rn(a, xh);
  float e = __fmaf_rn(a, xh, -p);
  e = __fmaf_rn(a, xl, e);
  // TwoSum(sh, p) = t + err exactly
  const float t = __fadd_rn(sh, p);
  const float z = __fadd_rn(t, -sh);
  const float err = __fadd_rn(__fadd_rn(sh, -__fadd_rn(t, -z)), __fadd_rn(p, -z));
  // Fast2Sum(t, u), |t| >= |u|: the renormalised pair
  const float u = __fadd_rn(sl, __fadd_rn(err, e));
  const float s2 = __fadd_rn(t, u);
  sl = __fadd_rn(u, -__fadd_rn(s2, -t));
  sh = s2;
}

// x = xh + xl with xh = fl32(x): the high part by rounding, the low part the
// FP32 rounding of the exact FP64 remainder
__device__ __forceinline__ void df_split(double x, float &xh, float &xl) {
  xh = (float)x;
  xl = (float)(x - widen(xh));
}

// Y[r, c] += alpha * sum_j A[r, j] X[j, c] for K right-hand sides (a
// compile-time count); the n columns are split over gridDim.y CTAs that add
// their partial sums with FP64 atomics.
template <int K>
__global__ void __launch_bounds__(TQR_THREADS)
k_gemm_sd_n(int m, int n, const float *__restrict__ A, int lda, const double *__restrict__ X,
            int ldx, double *__restrict__ Y, int ldy, double alpha, int jchunk)
{
  __shared__ float Xh[256][K], Xl[256][K];
  const int r = blockIdx.x * TQR_THREADS + threadIdx.x;
  const int j0 = blockIdx.y * jchunk, j1 = min(n, j0 + jchunk);
  double acc[K];
#pragma unroll
  for (int c = 0; c < K; ++c) acc[c] = 0.0;
  for (int jb = j0; jb < j1; jb += 256) {
    const int jn = min(256, j1 - jb);
    __syncthreads();
    for (int idx = threadIdx.x; idx < jn * K; idx += TQR_THREADS) {
      int jj = idx % jn, c = idx / jn;
      df_split(X[ix(jb + jj, c, ldx)], Xh[jj][c], Xl[jj][c]);
    }
    __syncthreads();
    if (r < m) {
      const float *ap = A + ix(r, jb, lda);
      for (int g0 = 0; g0 < jn; g0 += kDfFlush) {
        const int g1 = min(jn, g0 + kDfFlush);
        float sh[K], sl[K];
#pragma unroll
        for (int c = 0; c < K; ++c) sh[c] = sl[c] = 0.0f;
        int jj = g0;
        for (; jj + 16 <= g1; jj += 16) {    // sixteen loads of A in flight, then their terms in order
          float av[16];
#pragma unroll
          for (int u = 0; u < 16; ++u) av[u] = __ldg(ap + (size_t)(jj + u) * lda);
#pragma unroll
          for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int c = 0; c < K; ++c) df_mad(av[u], Xh[jj + u][c], Xl[jj + u][c], sh[c], sl[c]);
        }
        for (; jj < g1; ++jj) {
          const float a = __ldg(ap + (size_t)jj * lda);
#pragma unroll
          for (int c = 0; c < K; ++c) df_mad(a, Xh[jj][c], Xl[jj][c], sh[c], sl[c]);
        }
#pragma unroll
        for (int c = 0; c < K; ++c) acc[c] += widen(sh[c]) + widen(sl[c]);
      }
    }
  }
  if (r < m)
#pragma unroll
    for (int c = 0; c < K; ++c) atomicAdd(Y + ix(r, c, ldy), alpha * acc[c]);
}

// Z[j, c] += alpha * sum_r A[r, j] R[r, c] over the row block of this CTA;
// one warp per column, lanes over rows, one atomic add per (column, rhs).
template <int K>
__global__ void __launch_bounds__(TQR_THREADS)
k_gemm_sd_t(int m, int n, const float *__restrict__ A, int lda, const double *__restrict__ R,
            int ldr, double *__restrict__ Z, int ldz, double alpha, int rchunk, int cols_per_cta)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *Rh = reinterpret_cast<float *>(smem_raw);      // rchunk x K
  float *Rl = Rh + (size_t)rchunk * K;                  // rchunk x K
  const int r0 = blockIdx.x * rchunk, r1 = min(m, r0 + rchunk), rn = r1 - r0;
  const int j0 = blockIdx.y * cols_per_cta, j1 = min(n, j0 + cols_per_cta);
  for (int idx = threadIdx.x; idx < rn * K; idx += TQR_THREADS) {
    int rr = idx % rn, c = idx / rn;
    df_split(R[ix(r0 + rr, c, ldr)], Rh[rr + c * rchunk], Rl[rr + c * rchunk]);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = j0 + warp; j < j1; j += TQR_WARPS) {
    double acc[K];
#pragma unroll
    for (int c = 0; c < K; ++c) acc[c] = 0.0;
    const float *ap = A + ix(r0, j, lda);
    for (int g0 = 0; g0 < rn; g0 += 32 * kDfFlush) {
      const int g1 = min(rn, g0 + 32 * kDfFlush);
      float sh[K], sl[K];
#pragma unroll
      for (int c = 0; c < K; ++c) sh[c] = sl[c] = 0.0f;
      int rr = g0 + lane;
      for (; rr + 7 * 32 < g1; rr += 8 * 32) {    // eight loads of A in flight, then their terms in order
        float av[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) av[u] = __ldg(ap + rr + 32 * u);
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int c = 0; c < K; ++c)
            df_mad(av[u], Rh[rr + 32 * u + c * rchunk], Rl[rr + 32 * u + c * rchunk], sh[c], sl[c]);
      }
      for (; rr < g1; rr += 32) {
        const float a = __ldg(ap + rr);
#pragma unroll
        for (int c = 0; c < K; ++c) df_mad(a, Rh[rr + c * rchunk], Rl[rr + c * rchunk], sh[c], sl[c]);
      }
#pragma unroll
      for (int c = 0; c < K; ++c) acc[c] += widen(sh[c]) + widen(sl[c]);
    }
#pragma unroll
    for (int c = 0; c < K; ++c) {
      double v = warp_sum(acc[c]);
      if (lane == 0) atomicAdd(Z + ix(j, c, ldz), alpha * v);
    }
  }
}

// column-wise sums of squares of an m-by-k matrix into out[c] (FP64 atomics)
__global__ void k_colnorm2(int m, int k, const double *__restrict__ X, int ldx, double *out) {
  const int c = blockIdx.y;
  double s = 0.0;
  for (int r = blockIdx.x * TQR_THREADS + threadIdx.x; r < m; r += gridDim.x * TQR_THREADS) {
    double v = X[ix(r, c, ldx)];
    s = fma(v, v, s);
  }
  __shared__ double red[TQR_WARPS];
  s = block_sum(s, red);
  if (threadIdx.x == 0) atomicAdd(out + c, s);
}

// Y[:, c] += f(c) * X[:, c] with f = scale[c] (or -scale[c] when neg)
__global__ void k_axpy_cols(int m, int k, const double *__restrict__ scale, int neg, const double *__restrict__ X,
                            int ldx, double *__restrict__ Y, int ldy) {
  const int c = blockIdx.y;
  const double a = neg ? -scale[c] : scale[c];
  for (int r = blockIdx.x * TQR_THREADS + threadIdx.x; r < m; r += gridDim.x * TQR_THREADS)
    Y[ix(r, c, ldy)] = fma(a, X[ix(r, c, ldx)], Y[ix(r, c, ldy)]);
}

// P[:, c] = S[:, c] + beta[c] P[:, c]
__global__ void k_xpby_cols(int m, int k, const double *__restrict__ S, int lds, const double *__restrict__ beta,
                            double *__restrict__ P, int ldp) {
  const int c = blockIdx.y;
  const double b = beta[c];
  for (int r = blockIdx.x * TQR_THREADS + threadIdx.x; r < m; r += gridDim.x * TQR_THREADS)
    P[ix(r, c, ldp)] = fma(b, P[ix(r, c, ldp)], S[ix(r, c, lds)]);
}

// CGLS scalars: alpha = gamma / qq, then (after the new gamma) beta = gnew / gamma.
// A column whose preconditioned normal-equation residual has dropped below
// tol2 * g0 is frozen (alpha = 0): iterating past the attainable accuracy
// only feeds rounding noise back into the iterate.
__global__ void k_cgls_alpha(int k, const double *gamma, const double *qq, const double *g0, double tol2,
                             double *alpha) {
  const int c = threadIdx.x;
  if (c < k) alpha[c] = (qq[c] > 0.0 && gamma[c] > tol2 * g0[c]) ? gamma[c] / qq[c] : 0.0;
}
__global__ void k_cgls_beta(int k, double *gamma, const double *gnew, double *beta) {
  const int c = threadIdx.x;
  if (c < k) {
    beta[c] = (gamma[c] > 0.0) ? gnew[c] / gamma[c] : 0.0;
    gamma[c] = gnew[c];
  }
}

__global__ void k_f64_to_f32(long long n, const double *__restrict__ x, float *__restrict__ y) {
  for (long long i = blockIdx.x * (long long)TQR_THREADS + threadIdx.x; i < n; i += (long long)gridDim.x * TQR_THREADS)
    y[i] = (float)x[i];
}
__global__ void k_f32_to_f64_mat(int m, int k, const float *__restrict__ x, int ldx, double *__restrict__ y, int ldy) {
  const int c = blockIdx.y;
  for (int r = blockIdx.x * TQR_THREADS + threadIdx.x; r < m; r += gridDim.x * TQR_THREADS)
    y[ix(r, c, ldy)] = (double)x[ix(r, c, ldx)];
}
__global__ void k_f64_to_f32_mat(int m, int k, const double *__restrict__ x, int ldx, float *__restrict__ y, int ldy) {
  const int c = blockIdx.y;
  for (int r = blockIdx.x * TQR_THREADS + threadIdx.x; r < m; r += gridDim.x * TQR_THREADS)
    y[ix(r, c, ldy)] = (float)x[ix(r, c, ldx)];
}
__global__ void k_copy_f32_mat(int m, int n, const float *__restrict__ x, int ldx, float *__restrict__ y, int ldy) {
  for (long long idx = blockIdx.x * (long long)TQR_THREADS + threadIdx.x; idx < (long long)m * n;
       idx += (long long)gridDim.x * TQR_THREADS) {
    const int r = (int)(idx % m), c = (int)(idx / m);
    y[ix(r, c, ldy)] = x[ix(r, c, ldx)];
  }
}

static inline int blocks_for(long long n) { return (int)std::min<long long>(4096, (n + TQR_THREADS - 1) / TQR_THREADS); }

#define LS_CU(x)                            \
  do {                                      \
    cudaError_t _e = (x);                   \
    if (_e != cudaSuccess) return (int)_e;  \
  } while (0)
#define LS_TRY(x)                           \
  do {                                      \
    int _r = (x);                           \
    if (_r != 0) return _r;                 \
  } while (0)

template <int K>
static int gemm_sd_n_k(int m, int n, const float *A, int lda, const double *X, int ldx, double *Y, int ldy,
                       double alpha, cudaStream_t st) {
  const int gx = (m + TQR_THREADS - 1) / TQR_THREADS;
  int gy = std::max(1, std::min((n + 255) / 256, (8 * 152 + gx - 1) / gx));
  const int jchunk = ((n + gy - 1) / gy + 255) / 256 * 256;
  gy = (n + jchunk - 1) / jchunk;
  k_gemm_sd_n<K><<<dim3(gx, gy), TQR_THREADS, 0, st>>>(m, n, A, lda, X, ldx, Y, ldy, alpha, jchunk);
  count_launch();
  return (int)cudaGetLastError();
}

// Y = alpha A X + beta Y, beta 0 or 1 (right-hand sides in groups of 4, 2, 1)
static int gemm_sd_n(int m, int n, int k, const float *A, int lda, const double *X, int ldx, double *Y, int ldy,
                     double alpha, double beta, cudaStream_t st) {
  if (m <= 0 || k <= 0) return 0;
  if (beta == 0.0) {
    for (int c = 0; c < k; ++c) LS_CU(cudaMemsetAsync(Y + ix(0, c, ldy), 0, sizeof(double) * m, st));
  } else if (beta != 1.0) {
    return -1;   // not needed by the solver
  }
  if (n <= 0) return 0;
  for (int c = 0; c < k;) {
    const int rem = k - c;
    const double *Xc = X + ix(0, c, ldx);
    double *Yc = Y + ix(0, c, ldy);
    if (rem >= 4) { LS_TRY(gemm_sd_n_k<4>(m, n, A, lda, Xc, ldx, Yc, ldy, alpha, st)); c += 4; }
    else if (rem >= 2) { LS_TRY(gemm_sd_n_k<2>(m, n, A, lda, Xc, ldx, Yc, ldy, alpha, st)); c += 2; }
    else { LS_TRY(gemm_sd_n_k<1>(m, n, A, lda, Xc, ldx, Yc, ldy, alpha, st)); c += 1; }
  }
  return 0;
}

template <int K>
static int gemm_sd_t_k(int m, int n, const float *A, int lda, const double *R, int ldr, double *Z, int ldz,
                       double alpha, cudaStream_t st) {
  const int rchunk = 2048, cols = 64;
  dim3 grid((m + rchunk - 1) / rchunk, (n + cols - 1) / cols);
  const size_t sm = 2 * sizeof(float) * rchunk * K;   // 64 KB at K = 4: above the default limit
  LS_CU(cudaFuncSetAttribute(k_gemm_sd_t<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  k_gemm_sd_t<K><<<grid, TQR_THREADS, sm, st>>>(m, n, A, lda, R, ldr, Z, ldz, alpha, rchunk, cols);
  count_launch();
  return (int)cudaGetLastError();
}

// Z = alpha A^T R + beta Z (beta 0 or 1)
static int gemm_sd_t(int m, int n, int k, const float *A, int lda, const double *R, int ldr, double *Z, int ldz,
                     double alpha, double beta, cudaStream_t st) {
  if (n <= 0 || k <= 0) return 0;
  if (beta == 0.0) {
    for (int c = 0; c < k; ++c) LS_CU(cudaMemsetAsync(Z + ix(0, c, ldz), 0, sizeof(double) * n, st));
  } else if (beta != 1.0) {
    return -1;
  }
  if (m <= 0) return 0;
  for (int c = 0; c < k;) {
    const int rem = k - c;
    const double *Rc = R + ix(0, c, ldr);
    double *Zc = Z + ix(0, c, ldz);
    if (rem >= 4) { LS_TRY(gemm_sd_t_k<4>(m, n, A, lda, Rc, ldr, Zc, ldz, alpha, st)); c += 4; }
    else if (rem >= 2) { LS_TRY(gemm_sd_t_k<2>(m, n, A, lda, Rc, ldr, Zc, ldz, alpha, st)); c += 2; }
    else { LS_TRY(gemm_sd_t_k<1>(m, n, A, lda, Rc, ldr, Zc, ldz, alpha, st)); c += 1; }
  }
  return 0;
}

// ---- triangular solves through inverted diagonal blocks -------------------
// A serial back substitution costs ~450 cycles per row on GB300 (every FP64
// instruction holds the pipe ~64 cycles), so the refinement inverts R's
// 256-by-256 diagonal blocks once (in parallel, FP64) and every later solve
// is a chain of small parallel products.

// Rinv_b = R_bb^-1 (FP64, upper, 256-by-256 per block, ld 256) for column
// chunk blockIdx.y (16 columns of the identity) of block blockIdx.x.
__global__ void __launch_bounds__(TQR_THREADS)
k_trinv_diag(int n, const float *__restrict__ Rm, int ldr, double *__restrict__ Rinv, double *__restrict__ RinvT)
{
  __shared__ double x[256][17];
  __shared__ double rinv[256];
  const int b = blockIdx.x, b0 = b * 256, nbk = min(256, n - b0);
  const int c0 = blockIdx.y * 16;
  if (c0 >= nbk) return;
  const int nc = min(16, nbk - c0);
  const float *R = Rm + ix(b0, b0, ldr);
  double *out = Rinv + (size_t)b * 256 * 256;
  for (int idx = threadIdx.x; idx < nbk; idx += TQR_THREADS) rinv[idx] = 1.0 / (double)R[ix(idx, idx, ldr)];
  for (int idx = threadIdx.x; idx < 256 * 16; idx += TQR_THREADS) {
    int r = idx % 256, c = idx / 256;
    x[r][c] = (r == c0 + c) ? 1.0 : 0.0;
  }
  __syncthreads();
  const int t = threadIdx.x;
  // rows above c0 + nc - 1 are the only ones the identity columns reach
  for (int i = c0 + nc - 1; i >= 0; --i) {
    if (t < nc) x[i][t] *= rinv[i];
    __syncthreads();
    if (t < i) {
      const double a = (double)R[ix(t, i, ldr)];
      for (int c = 0; c < nc; ++c) x[t][c] = fma(-a, x[i][c], x[t][c]);
    }
    __syncthreads();
  }
  double *outT = RinvT ? RinvT + (size_t)b * 256 * 256 : nullptr;
  for (int idx = threadIdx.x; idx < 256 * nc; idx += TQR_THREADS) {
    int r = idx % 256, c = idx / 256;
    const double v = (r < nbk) ? x[r][c] : 0.0;
    out[ix(r, c0 + c, 256)] = v;
    if (outT) outT[ix(c0 + c, r, 256)] = v;
  }
}

// X_b = op(Rinv_b) B_b for one diagonal block: trans 0 uses Rinv_b (upper),
// trans 1 its transpose.  Threads: consecutive rows in a warp, k columns.
__global__ void __launch_bounds__(TQR_THREADS)
k_blk_solve(int trans, int nbk, int k, const double *__restrict__ Ri, const double *__restrict__ B, int ldb,
            double *__restrict__ X, int ldx)
{
  const int rows = TQR_THREADS / k;
  const int r = blockIdx.x * rows + threadIdx.x % rows, c = threadIdx.x / rows;
  if (c >= k || r >= nbk || threadIdx.x >= rows * k) return;
  const double *bc = B + ix(0, c, ldb);
  double s0 = 0.0, s1 = 0.0;
  if (!trans) {
    int q = r;
    for (; q + 1 < nbk; q += 2) {
      s0 = fma(Ri[ix(r, q, 256)], bc[q], s0);
      s1 = fma(Ri[ix(r, q + 1, 256)], bc[q + 1], s1);
    }
    if (q < nbk) s0 = fma(Ri[ix(r, q, 256)], bc[q], s0);
  } else {
    int q = 0;
    for (; q + 1 <= r; q += 2) {
      s0 = fma(Ri[ix(q, r, 256)], bc[q], s0);
      s1 = fma(Ri[ix(q + 1, r, 256)], bc[q + 1], s1);
    }
    if (q <= r) s0 = fma(Ri[ix(q, r, 256)], bc[q], s0);
  }
  X[ix(r, c, ldx)] = s0 + s1;
}

static int trinv_diag(int n, const float *Rm, int ldr, double *Rinv, double *RinvT, cudaStream_t st) {
  const int nblk = (n + 255) / 256;
  k_trinv_diag<<<dim3(nblk, 16), TQR_THREADS, 0, st>>>(n, Rm, ldr, Rinv, RinvT);
  count_launch();
  return (int)cudaGetLastError();
}

// ---- the same solve as one cooperative persistent launch ------------------
// The blocked solve is a chain of 2 * n / 256 small products; launched one by
// one they are launch- and latency-bound.  Here every CTA of one cooperative
// grid takes rows of each step and the steps are separated by a grid
// barrier (bounded spin, error word on timeout).
struct GridBar {
  int count;
  int gen;
  int error;
  int pad[61];
};
static_assert(sizeof(GridBar) == 256, "GridBar layout");

__device__ __forceinline__ int ls_ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// All CTAs of the grid; false (in every thread of every CTA that gets here)
// once any wait has timed out.
__device__ bool grid_sync(GridBar *gb, unsigned nblocks) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const int g = ls_ld_acquire(&gb->gen);
    __threadfence();
    if (atomicAdd(&gb->count, 1) == (int)nblocks - 1) {
      atomicExch(&gb->count, 0);
      __threadfence();
      atomicAdd(&gb->gen, 1);
    } else {
      unsigned long long t0, t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      while (ls_ld_acquire(&gb->gen) == g) {
        if (ls_ld_acquire(&gb->error)) { ok = 0; break; }
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > 2000000000ull) { atomicExch(&gb->error, 1); ok = 0; break; }
        __nanosleep(64);
      }
    }
    if (ls_ld_acquire(&gb->error)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// X = op(R)^-1 B, op = R (trans 0, backward over the blocks) or R^T (trans
// 1, forward).  Rinv holds R's inverted 256 x 256 diagonal blocks (ld 256)
// and RinvT their transposes, so both directions read them along columns; B
// is consumed.  Per step: X_b = op(Rinv_b) B_b with one warp per row (lanes
// split the 256-term sum), then the other rows' update -- R^T: one warp per
// row again; R: lanes over 32 consecutive rows, warps over eight 32-column
// parts of the block, combined with FP64 atomics.
template <int K>
__global__ void __launch_bounds__(TQR_THREADS)
k_trsv_coop(int trans, int n, const float *__restrict__ Rm, int ldr, const double *__restrict__ Rinv,
            const double *__restrict__ RinvT, double *B, int ldb, double *X, int ldx, GridBar *gb) {
  const int nblk = (n + 255) / 256;
  const int lane = threadIdx.x & 31;
  const int gwarp = blockIdx.x * TQR_WARPS + (threadIdx.x >> 5), nwarps = gridDim.x * TQR_WARPS;
  for (int q = 0; q < nblk; ++q) {
    const int b = trans ? q : nblk - 1 - q;
    const int b0 = b * 256, nbk = min(256, n - b0);
    // column r of M holds op(Rinv_b)[r][.]: RinvT for R (row r of Rinv_b), Rinv for R^T
    const double *M = (trans ? Rinv : RinvT) + (size_t)b * 65536;
    for (int r = gwarp; r < nbk; r += nwarps) {
      double acc[K];
#pragma unroll
      for (int c = 0; c < K; ++c) acc[c] = 0.0;
      const int q0 = trans ? 0 : r, q1 = trans ? r + 1 : nbk;
      for (int qq = q0 + lane; qq < q1; qq += 32) {
        const double a = M[ix(qq, r, 256)];
#pragma unroll
        for (int c = 0; c < K; ++c) acc[c] = fma(a, __ldcg(B + ix(b0 + qq, c, ldb)), acc[c]);
      }
#pragma unroll
      for (int c = 0; c < K; ++c) {
        const double v = warp_sum(acc[c]);
        if (lane == 0) X[ix(b0 + r, c, ldx)] = v;
      }
    }
    __threadfence();
    if (!grid_sync(gb, gridDim.x)) return;
    if (trans) {
      // rows r >= b0 + nbk: B[r] -= sum_j R[b0 + j][r] X[b0 + j]
      for (int r = b0 + nbk + gwarp; r < n; r += nwarps) {
        double acc[K];
#pragma unroll
        for (int c = 0; c < K; ++c) acc[c] = 0.0;
        for (int j = lane; j < nbk; j += 32) {
          const double a = widen(Rm[ix(b0 + j, r, ldr)]);
#pragma unroll
          for (int c = 0; c < K; ++c) acc[c] = fma(a, __ldcg(X + ix(b0 + j, c, ldx)), acc[c]);
        }
#pragma unroll
        for (int c = 0; c < K; ++c) {
          const double v = warp_sum(acc[c]);
          if (lane == 0) B[ix(r, c, ldb)] -= v;
        }
      }
    } else if (b0 > 0) {
      // rows r < b0: B[r] -= sum_j R[r][b0 + j] X[b0 + j]; item = (32-row group, 32-column part)
      const int groups = (b0 + 31) / 32, parts = (nbk + 31) / 32;
      for (int item = gwarp; item < groups * parts; item += nwarps) {
        const int r = (item % groups) * 32 + lane, j0 = (item / groups) * 32, j1 = min(nbk, j0 + 32);
        if (r < b0) {
          double acc[K];
#pragma unroll
          for (int c = 0; c < K; ++c) acc[c] = 0.0;
          for (int j = j0; j < j1; ++j) {
            const double a = widen(Rm[ix(r, b0 + j, ldr)]);
#pragma unroll
            for (int c = 0; c < K; ++c) acc[c] = fma(a, __ldcg(X + ix(b0 + j, c, ldx)), acc[c]);
          }
#pragma unroll
          for (int c = 0; c < K; ++c) atomicAdd(B + ix(r, c, ldb), -acc[c]);
        }
      }
    }
    __threadfence();
    if (!grid_sync(gb, gridDim.x)) return;
  }
}

// ---- the same solve as a pipelined task list (no grid barrier) ------------
// The cooperative form above spends most of its time in its 2 n / 256 grid
// barriers.  Here the 256-row blocks are taken in solve order s = 0, 1, ...
// (trans 0: the last block first; trans 1: the first block first), and the
// work is cut into tasks of kPipeRows rows (one warp per row) of a block:
//   X(s, p):    X_s[rows] = op(Rinv_s) B_s            needs every chain U(s, ., q) complete
//   U(t, s, p): B_t[rows] -= op(R)_{t,s} X_s, s < t   needs X(s) and U(t, s - 1, p)
// listed as X(0); then for s = 1 .. nblk - 1: U(s, s - 1), X(s), and
// U(t, s - 1) for t = s + 1 .. nblk - 1.  The critical chain per block is
// one U and one X, the other U tasks fill the machine meanwhile.  Every
// dependency is an earlier task and CTAs take tasks in list order, so the
// first unfinished task can always run.  Each B row is updated by one chain
// in source order and every sum runs in a fixed order: the result does not
// depend on timing.  Flags (ints): [0] next task, [1] error (stops this
// launch), [2] sticky error (kept across launches until the solve reads it),
// then X parts done per block, U chains completed per block, and per
// (block, row part) the sources applied so far.
constexpr int kPipeRows = TQR_WARPS;
constexpr int kPipeParts = 256 / kPipeRows;

__host__ __device__ inline int pipe_units(int nblk) { return 1 + (nblk - 1) * (nblk + 2) / 2; }
__host__ __device__ inline size_t pipe_flag_ints(int nblk) { return 4 + 2 * (size_t)nblk + (size_t)nblk * kPipeParts; }

// Unit u of the list: kind 0 = X(t), 1 = U(t, s).
__host__ __device__ inline void pipe_unit(int u, int nblk, int &kind, int &t, int &s) {
  kind = 0; t = 0; s = 0;
  if (u == 0) return;
  int rem = u - 1;
  for (int q = 1; q < nblk; ++q) {
    const int len = nblk + 1 - q;
    if (rem < len) {
      if (rem == 1) { kind = 0; t = q; }
      else { kind = 1; t = rem == 0 ? q : q + rem - 1; s = q - 1; }
      return;
    }
    rem -= len;
  }
  kind = -1;
}

__device__ inline bool pipe_wait(const int *f, int target, int *err) {
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  while (ls_ld_acquire(f) < target) {
    if (ls_ld_acquire(err)) return false;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > 2000000000ull) {
      atomicExch(err, 1);
      atomicExch(err + 1, 1);
      return false;
    }
    __nanosleep(32);
  }
  return true;
}

template <int K>
__global__ void __launch_bounds__(TQR_THREADS)
k_trsv_pipe(int trans, int n, const float *__restrict__ Rm, int ldr, const double *__restrict__ Rinv,
            const double *__restrict__ RinvT, double *B, int ldb, double *X, int ldx, int *flags) {
  __shared__ int s_task, s_ok;
  __shared__ double part[TQR_WARPS][kPipeRows][K];
  const int nblk = (n + 255) / 256, ntask = pipe_units(nblk) * kPipeParts;
  int *xdone = flags + 4, *ucnt = xdone + nblk, *uprog = ucnt + nblk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(flags, 1);
    __syncthreads();
    const int task = s_task;
    if (task >= ntask) return;
    const int pr = task % kPipeParts;
    int kind, t, s;
    pipe_unit(task / kPipeParts, nblk, kind, t, s);
    const int bt = trans ? t : nblk - 1 - t, bt0 = bt * 256, nbt = min(256, n - bt0);
    const int bs = trans ? s : nblk - 1 - s, bs0 = bs * 256, nbs = min(256, n - bs0);
    const int r0 = pr * kPipeRows;
    // The matrix operand of the task (an inverted diagonal block or a block
    // of R) does not depend on other tasks: its eight values per lane are
    // loaded before the wait, so only X or B is read after it.
    double mv[8];
    int jv[8];
    if (kind == 0) {
      // X_t rows: column r of M holds op(Rinv_t)[r][.]; lane takes q = q0 + lane + 32 u
      const int r = r0 + warp;
      const double *M = (trans ? Rinv : RinvT) + (size_t)bt * 65536;
      const int q0 = trans ? 0 : r, q1 = trans ? r + 1 : nbt;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int qq = q0 + lane + 32 * u;
        jv[u] = (r < nbt && qq < q1) ? qq : -1;
        mv[u] = jv[u] >= 0 ? M[ix(qq, r, 256)] : 0.0;
      }
    } else if (trans) {
      // R^T: row r of B_t takes column bt0 + r of R's block (s, t), lanes along it
      const int r = r0 + warp;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = lane + 32 * u;
        jv[u] = (r < nbt && j < nbs) ? j : -1;
        mv[u] = jv[u] >= 0 ? widen(Rm[ix(bs0 + j, bt0 + r, ldr)]) : 0.0;
      }
    } else {
      // R: the task's rows are 8 consecutive entries of each column of R's
      // block (t, s); warp w takes columns [32 w, 32 w + 32), lane = row +
      // 8 x (column mod 4)
      const int rr = lane & 7, jj = lane >> 3, r = r0 + rr;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = 32 * warp + jj + 4 * u;
        jv[u] = (r < nbt && j < nbs) ? j : -1;
        mv[u] = jv[u] >= 0 ? widen(Rm[ix(bt0 + r, bs0 + j, ldr)]) : 0.0;
      }
    }
    if (threadIdx.x == 0) {
      bool ok = true;
      if (kind == 0 && t > 0) ok = pipe_wait(ucnt + t, kPipeParts, flags + 1);
      if (kind == 1) ok = pipe_wait(xdone + s, kPipeParts, flags + 1) && pipe_wait(uprog + t * kPipeParts + pr, s, flags + 1);
      s_ok = ok && kind >= 0;
    }
    __syncthreads();
    if (!s_ok) return;
    // the dependent operand (B_t for X, X_s for U), all eight terms in flight
    const double *src = kind == 0 ? B + bt0 : X + bs0;
    const int lds = kind == 0 ? ldb : ldx;
    double acc[K];
#pragma unroll
    for (int c = 0; c < K; ++c) acc[c] = 0.0;
    {
      double xv[8][K];
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int c = 0; c < K; ++c) xv[u][c] = jv[u] >= 0 ? __ldcg(src + ix(jv[u], c, lds)) : 0.0;
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int c = 0; c < K; ++c) acc[c] = fma(mv[u], xv[u][c], acc[c]);
    }
    if (kind == 0 || trans) {
      const int r = r0 + warp;
#pragma unroll
      for (int c = 0; c < K; ++c) {
        const double v = warp_sum(acc[c]);
        if (lane == 0 && r < nbt) {
          if (kind == 0) X[ix(bt0 + r, c, ldx)] = v;
          else B[ix(bt0 + r, c, ldb)] = __ldcg(B + ix(bt0 + r, c, ldb)) - v;
        }
      }
    } else {
      // a fixed-order sum over the lanes of one row, then over the warps
      const int rr = lane & 7, jj = lane >> 3;
#pragma unroll
      for (int c = 0; c < K; ++c) {
        acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 8);
        acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 16);
        if (jj == 0) part[warp][rr][c] = acc[c];
      }
      __syncthreads();
      if (threadIdx.x < kPipeRows * K) {
        const int q = threadIdx.x % kPipeRows, c = threadIdx.x / kPipeRows;
        if (r0 + q < nbt) {
          double v = 0.0;
#pragma unroll
          for (int w = 0; w < TQR_WARPS; ++w) v += part[w][q][c];
          B[ix(bt0 + r0 + q, c, ldb)] = __ldcg(B + ix(bt0 + r0 + q, c, ldb)) - v;
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (kind == 0) {
        atomicAdd(xdone + t, 1);
      } else {
        asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(uprog + t * kPipeParts + pr), "r"(s + 1) : "memory");
        if (s == t - 1) atomicAdd(ucnt + t, 1);
      }
    }
  }
}

template <int K>
static int trsv_pipe_k(int trans, int n, const float *Rm, int ldr, const double *Rinv, const double *RinvT, double *B,
                       int ldb, double *X, int ldx, int *flags, cudaStream_t st) {
  int dev = 0, sms = 0, per = 0;
  LS_CU(cudaGetDevice(&dev));
  LS_CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  LS_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trsv_pipe<K>, TQR_THREADS, 0));
  if (per < 1) return (int)cudaErrorInvalidConfiguration;
  const int nblk = (n + 255) / 256;
  const int ntask = pipe_units(nblk) * kPipeParts;
  // everything but the sticky error word
  LS_CU(cudaMemsetAsync(flags, 0, sizeof(int) * 2, st));
  LS_CU(cudaMemsetAsync(flags + 4, 0, sizeof(int) * (pipe_flag_ints(nblk) - 4), st));
  k_trsv_pipe<K><<<std::min(sms * std::min(per, 2), ntask), TQR_THREADS, 0, st>>>(trans, n, Rm, ldr, Rinv, RinvT,
                                                                                  B, ldb, X, ldx, flags);
  count_launch();
  LS_CU(cudaGetLastError());
  return 0;
}

// Whether the mixed solve's CGLS runs its triangular solves as the pipelined
// task list (tqr_dsgels_trsv_pipelined) or with grid barriers.
static int g_trsv_pipe = 1;

template <int K>
static int trsv_coop_k(int trans, int n, const float *Rm, int ldr, const double *Rinv, const double *RinvT, double *B,
                       int ldb, double *X, int ldx, GridBar *gb, cudaStream_t st) {
  int dev = 0, sms = 0, per = 0;
  LS_CU(cudaGetDevice(&dev));
  LS_CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  LS_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trsv_coop<K>, TQR_THREADS, 0));
  if (per < 1) return (int)cudaErrorInvalidConfiguration;
  const int grid = sms * std::min(per, 2);
  LS_CU(cudaMemsetAsync(gb, 0, sizeof(GridBar), st));
  void *args[] = {&trans, &n, &Rm, &ldr, &Rinv, &RinvT, &B, &ldb, &X, &ldx, &gb};
  LS_CU(cudaLaunchCooperativeKernel((const void *)k_trsv_coop<K>, dim3(grid), dim3(TQR_THREADS), args, 0, st));
  count_launch();
  return 0;
}

// X = op(R)^-1 B in one cooperative launch (k = 1, 2, 4; others fall back to
// the launch-per-step form below).
static int trsv_coop(int trans, int n, int k, const float *Rm, int ldr, const double *Rinv, const double *RinvT,
                     double *B, int ldb, double *X, int ldx, GridBar *gb, cudaStream_t st);

// X = op(R)^-1 B for the FP32 upper R with its inverted diagonal blocks; B
// (n-by-k) is consumed as scratch, X receives the solution.
static int trsm_sd_inv(int trans, int n, int k, const float *Rm, int ldr, const double *Rinv, double *B, int ldb,
                       double *X, int ldx, cudaStream_t st) {
  const int nblk = (n + 255) / 256;
  const int rows = TQR_THREADS / k;
  for (int q = 0; q < nblk; ++q) {
    const int b = trans ? q : nblk - 1 - q;
    const int b0 = b * 256, nbk = std::min(256, n - b0);
    k_blk_solve<<<(nbk + rows - 1) / rows, TQR_THREADS, 0, st>>>(trans, nbk, k, Rinv + (size_t)b * 65536,
                                                                B + b0, ldb, X + b0, ldx);
    count_launch();
    LS_CU(cudaGetLastError());
    if (!trans && b0 > 0) {
      LS_TRY(gemm_sd_n(b0, nbk, k, Rm + ix(0, b0, ldr), ldr, X + b0, ldx, B, ldb, -1.0, 1.0, st));
    } else if (trans && b0 + nbk < n) {
      const int b1 = b0 + nbk;
      LS_TRY(gemm_sd_t(nbk, n - b1, k, Rm + ix(b0, b1, ldr), ldr, X + b0, ldx, B + b1, ldb, -1.0, 1.0, st));
    }
  }
  return 0;
}

static int trsv_coop(int trans, int n, int k, const float *Rm, int ldr, const double *Rinv, const double *RinvT,
                     double *B, int ldb, double *X, int ldx, GridBar *gb, cudaStream_t st) {
  if (g_trsv_pipe) {
    int *flags = reinterpret_cast<int *>(gb);
    switch (k) {
      case 4: return trsv_pipe_k<4>(trans, n, Rm, ldr, Rinv, RinvT, B, ldb, X, ldx, flags, st);
      case 2: return trsv_pipe_k<2>(trans, n, Rm, ldr, Rinv, RinvT, B, ldb, X, ldx, flags, st);
      case 1: return trsv_pipe_k<1>(trans, n, Rm, ldr, Rinv, RinvT, B, ldb, X, ldx, flags, st);
      default: break;
    }
  }
  switch (k) {
    case 4: return trsv_coop_k<4>(trans, n, Rm, ldr, Rinv, RinvT, B, ldb, X, ldx, gb, st);
    case 2: return trsv_coop_k<2>(trans, n, Rm, ldr, Rinv, RinvT, B, ldb, X, ldx, gb, st);
    case 1: return trsv_coop_k<1>(trans, n, Rm, ldr, Rinv, RinvT, B, ldb, X, ldx, gb, st);
    default: return trsm_sd_inv(trans, n, k, Rm, ldr, Rinv, B, ldb, X, ldx, st);
  }
}

static int colnorm2(int m, int k, const double *X, int ldx, double *out, cudaStream_t st) {
  LS_CU(cudaMemsetAsync(out, 0, sizeof(double) * k, st));
  k_colnorm2<<<dim3(std::min(256, blocks_for(m)), k), TQR_THREADS, 0, st>>>(m, k, X, ldx, out);
  count_launch();
  return (int)cudaGetLastError();
}

static int axpy_cols(int m, int k, const double *scale, int neg, const double *X, int ldx, double *Y, int ldy,
                     cudaStream_t st) {
  k_axpy_cols<<<dim3(blocks_for(m), k), TQR_THREADS, 0, st>>>(m, k, scale, neg, X, ldx, Y, ldy);
  count_launch();
  return (int)cudaGetLastError();
}

// Phase times of the last tqr_dsgels call (FP32 factorisation, X0, CGLS), from
// CUDA events on the solve's stream; read by tqr_dsgels_phases.
static double g_phase_ms[3] = {0, 0, 0};
static int g_phase_iters = 0;

struct PhaseTimer {
  cudaStream_t st;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool ok = true;
  explicit PhaseTimer(cudaStream_t s) : st(s) {
    for (auto &e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    if (ok) cudaEventRecord(ev[0], st);
  }
  void mark(int i) {
    if (ok) cudaEventRecord(ev[i], st);
  }
  void finish(int iters) {
    if (!ok) return;
    cudaEventSynchronize(ev[3]);
    for (int i = 0; i < 3; ++i) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      g_phase_ms[i] = t;
    }
    g_phase_iters = iters;
  }
  ~PhaseTimer() {
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  }
};

// Workspace layout (bytes, each piece 256-aligned)
struct MixedWs {
  size_t F, T, tau, T2, tau2, dag, x32, r, s, p, t, q, sc, rinv, rinvt, tmpn, gbar, total;
};

// Factorisation schedule of tqr_dsgels: grp > 0 = the hierarchical tree with
// groups of grp tiles for matrices of at least 2 grp tile rows (the FP64
// panel steps make the flat tree's tsqrt chain per panel the critical path:
// 32768 x 4096 factors in 86.8 ms with groups of 16 against 109.4 ms flat);
// 0 = always the flat tree (tqr_dsgels_hqr_group).
static int g_dsgels_grp = 16;

// (the hierarchical form exists with FP64 panel steps only: with
// tqr_dsgels_fp64_panels(0) the solve uses the flat tree)
static bool use_hqr(int m, int n, int nb, int ib) {
  return g_dsgels_grp > 0 && dsgels_f64p_enabled() && m % nb == 0 && n % nb == 0 && ib <= 32 && m / nb >= 2 * g_dsgels_grp;
}

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

static int mixed_ws(int m, int n, int k, int nb, int ib, MixedWs *w) {
  const int MT = (m + nb - 1) / nb;
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += a256(bytes); return o; };
  w->F = take(sizeof(float) * (size_t)m * n);
  w->T = take(sizeof(float) * (size_t)MT * ib * n);
  w->tau = take(sizeof(float) * (size_t)n * MT);
  w->T2 = take(sizeof(float) * (size_t)MT * ib * n);
  w->tau2 = take(sizeof(float) * (size_t)n * MT);
  size_t dag = 0;
  if (tqr_tile_gels_worksize(m, n, k, nb, ib, &dag) != 0) dag = 0;
  if (use_hqr(m, n, nb, ib)) dag = std::max(dag, tree_dag_work_bytes(m, n, nb, ib, g_dsgels_grp, k));
  w->dag = take(dag ? dag : 256);
  w->x32 = take(sizeof(float) * (size_t)m * k);
  w->r = take(sizeof(double) * (size_t)m * k);
  w->s = take(sizeof(double) * (size_t)n * k);
  w->p = take(sizeof(double) * (size_t)n * k);
  w->t = take(sizeof(double) * (size_t)n * k);
  w->q = take(sizeof(double) * (size_t)m * k);
  w->sc = take(sizeof(double) * 8 * kLsMaxRhs);
  w->rinv = take(sizeof(double) * 65536 * (size_t)((n + 255) / 256));
  w->rinvt = take(sizeof(double) * 65536 * (size_t)((n + 255) / 256));
  w->tmpn = take(sizeof(double) * (size_t)n * k);
  w->gbar = take(std::max(sizeof(GridBar), sizeof(int) * pipe_flag_ints((n + 255) / 256)));
  w->total = off;
  return dag ? 0 : 1;
}

}  // namespace tqr

using namespace tqr;

extern "C" {

int tqr_dsgels_phases(double *ms, int *iters) {
  if (ms)
    for (int i = 0; i < 3; ++i) ms[i] = g_phase_ms[i];
  if (iters) *iters = g_phase_iters;
  return 0;
}

int tqr_dsgels_trsv_pipe_check(int n, long long *ntasks) {
  // Host replay of the pipelined solve's task list in list order: every wait
  // is on work finished earlier in the list, each row part applies its
  // sources in order 0, 1, ..., t - 1 before X(t), and every X and U runs once.
  if (n <= 0) return -1;
  const int nblk = (n + 255) / 256, nu = pipe_units(nblk);
  std::vector<int> xdone(nblk, 0), ucnt(nblk, 0), uprog((size_t)nblk * kPipeParts, 0);
  std::vector<int> seen_x(nblk, 0), seen_u((size_t)nblk * nblk, 0);
  long long nt = 0;
  for (int u = 0; u < nu; ++u) {
    int kind, t, s;
    pipe_unit(u, nblk, kind, t, s);
    if (kind < 0 || t < 0 || t >= nblk) return 1;
    if (kind == 0) {
      if (seen_x[t]++) return 2;
      if (t > 0 && ucnt[t] < kPipeParts) return 3;
    } else {
      if (s < 0 || s >= t || seen_u[(size_t)t * nblk + s]++) return 4;
      if (xdone[s] < kPipeParts) return 5;
    }
    for (int pr = 0; pr < kPipeParts; ++pr, ++nt) {
      if (kind == 0) {
        ++xdone[t];
      } else {
        int &g = uprog[(size_t)t * kPipeParts + pr];
        if (g != s) return 6;
        g = s + 1;
        if (s == t - 1) ++ucnt[t];
      }
    }
  }
  for (int t = 0; t < nblk; ++t) {
    if (!seen_x[t]) return 7;
    for (int s = 0; s < t; ++s)
      if (!seen_u[(size_t)t * nblk + s]) return 8;
  }
  if (ntasks) *ntasks = nt;
  return 0;
}

int tqr_dsgels_trsv_pipelined(int on) {
  const int old = g_trsv_pipe;
  g_trsv_pipe = on ? 1 : 0;
  return old;
}

int tqr_dsgels_hqr_group(int grp) {
  const int old = g_dsgels_grp;
  g_dsgels_grp = grp > 0 ? grp : 0;
  return old;
}

int tqr_dsgels_worksize(int m, int n, int nrhs, int nb, int ib, size_t *bytes) {
  if (!bytes) return -6;
  MixedWs w;
  mixed_ws(m, n, nrhs, nb, ib, &w);
  *bytes = w.total;
  return 0;
}

int tqr_dsgels(int m, int n, int nrhs, int nb, int ib, const float *A, int lda, const double *B, int ldb,
               double *X, int ldx, int maxit, double tol, void *work, size_t lwork, int *iters,
               double *relres, cudaStream_t stream) {
  if (m < 0) return -1;
  if (n < 0 || n > m) return -2;
  if (nrhs < 0 || nrhs > kLsMaxRhs) return -3;
  if (nb <= 0 || nb > 256) return -4;
  if (ib <= 0 || ib > nb || nb % ib) return -5;
  if (lda < m) return -7;
  if (ldb < m) return -9;
  if (ldx < n) return -11;
  if (maxit < 0) return -12;
  if (m == 0 || n == 0 || nrhs == 0) {
    if (iters) *iters = 0;
    return 0;
  }
  MixedWs w;
  mixed_ws(m, n, nrhs, nb, ib, &w);
  if (!work || ((uintptr_t)work & 255)) return -14;
  if (lwork < w.total) return -15;
  unsigned char *base = (unsigned char *)work;
  float *F = (float *)(base + w.F);
  float *T = (float *)(base + w.T);
  float *tau = (float *)(base + w.tau);
  float *x32 = (float *)(base + w.x32);
  double *r = (double *)(base + w.r), *s = (double *)(base + w.s), *p = (double *)(base + w.p);
  double *t = (double *)(base + w.t), *q = (double *)(base + w.q), *sc = (double *)(base + w.sc);
  double *gamma = sc, *gnew = sc + kLsMaxRhs, *qq = sc + 2 * kLsMaxRhs, *alpha = sc + 3 * kLsMaxRhs,
         *beta = sc + 4 * kLsMaxRhs, *g0d = sc + 5 * kLsMaxRhs;
  const int MT = (m + nb - 1) / nb, k = nrhs;
  cudaStream_t st = stream;
  PhaseTimer pt(st);
  // 1. tile QR of a copy of A: FP32 updates, FP64 panels
  k_copy_f32_mat<<<blocks_for((long long)m * n), TQR_THREADS, 0, st>>>(m, n, A, lda, F, m);
  count_launch();
  LS_CU(cudaGetLastError());
  k_f64_to_f32_mat<<<dim3(blocks_for(m), k), TQR_THREADS, 0, st>>>(m, k, B, ldb, x32, m);
  count_launch();
  LS_CU(cudaGetLastError());
  size_t dagb = 0;
  float *T2 = (float *)(base + w.T2), *tau2 = (float *)(base + w.tau2);
  if (use_hqr(m, n, nb, ib) && tree_dag_work_bytes(m, n, nb, ib, g_dsgels_grp, k) > 0) {
    // the hierarchical tree: B rides along as extra trailing columns
    LS_TRY(stile_gels_hqr_mixed(m, n, k, nb, ib, g_dsgels_grp, F, m, T, T2, MT * ib, tau, tau2, n, x32, m,
                                base + w.dag, w.x32 - w.dag, st));
    pt.mark(1);
  } else if (tqr_tile_gels_worksize(m, n, k, nb, ib, &dagb) == 0) {
    // 1+2 in one persistent launch: B (in FP32) rides along as an extra tile
    // column, so the factorisation leaves Q^T B behind; then R X0 = (Q^T B)[0:n]
    LS_TRY(stile_gels_dag_mixed(m, n, k, nb, ib, F, m, T, MT * ib, tau, n, x32, m, base + w.dag, dagb, st));
    pt.mark(1);
  } else {
    LS_TRY(tqr_stile_geqrf(m, n, nb, ib, F, m, T, MT * ib, tau, n, st));
    pt.mark(1);
    LS_TRY(tqr_stile_unmqr('C', m, n, k, nb, ib, F, m, T, MT * ib, x32, m, st));
    LS_TRY(tqr_strsm_lun(n, k, F, m, x32, m, st));
  }
  // 2. X0 = R^-1 (Q^T B)[0:n] in FP32, promoted
  k_f32_to_f64_mat<<<dim3(blocks_for(n), k), TQR_THREADS, 0, st>>>(n, k, x32, m, X, ldx);
  count_launch();
  LS_CU(cudaGetLastError());
  pt.mark(2);
  // 3. CGLS on min ||A R^-1 Y - B||, tracking X = R^-1 Y
  //    r = B - A X
  for (int c = 0; c < k; ++c)
    LS_CU(cudaMemcpyAsync(r + ix(0, c, m), B + ix(0, c, ldb), sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
  LS_TRY(gemm_sd_n(m, n, k, A, lda, X, ldx, r, m, -1.0, 1.0, st));
  //    R's diagonal blocks inverted once; s = R^-T A^T r ; p = s ; gamma = |s|^2
  double *Rinv = (double *)(base + w.rinv), *tmpn = (double *)(base + w.tmpn);
  double *RinvT = (double *)(base + w.rinvt);
  GridBar *gbar = (GridBar *)(base + w.gbar);
  int *sticky = reinterpret_cast<int *>(gbar) + 2;   // the pipelined solves' sticky error word
  LS_CU(cudaMemsetAsync(sticky, 0, sizeof(int), st));
  LS_TRY(trinv_diag(n, F, m, Rinv, RinvT, st));
  LS_TRY(gemm_sd_t(m, n, k, A, lda, r, m, tmpn, n, 1.0, 0.0, st));
  LS_TRY(trsv_coop(1, n, k, F, m, Rinv, RinvT, tmpn, n, s, n, gbar, st));
  LS_CU(cudaMemcpyAsync(p, s, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st));
  LS_TRY(colnorm2(n, k, s, n, gamma, st));
  LS_CU(cudaMemcpyAsync(g0d, gamma, sizeof(double) * k, cudaMemcpyDeviceToDevice, st));
  double g0[kLsMaxRhs], gh[kLsMaxRhs];
  LS_CU(cudaMemcpyAsync(g0, gamma, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
  LS_CU(cudaStreamSynchronize(st));
  int it = 0, no_gain = 0;
  double worst = 0.0, best = 1.0;
  const double tol2 = tol * tol;
  for (int c = 0; c < k; ++c) worst = std::max(worst, g0[c] > 0 ? 1.0 : 0.0);
  // Stops when every column is below tol (columns below it are frozen), or
  // when the worst column has not improved for three iterations (the
  // attainable accuracy is reached).
  while (it < maxit && worst > 0.0) {
    // t = R^-1 p ; q = A t ; alpha = gamma / |q|^2
    LS_CU(cudaMemcpyAsync(tmpn, p, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st));
    LS_TRY(trsv_coop(0, n, k, F, m, Rinv, RinvT, tmpn, n, t, n, gbar, st));
    LS_TRY(gemm_sd_n(m, n, k, A, lda, t, n, q, m, 1.0, 0.0, st));
    LS_TRY(colnorm2(m, k, q, m, qq, st));
    k_cgls_alpha<<<1, 32, 0, st>>>(k, gamma, qq, g0d, tol2, alpha);
    count_launch();
    //    X += alpha t ; r -= alpha q
    LS_TRY(axpy_cols(n, k, alpha, 0, t, n, X, ldx, st));
    LS_TRY(axpy_cols(m, k, alpha, 1, q, m, r, m, st));
    //    s = R^-T A^T r ; beta = |s|^2 / gamma ; p = s + beta p
    LS_TRY(gemm_sd_t(m, n, k, A, lda, r, m, tmpn, n, 1.0, 0.0, st));
    LS_TRY(trsv_coop(1, n, k, F, m, Rinv, RinvT, tmpn, n, s, n, gbar, st));
    LS_TRY(colnorm2(n, k, s, n, gnew, st));
    k_cgls_beta<<<1, 32, 0, st>>>(k, gamma, gnew, beta);
    count_launch();
    k_xpby_cols<<<dim3(blocks_for(n), k), TQR_THREADS, 0, st>>>(n, k, s, n, beta, p, n);
    count_launch();
    LS_CU(cudaGetLastError());
    ++it;
    int wait_err = 0;
    LS_CU(cudaMemcpyAsync(gh, gamma, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
    if (g_trsv_pipe) LS_CU(cudaMemcpyAsync(&wait_err, sticky, sizeof(int), cudaMemcpyDeviceToHost, st));
    LS_CU(cudaStreamSynchronize(st));
    if (wait_err) return (int)cudaErrorTimeout;   // a bounded wait of a triangular solve ran out
    worst = 0.0;
    for (int c = 0; c < k; ++c)
      if (g0[c] > 0) worst = std::max(worst, std::sqrt(gh[c] / g0[c]));
    if (worst <= tol) break;
    if (worst < best) {
      best = worst;
      no_gain = 0;
    } else if (++no_gain >= 3) {
      break;
    }
  }
  pt.mark(3);
  pt.finish(it);
  if (iters) *iters = it;
  if (relres) *relres = worst;
  return 0;
}

}  // extern "C"
