// common.cuh -- shared device helpers of the tile-QR library (sm_103a).
//
// Storage convention everywhere: column-major, element (r, c) of a matrix with
// leading dimension ld at p[r + c * ld], 0-based.  That is the layout NextLA.jl
// works on (Julia arrays and their @views), so a Julia caller passes
// pointer(A) and stride(A, 2) straight through.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>

#define TQR_THREADS 256
#define TQR_WARPS (TQR_THREADS / 32)

// Shared memory a CTA may use (sm_103a allows up to 227 KB per CTA).
#define TQR_SMEM_MAX (227 * 1024)

namespace tqr {

__host__ __device__ inline size_t ix(int r, int c, int ld) {
  return (size_t)c * (size_t)ld + (size_t)r;
}

// Odd leading dimension for shared-memory tiles: 8-byte words at an odd
// stride fall into distinct bank pairs for the 16 lanes of a half-warp.
__host__ __device__ inline int odd_ld(int rows) { return (rows | 1); }

template <typename R>
__device__ inline R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// CTA-wide sum; every thread receives the result.  red must hold TQR_WARPS
// elements.  Contains two __syncthreads().
template <typename R>
__device__ inline R block_sum(R v, R *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) red[w] = v;
  __syncthreads();
  R s = 0;
#pragma unroll
  for (int i = 0; i < TQR_WARPS; ++i) s += red[i];
  __syncthreads();
  return s;
}

template <typename R> __device__ inline R dev_sqrt(R x);
template <> __device__ inline double dev_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ inline float dev_sqrt<float>(float x) { return sqrtf(x); }

template <typename R> __device__ inline R dev_copysign(R a, R b);
template <> __device__ inline double dev_copysign<double>(double a, double b) { return copysign(a, b); }
template <> __device__ inline float dev_copysign<float>(float a, float b) { return copysignf(a, b); }

// ---------------------------------------------------------------------------
// Element types.  The tile kernels are written once over an element type E:
// double, float, cx<double> (Julia's ComplexF64) or cx<float> (ComplexF32).
// cx<R> is two R's, real part first -- the layout of Julia's Complex{R}, of
// C99's R _Complex and of the C-ABI's tqr_zcomplex / tqr_ccomplex -- aligned
// to its size so a load or store is one 16-byte (8-byte) access.
//
// The helpers below make the real instantiations compile to exactly the
// arithmetic the real-only kernels had: conj_ is the identity, mad / madc are
// one fma, abs2_add is fma(v, v, s).
// ---------------------------------------------------------------------------
template <typename R>
struct __align__(2 * sizeof(R)) cx {
  R x, y;   // real, imaginary
  cx() = default;
  __host__ __device__ constexpr cx(R re, R im = R(0)) : x(re), y(im) {}
};

template <typename E> struct elem_traits { using real = E; static constexpr bool complex = false; };
template <typename R> struct elem_traits<cx<R>> { using real = R; static constexpr bool complex = true; };
template <typename E> using real_t = typename elem_traits<E>::real;
template <typename E> constexpr bool is_cx = elem_traits<E>::complex;

template <typename R> __host__ __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return cx<R>(a.x + b.x, a.y + b.y); }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return cx<R>(a.x - b.x, a.y - b.y); }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator-(cx<R> a) { return cx<R>(-a.x, -a.y); }
// The product with its fused multiply-adds spelled out: left as
// a.x * b.x - a.y * b.y the compiler may fuse either product, and may choose
// differently in different kernels, which would make two drivers that run
// the same arithmetic round differently.
template <typename R> __host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
  return cx<R>(fma(a.x, b.x, -(a.y * b.y)), fma(a.x, b.y, a.y * b.x));
}
template <typename R> __host__ __device__ __forceinline__ cx<R> &operator+=(cx<R> &a, cx<R> b) { a = a + b; return a; }
template <typename R> __host__ __device__ __forceinline__ cx<R> &operator-=(cx<R> &a, cx<R> b) { a = a - b; return a; }
template <typename R> __host__ __device__ __forceinline__ cx<R> &operator*=(cx<R> &a, cx<R> b) { a = a * b; return a; }
template <typename R> __host__ __device__ __forceinline__ bool operator==(cx<R> a, cx<R> b) { return a.x == b.x && a.y == b.y; }
template <typename R> __host__ __device__ __forceinline__ bool operator!=(cx<R> a, cx<R> b) { return !(a == b); }

__device__ __forceinline__ double conj_(double a) { return a; }
__device__ __forceinline__ float conj_(float a) { return a; }
template <typename R> __device__ __forceinline__ cx<R> conj_(cx<R> a) { return cx<R>(a.x, -a.y); }

// conj_ only when c holds (complex elements; the identity for real ones)
template <typename E> __device__ __forceinline__ E conj_if(E a, bool c) {
  if constexpr (is_cx<E>) { return c ? conj_(a) : a; } else { (void)c; return a; }
}

// mad(a, b, c) = a b + c
__device__ __forceinline__ double mad(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }
template <typename R> __device__ __forceinline__ cx<R> mad(cx<R> a, cx<R> b, cx<R> c) {
  return cx<R>(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// madc(a, b, c) = conj(a) b + c
__device__ __forceinline__ double madc(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float madc(float a, float b, float c) { return fmaf(a, b, c); }
template <typename R> __device__ __forceinline__ cx<R> madc(cx<R> a, cx<R> b, cx<R> c) {
  return cx<R>(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
// |v|^2 + s
__device__ __forceinline__ double abs2_add(double v, double s) { return fma(v, v, s); }
__device__ __forceinline__ float abs2_add(float v, float s) { return fmaf(v, v, s); }
template <typename R> __device__ __forceinline__ R abs2_add(cx<R> v, R s) { return fma(v.x, v.x, fma(v.y, v.y, s)); }

// a / b: the division itself for real elements; for complex elements Smith's
// algorithm (R. L. Smith, "Algorithm 116: Complex division", CACM 5(8), 1962),
// which scales by the larger part of b so |b|^2 is never formed.
__device__ __forceinline__ double div_(double a, double b) { return a / b; }
__device__ __forceinline__ float div_(float a, float b) { return a / b; }
template <typename R>
__device__ __forceinline__ cx<R> div_(cx<R> a, cx<R> b) {
  if (fabs(b.x) >= fabs(b.y)) {
    const R r = b.y / b.x, d = b.x + b.y * r;
    return cx<R>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const R r = b.x / b.y, d = b.y + b.x * r;
  return cx<R>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}

template <typename R>
__device__ inline cx<R> warp_sum(cx<R> v) {
  return cx<R>(warp_sum(v.x), warp_sum(v.y));
}

// Loads through L2 only (ld.global.cg): in the persistent kernels other SMs
// write the same tiles between tasks and L1 is not coherent with them.
__device__ __forceinline__ double ldg_cg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldg_cg(const float *p) { return __ldcg(p); }
__device__ __forceinline__ cx<double> ldg_cg(const cx<double> *p) {
  const double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
  return cx<double>(v.x, v.y);
}
__device__ __forceinline__ cx<float> ldg_cg(const cx<float> *p) {
  const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
  return cx<float>(v.x, v.y);
}

// ---------------------------------------------------------------------------
// 16-byte staging of column blocks between global and shared memory.
// A strided scalar loop (one load, one store per element) lets a warp wait out
// the L2 latency once per element: the compiler cannot move a global load
// above a shared store it cannot prove disjoint.  These copy an nr-by-ncl
// column-major block with 16-byte global accesses, each thread issuing up to
// kStageVec loads before its first store.  Preconditions (checked by
// cols16_ok): the global block and its column stride are 16-byte aligned and
// nr is a multiple of 16 / sizeof(E).  The shared side keeps any column
// stride (odd strides avoid bank conflicts) and is written element by element.
// ---------------------------------------------------------------------------
constexpr int kStageVec = 4;

// Used for FP32 elements only: an FP32 task is latency-bound on the one CTA a
// TMEM kernel gets per SM, while the FP64 kernels run two CTAs per SM whose
// DFMA work hides the scalar loop's waits (and have no registers to spare).
template <typename E>
__device__ __forceinline__ bool cols16_ok(const E *g, size_t ldg, int nr) {
  constexpr int VE = 16 / sizeof(E);
  return std::is_same<E, float>::value && ((uintptr_t)g & 15) == 0 && ((ldg * sizeof(E)) & 15) == 0 &&
         nr % VE == 0;
}

// dst[r + c * ldd] = conj_if(src[r + c * lds], cj), r < nr, c < ncl
template <typename E>
__device__ __forceinline__ void stage_cols16(const E *src, size_t lds, int nr, int ncl, E *dst, int ldd, bool cj) {
  constexpr int VE = 16 / sizeof(E);
  const int per_col = nr / VE, nvec = per_col * ncl;
  for (int base = threadIdx.x; base < nvec; base += kStageVec * TQR_THREADS) {
    uint4 buf[kStageVec];
#pragma unroll
    for (int u = 0; u < kStageVec; ++u) {
      const int idx = base + u * TQR_THREADS;
      if (idx < nvec) {
        const int c = idx / per_col, q = idx - c * per_col;
        buf[u] = __ldcg(reinterpret_cast<const uint4 *>(src + (size_t)c * lds) + q);
      }
    }
#pragma unroll
    for (int u = 0; u < kStageVec; ++u) {
      const int idx = base + u * TQR_THREADS;
      if (idx < nvec) {
        const int c = idx / per_col, q = idx - c * per_col;
        E e[VE];
        memcpy(e, &buf[u], 16);
        E *d = dst + (size_t)c * ldd + q * VE;
#pragma unroll
        for (int t = 0; t < VE; ++t) d[t] = conj_if(e[t], cj);
      }
    }
  }
}

// dst[r + c * ldd] = conj_if(src[r + c * lds], cj) from shared src to global dst
template <typename E>
__device__ __forceinline__ void unstage_cols16(const E *src, int lds, int nr, int ncl, E *dst, size_t ldd, bool cj) {
  constexpr int VE = 16 / sizeof(E);
  const int per_col = nr / VE, nvec = per_col * ncl;
  for (int idx = threadIdx.x; idx < nvec; idx += TQR_THREADS) {
    const int c = idx / per_col, q = idx - c * per_col;
    const E *s = src + (size_t)c * lds + q * VE;
    E e[VE];
#pragma unroll
    for (int t = 0; t < VE; ++t) e[t] = conj_if(s[t], cj);
    uint4 v;
    memcpy(&v, e, 16);
    reinterpret_cast<uint4 *>(dst + (size_t)c * ldd)[q] = v;
  }
}

// The call sites: the 16-byte copies for FP32 elements (cols16_ok is false
// for every other type, so these are never reached with one).
template <typename E>
__device__ __forceinline__ void stage_cols16_f32(const E *src, size_t lds, int nr, int ncl, E *dst, int ldd, bool cj) {
  if constexpr (std::is_same<E, float>::value) stage_cols16(src, lds, nr, ncl, dst, ldd, cj);
}
template <typename E>
__device__ __forceinline__ void unstage_cols16_f32(const E *src, int lds, int nr, int ncl, E *dst, size_t ldd, bool cj) {
  if constexpr (std::is_same<E, float>::value) unstage_cols16(src, lds, nr, ncl, dst, ldd, cj);
}

// Householder scalars in NextLA's convention (src/geqr2.jl:37-68,
// src/tsqrt.jl:52-73): beta = -copysign(sqrt(|alpha|^2 + |x|^2), re(alpha))
// (real), tau = (beta - alpha) / beta -- for complex elements
// ((beta - re)/beta, -im/beta) -- and scale = 1 / (alpha - beta), formed for
// complex elements as conj(alpha - beta) / |alpha - beta|^2 without a complex
// division.  Returns false for "no reflector" (tau = 0): |x| == 0, and for
// complex elements also im(alpha) == 0.
template <typename R>
__device__ inline bool householder(R alpha, R xnorm_sq, R &beta, R &tau, R &scale) {
  if (xnorm_sq == R(0)) return false;
  beta = -dev_copysign(dev_sqrt(alpha * alpha + xnorm_sq), alpha);
  tau = (beta - alpha) / beta;
  scale = R(1) / (alpha - beta);
  return true;
}

template <typename R>
__device__ inline bool householder(cx<R> alpha, R xnorm_sq, cx<R> &beta, cx<R> &tau, cx<R> &scale) {
  const R ar = alpha.x, ai = alpha.y;
  if (xnorm_sq == R(0) && ai == R(0)) return false;
  const R b = -dev_copysign(dev_sqrt(fma(ar, ar, ai * ai) + xnorm_sq), ar);   // fusions spelled out
  beta = cx<R>(b);
  tau = cx<R>((b - ar) / b, -ai / b);
  const R dr = ar - b, di = ai;
  const R a2 = fma(dr, dr, di * di);
  scale = cx<R>(dr / a2, -di / a2);
  return true;
}

}  // namespace tqr
