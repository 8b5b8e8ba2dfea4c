// common.cuh -- shared device helpers of the tile-QR library (sm_103a).
//
// Storage convention everywhere: column-major, element (r, c) of a matrix with
// leading dimension ld at p[r + c * ld], 0-based.  That is the layout NextLA.jl
// works on (Julia arrays and their @views), so a Julia caller passes
// pointer(A) and stride(A, 2) straight through.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

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

// Householder scalars in NextLA's convention (src/geqr2.jl:48-68,
// src/tsqrt.jl:61-70): beta = -copysign(sqrt(alpha^2 + |x|^2), alpha),
// tau = (beta - alpha) / beta, scale = 1 / (alpha - beta).  xnorm_sq == 0
// means "no reflector" (tau = 0).
template <typename R>
__device__ inline void householder(R alpha, R xnorm_sq, R &beta, R &tau, R &scale) {
  beta = -dev_copysign(dev_sqrt(alpha * alpha + xnorm_sq), alpha);
  tau = (beta - alpha) / beta;
  scale = R(1) / (alpha - beta);
}

}  // namespace tqr
