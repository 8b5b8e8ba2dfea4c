// tc.cu -- stand-alone launcher of the tensor-core FP32 tsmqr update
// (tc_apply.cuh): one CTA per 128-column chunk of [A1; A2].
#include <cstring>
#include <mutex>

#include "tc_apply.cuh"
#include "tc_wy.cuh"
#include "tileqr.h"
#include "tileqr_internal.h"

namespace tqr {

// ---- tensor maps for the tensor-core chunk routine's TMA loads -------------
// cuTensorMapEncodeTiled is a driver entry point; it is looked up once through
// the runtime (no link against the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn tmap_encoder() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

cudaError_t make_tmap_f32(void *tm, const float *base, long long rows, long long cols, long long ld, int box_rows,
                          int box_cols, int swizzle_bytes) {
  // 16-byte aligned base and column stride; the inner box spans at most the
  // swizzle (64 or 128 bytes); FP32 inner extent a multiple of 16 bytes
  if (swizzle_bytes != 64 && swizzle_bytes != 128) return cudaErrorInvalidValue;
  if (!tm || !base || ((uintptr_t)base & 15) || ((ld * 4) & 15) || rows <= 0 || cols <= 0 || ld < rows ||
      box_rows <= 0 || box_rows * 4 > swizzle_bytes || (box_rows * 4) % 16 || box_cols <= 0 || box_cols > 256)
    return cudaErrorInvalidValue;
  EncodeTiledFn f = tmap_encoder();
  if (!f) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
  const cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = f(static_cast<CUtensorMap *>(tm), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base),
                       dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                       swizzle_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

static int g_tma_enabled = 1;
bool tc_tma_enabled() { return g_tma_enabled != 0; }
static int g_wy_enabled = 0;
bool tc_wy_enabled() { return g_wy_enabled != 0; }

// The stand-alone launch's maps of A1, A2 and V (kernel parameter space).
struct TcLaunchMaps {
  CUtensorMap a1, a2, v;
  int tma;
};

// TMEM allocation / release and the MMA mbarriers for one CTA.
__device__ __forceinline__ void tc_setup(uint64_t *bars, uint32_t *tmem_slot) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < tc::kBars; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::saddr(&bars[i])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::saddr(tmem_slot)),
                 "r"(tc::kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// After a failed wait, one more commit (it arrives once every earlier MMA of
// this thread has completed) and one bounded wait for it; then release TMEM.
__device__ __forceinline__ void tc_teardown(uint64_t *bars, uint32_t *phase, bool failed, uint32_t tmem) {
  if (failed) {
    if (threadIdx.x == 0) tc::commit(&bars[2]);
    tc::bar_wait(&bars[2], phase[2]);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::kTmemCols));
}

__global__ void __launch_bounds__(TQR_THREADS, 1)
k_tsmqr_tc(int m2, int k, float *A1, int lda1, float *A2, int lda2, const float *V, int ldv, const float *T, int ldt,
           int *err, const __grid_constant__ TcLaunchMaps maps) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[tc::kBars];
  __shared__ uint32_t tmem_slot;
  unsigned char *smem = smem_raw + ((1024 - (tc::saddr(smem_raw) & 1023)) & 1023);
  tc_setup(bars, &tmem_slot);
  const uint32_t tmem = tmem_slot;
  uint32_t phase[tc::kBars] = {0u, 0u, 0u, 0u};
  const size_t c0 = (size_t)blockIdx.x * tc::kChunk;
  const tc::TcMaps mp{&maps.a1, &maps.a2, &maps.v, 0, (int)c0, 0, (int)c0, 0, 0};
  const bool ok = tc::tsmqr_chunk(m2, k, A1 + c0 * lda1, lda1, A2 + c0 * lda2, lda2, V, ldv, T, ldt, tmem, bars,
                                  phase, smem, tc::kVFull, maps.tma ? &mp : nullptr);
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);
  tc_teardown(bars, phase, !ok, tmem);
}

// ---- the compact-WY form (tc_wy.cuh) ---------------------------------------
struct WyLaunchMaps {
  CUtensorMap a1, a2;
};

// The WY routines' mbarriers (A-ready ones count the worker warps) and TMEM.
__device__ __forceinline__ void wy_setup(uint64_t *bars, uint32_t *tmem_slot) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < tc::wy::kBars; ++i) {
      const int count = (i >= 2 * tc::wy::kRing && i < 3 * tc::wy::kRing) ? tc::wy::kWorkers : 1;
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc::saddr(&bars[i])), "r"(count));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::saddr(tmem_slot)),
                 "r"(tc::kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// After a failure: a commit on the spare barrier (it arrives once every earlier
// MMA of the issuing thread has completed), one bounded wait, then TMEM goes.
__device__ __forceinline__ void wy_teardown(uint64_t *bars, bool failed, uint32_t tmem) {
  if (failed) {
    if (threadIdx.x == 0) tc::commit(&bars[tc::wy::kDownBar]);
    tc::bar_wait(&bars[tc::wy::kDownBar], 0u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::kTmemCols));
}

__global__ void __launch_bounds__(TQR_THREADS, 1)
k_wy_build(int m2, int k, const float *V, int ldv, const float *T, int ldt, int vmode, unsigned char *slot, int *err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[tc::wy::kBars];
  __shared__ uint32_t tmem_slot;
  unsigned char *smem = smem_raw + ((1024 - (tc::saddr(smem_raw) & 1023)) & 1023);
  wy_setup(bars, &tmem_slot);
  uint32_t ph[tc::wy::kPh] = {};
  const bool ok = tc::wy::wy_build(m2, k, V, ldv, T, ldt, vmode, slot, tmem_slot, bars, ph, smem);
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);
  wy_teardown(bars, !ok, tmem_slot);
}

__global__ void __launch_bounds__(TQR_THREADS, 1)
k_wy_apply(int m2, int k, float *A1, int lda1, float *A2, int lda2, const unsigned char *slot, int *err,
           const __grid_constant__ WyLaunchMaps maps) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[tc::wy::kBars];
  __shared__ uint32_t tmem_slot;
  unsigned char *smem = smem_raw + ((1024 - (tc::saddr(smem_raw) & 1023)) & 1023);
  wy_setup(bars, &tmem_slot);
  uint32_t ph[tc::wy::kPh] = {};
  const int c0 = blockIdx.x * tc::kChunk;
  const tc::wy::WyMaps mp{&maps.a1, &maps.a2, 0, c0, 0, c0};
  const bool ok = tc::wy::wy_chunk(m2, k, A1 ? A1 + (size_t)c0 * lda1 : nullptr, lda1, A2 + (size_t)c0 * lda2, lda2,
                                   slot, mp, tmem_slot, bars, ph, smem);
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);
  wy_teardown(bars, !ok, tmem_slot);
}

}  // namespace tqr

using namespace tqr;

extern "C" {

int tqr_stsmqr_tc(int m1, int n, int m2, int k, float *A1, int lda1, float *A2, int lda2, const float *V, int ldv,
                  const float *T, int ldt, int *err, cudaStream_t stream) {
  if (m1 < 0) return -1;
  if (n < 0 || n % tc::kChunk) return -2;
  if (m2 != 128 && m2 != 256) return -3;
  if (k < 0 || k % tc::kIb || k > m1 || k > m2) return -4;
  if (n == 0 || k == 0) return 0;
  if (!A1 || lda1 < m1) return -6;
  if (!A2 || lda2 < m2) return -8;
  if (!V || ldv < m2) return -10;
  if (!T || ldt < tc::kIb) return -12;
  // 16-byte copies and loads
  if (((uintptr_t)A1 & 15) || (lda1 & 3)) return -6;
  if (((uintptr_t)A2 & 15) || (lda2 & 3) || ((uintptr_t)V & 15) || (ldv & 3)) return -8;
  if (!err) return -13;
  // kernels that use TMEM run one CTA per SM: all of TMEM and shared memory
  const size_t sm = tc::kSmem;
  cudaError_t e = cudaFuncSetAttribute(k_tsmqr_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return (int)e;
  TcLaunchMaps maps;
  maps.tma = tc_tma_enabled() && make_tmap_f32(&maps.a1, A1, m1, n, lda1, 32, tc::kChunk, 128) == cudaSuccess &&
             make_tmap_f32(&maps.a2, A2, m2, n, lda2, 32, tc::kChunk, 128) == cudaSuccess &&
             make_tmap_f32(&maps.v, V, m2, k, ldv, 32, tc::kIb, 128) == cudaSuccess;
  k_tsmqr_tc<<<n / tc::kChunk, TQR_THREADS, sm, stream>>>(m2, k, A1, lda1, A2, lda2, V, ldv, T, ldt, err, maps);
  count_launch();
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

size_t tqr_swy_slot_bytes(void) { return tc::wy::kSlotBytes; }

int tqr_swy_build(int m2, int k, const float *V, int ldv, const float *T, int ldt, int vmode, void *slot,
                  size_t lslot, int *err, cudaStream_t stream) {
  if (m2 != 128 && m2 != 256) return -1;
  if (k < 0 || k % tc::kIb || k > m2) return -2;
  if (k == 0) return 0;
  if (!V || ldv < m2 || ((uintptr_t)V & 15) || (ldv & 3)) return -4;
  if (!T || ldt < tc::kIb) return -6;
  if (vmode < tc::kVFull || vmode > tc::kVUpper) return -7;
  if (!slot || ((uintptr_t)slot & 255)) return -8;
  if (lslot < tc::wy::kSlotBytes) return -9;
  if (!err) return -10;
  cudaError_t e = cudaFuncSetAttribute(k_wy_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::wy::kSmem);
  if (e != cudaSuccess) return (int)e;
  k_wy_build<<<1, TQR_THREADS, tc::wy::kSmem, stream>>>(m2, k, V, ldv, T, ldt, vmode,
                                                         static_cast<unsigned char *>(slot), err);
  count_launch();
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

int tqr_swy_apply(int m1, int n, int m2, int k, float *A1, int lda1, float *A2, int lda2, const void *slot, int *err,
                  cudaStream_t stream) {
  if (m1 < 0) return -1;
  if (n < 0 || n % tc::kChunk) return -2;
  if (m2 != 128 && m2 != 256) return -3;
  if (k < 0 || k % tc::kIb || k > m2 || (A1 && k > m1)) return -4;
  if (n == 0 || k == 0) return 0;
  if (A1 && (lda1 < m1 || ((uintptr_t)A1 & 15) || (lda1 & 3))) return -6;
  if (!A2 || lda2 < m2 || ((uintptr_t)A2 & 15) || (lda2 & 3)) return -8;
  if (!slot || ((uintptr_t)slot & 255)) return -9;
  if (!err) return -10;
  cudaError_t e = cudaFuncSetAttribute(k_wy_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::wy::kSmem);
  if (e != cudaSuccess) return (int)e;
  WyLaunchMaps maps;
  std::memset(&maps, 0, sizeof(maps));
  if (A1 && (e = make_tmap_f32(&maps.a1, A1, m1, n, lda1, tc::wy::kKs, tc::kChunk, 64)) != cudaSuccess) return (int)e;
  if ((e = make_tmap_f32(&maps.a2, A2, m2, n, lda2, tc::wy::kKs, tc::kChunk, 64)) != cudaSuccess) return (int)e;
  k_wy_apply<<<n / tc::kChunk, TQR_THREADS, tc::wy::kSmem, stream>>>(m2, k, A1, lda1, A2, lda2,
                                                                      static_cast<const unsigned char *>(slot), err, maps);
  count_launch();
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

int tqr_stsmqr_wy(int m1, int n, int m2, int k, float *A1, int lda1, float *A2, int lda2, const float *V, int ldv,
                  const float *T, int ldt, void *slot, size_t lslot, int *err, cudaStream_t stream) {
  if (n % tc::kChunk) return -2;
  if (!A1) return -6;
  int r = tqr_swy_build(m2, k, V, ldv, T, ldt, tc::kVFull, slot, lslot, err, stream);
  if (r) return r;
  return tqr_swy_apply(m1, n, m2, k, A1, lda1, A2, lda2, slot, err, stream);
}

int tqr_tile_tc_tma(int on) {
  const int old = tqr::g_tma_enabled;
  tqr::g_tma_enabled = on ? 1 : 0;
  return old;
}

int tqr_tile_tc_wy(int on) {
  const int old = tqr::g_wy_enabled;
  tqr::g_wy_enabled = on ? 1 : 0;
  return old;
}

}  // extern "C"
