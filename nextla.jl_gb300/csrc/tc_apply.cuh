// tc_apply.cuh -- FP32 tsmqr!('L','C') on the 5th-generation tensor cores.
//
// The trailing update of NextLA's tsmqr! (src/tsmqr.jl:47-146 with parfb!/
// pamm!, l = 0) for one 128-column chunk of a tile pair, per ib = 32 block b:
//
//   W^T  = A2^T V_b              GEMM1: M = 128 (chunk columns), N = 32, K = m2
//   W    = T_b^T (A1_b + W)      SIMT on the TMEM read-back (32 x 32 triangle)
//   A1_b = A1_b - W
//   D2   = W^T V_b^T             GEMM2: M = 128, N = m2, K = 32
//   A2^T = A2^T - D2             SIMT, IEEE FP32, on A2^T kept in TMEM
//
// Both GEMMs run as tcgen05.mma kind::tf32 with FP32 accumulators in TMEM,
// issued by one thread and completed through an mbarrier; every operand is
// split x = hi + lo with hi = tf32(x), lo = tf32(x - hi), which keeps
// FP32-level accuracy.  GEMM2 takes hi*hi + hi*lo + lo*hi (three MMAs into
// one accumulator; the dropped lo*lo term is ~2^-22 relative).  GEMM1's N =
// 32 is too narrow to keep the tensor core busy, so its B operand is [V_hi;
// V_lo] (N = 64) and two MMAs per K step, A_hi [V_hi; V_lo] + A_lo [V_hi;
// V_lo], leave W's two halves side by side (the read-back adds them): the
// MMA count of a K step drops from three to two.
//
// Shared-memory operands use the no-swizzle K-major core-matrix layout: 8
// rows x 16 bytes per core matrix, consecutive K groups 128 bytes apart (the
// leading byte offset), consecutive 8-row groups SBO bytes apart.
//
// The same routine serves the other two trailing updates of the tile QR by
// masking V while it is staged (VMode): unmqr! of a geqrt! factor (V unit
// lower triangular in the tile, no A1: W = V_b^T C, C -= V_b W over the whole
// tile, src/unmqr.jl:99-148) and ttmqr! (V upper triangular: reflector p of
// the block at column d0 holds rows [0, d0 + p] only, src/ttmqr.jl:1-95).
//
// The caller owns the TMEM allocation (kTmemCols columns at tmem) and kBars
// mbarriers (initialised with count 1; phase[] tracks their parities).
// Every mbarrier wait is bounded: on expiry the routine returns false and
// issues no further MMA.  Kernels that use TMEM run one CTA per SM, so the
// routine has the SM's TMEM and up to 227 KB of shared memory to itself.
#pragma once
#include <cuda.h>   // CUtensorMap (the tensor maps are encoded on the host)

#include "common.cuh"

namespace tqr {
namespace tc {

constexpr int kChunk = 128;            // chunk columns (GEMM1 M, GEMM2 N)
constexpr int kIb = 32;                // reflectors per block (GEMM1 N, GEMM2 K)
constexpr int kKc = 64;                // GEMM1 K chunk (rows of A2 staged at once)
// TMEM columns: D2 (row r of A2 in column r) in [0, m2), A2^T in [256,
// 256 + m2); D1 (64 columns, W's two halves) in [0, 64), consumed before
// GEMM2 overwrites it
constexpr int kTmemCols = 512;
constexpr uint32_t kA2Col = 256;
// dynamic shared memory: two GEMM1 stage buffers, each A hi/lo (2 x 32 KB) and
// B hi/lo (2 x 8 KB); GEMM2 reuses them (V_b^T hi/lo in stage 0's A, W^T
// hi/lo in stage 1's A), and A2 passes through them on its way into and out
// of TMEM as m2 / 32 boxes of 32 rows x 128 columns; then V_b (m2 / 32 boxes
// of 32 rows x 32 columns) and A1_b (one box of 32 rows x 128 columns) of the
// current block, fetched one block ahead, and the T block.  The raw buffers
// use the 128-byte swizzle of the tensor memory accelerator's tiled loads:
// a box is stored as 128-byte rows (32 consecutive matrix rows of one
// column), and in row y the 16-byte chunk c sits at position c ^ (y % 8).
// The TMA loads write them so, the cp.async fallback writes the same layout,
// and every reader (one 16-byte run per column, 8 columns by 4 runs, or 32
// consecutive rows of a column per warp) spreads over all banks.
constexpr size_t kBufA = 32768, kBufB = 8192;
constexpr size_t kStage = 2 * kBufA + 2 * kBufB;
constexpr uint32_t kA2Box = 32 * kChunk * 4;               // 32 rows x 128 columns
constexpr uint32_t kVBox = 32 * kIb * 4;                   // 32 rows x 32 columns
constexpr int kTLd = 36;
constexpr size_t kVraw = 8 * (size_t)kVBox;                // V_b: up to 256 rows
constexpr size_t kA1s = kA2Box;                            // A1_b: 32 rows x 128 columns
constexpr size_t kTs = sizeof(float) * 32 * kTLd;          // T_b: 32 x 32
constexpr size_t kSmem = 2 * kStage + kVraw + kA1s + kTs + 1024;
static_assert(8 * (size_t)kA2Box <= 2 * kStage, "A2 staging fits the stage buffers");
static_assert((2 * kStage) % 1024 == 0 && kVraw % 1024 == 0, "swizzled boxes start 1024-byte aligned");
constexpr int kBars = 4;               // GEMM1 stage 0, GEMM1 stage 1, GEMM2, operand loads
constexpr long kWaitLimit = 1L << 26;  // mbarrier polls before giving up

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, c) -- matrix row r, column c -- in a stack of
// 128-byte-swizzled boxes of 32 rows each, box_bytes apart (see above).
__device__ __forceinline__ uint32_t swz(int r, int c, uint32_t box_bytes) {
  return (uint32_t)(r >> 5) * box_bytes + (uint32_t)c * 128u +
         ((uint32_t)(((r & 31) >> 2) ^ (c & 7)) << 4) + ((uint32_t)(r & 3) << 2);
}

// Where the operands come from: tensor maps of the FP32 matrices (128-byte
// swizzle; a1 and a2 with 32 x 128 boxes, v with 32 x 32 boxes) and the
// element coordinates (row, column) of A1, A2 and V.  Loads then go through
// the tensor memory accelerator; a null TcMaps uses 16-byte cp.async copies
// into the same layout.
struct TcMaps {
  const CUtensorMap *a1, *a2, *v;
  int a1r, a1c, a2r, a2c, vr, vc;
};

// One tiled TMA load of a 2-D box at element coordinates (x = row, y =
// column), completing on the mbarrier with its byte count.  x is a multiple
// of 32 here (16-byte aligned start for FP32).
__device__ __forceinline__ void tma_load2d(void *sdst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(saddr(sdst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(saddr(bar))
      : "memory");
}

__device__ __forceinline__ void arm_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}

// tcgen05 shared-memory matrix descriptor: no swizzle, version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::tf32: D F32, A and B TF32, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Byte offset of element (row, k) in a K-major core-matrix tile.
__device__ __forceinline__ int kmaj(int row, int k, int sbo) {
  return (row >> 3) * sbo + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
               "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
               ::"r"(d), "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar)));
}

// Waits for the mbarrier phase with parity `parity`; false after kWaitLimit polls.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity) {
  for (long it = 0; it < kWaitLimit; ++it) {
    uint32_t ok;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(saddr(bar)), "r"(parity) : "memory");
    if (ok) return true;
  }
  return false;
}

// 32 TMEM columns of this warp's lane quarter; the load and its wait are one
// asm statement, so no use of the registers can be scheduled before the wait.
__device__ __forceinline__ void ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// Shared memory written by threads -> visible to the tensor core; all threads.
__device__ __forceinline__ void to_async_proxy() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Waits (all threads) for the next phase of barrier `bar`; every thread gets the
// same result.
__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t *phase) {
  const bool ok = __syncthreads_and(bar_wait(bar, *phase)) != 0;
  *phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return ok;
}

__device__ __forceinline__ void put_split4(unsigned char *hi, unsigned char *lo, int off, float4 x) {
  float4 h, l;
  h.x = tf32_round(x.x); l.x = tf32_round(x.x - h.x);
  h.y = tf32_round(x.y); l.y = tf32_round(x.y - h.y);
  h.z = tf32_round(x.z); l.z = tf32_round(x.z - h.z);
  h.w = tf32_round(x.w); l.w = tf32_round(x.w - h.w);
  *reinterpret_cast<float4 *>(hi + off) = h;
  *reinterpret_cast<float4 *>(lo + off) = l;
}

__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// TMEM writes of every thread -> visible to every thread and to the MMAs.
__device__ __forceinline__ void tmem_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void cp16(void *sdst, const void *gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr(sdst)), "l"(gsrc) : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

__device__ __forceinline__ void prefetch_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// How V is read: as stored (tsmqr!), unit lower triangular within the tile
// (the V of geqrt!, for unmqr!: zeros above the diagonal, ones on it, the R
// stored there is not read), or upper triangular (the V of ttqrt!, for
// ttmqr!: zeros below the diagonal, where the tile keeps geqrt!'s V).
enum VMode : int { kVFull = 0, kVUnitLower = 1, kVUpper = 2 };

// Row r of a reflector under the mode; diag is the reflector's diagonal row
// (the row of its implicit or stored leading entry).
__device__ __forceinline__ float vmask(int vmode, int r, int diag, float v) {
  if (vmode == kVUnitLower) return r < diag ? 0.0f : (r == diag ? 1.0f : v);
  if (vmode == kVUpper) return r <= diag ? v : 0.0f;
  return v;
}

// Bytes of block b's operands (V_b, and A1_b when there is one).
__device__ __forceinline__ uint32_t block_bytes(int m2, bool has_a1) {
  return (uint32_t)m2 * kIb * 4 + (has_a1 ? kA2Box : 0u);
}

// The TMA boxes of block b's operands (one thread; the barrier is armed by
// the caller for every byte of the phase before the first load is issued).
__device__ __forceinline__ void tma_block(const TcMaps *mp, int b, int m2, unsigned char *Vraw, bool has_a1,
                                          unsigned char *A1s, uint64_t *bar) {
  for (int q = 0; q < m2 / 32; ++q) tma_load2d(Vraw + q * kVBox, mp->v, mp->vr + 32 * q, mp->vc + b * kIb, bar);
  if (has_a1) tma_load2d(A1s, mp->a1, mp->a1r + b * kIb, mp->a1c, bar);
}

// Block b's raw operands into the swizzled Vraw (V_b, m2 x 32) and A1s
// (A1_b, 32 x 128; skipped when A1b is null).  TMA: thread 0 arms bar with
// the byte count and issues the boxes (the caller has synchronised the CTA
// since the buffers were last read); otherwise every thread issues 16-byte
// cp.async copies, one commit group.  Sources 16-byte aligned, leading
// dimensions multiples of 4.
__device__ __forceinline__ void prefetch_block(const TcMaps *mp, int b, const float *Vb, int ldv, int m2,
                                               unsigned char *Vraw, const float *A1b, int lda1, unsigned char *A1s,
                                               uint64_t *bar) {
  if (mp) {
    if (threadIdx.x == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      arm_tx(bar, block_bytes(m2, A1b != nullptr));
      tma_block(mp, b, m2, Vraw, A1b != nullptr, A1s, bar);
    }
    return;
  }
  const int per_col = m2 / 4;
  for (int idx = threadIdx.x; idx < kIb * per_col; idx += TQR_THREADS) {
    const int p = idx / per_col, r4 = idx % per_col;
    cp16(Vraw + swz(4 * r4, p, kVBox), Vb + (size_t)p * ldv + 4 * r4);
  }
  for (int idx = threadIdx.x; A1b && idx < kChunk * (kIb / 4); idx += TQR_THREADS) {
    const int cc = idx / (kIb / 4), p4 = idx % (kIb / 4);
    cp16(A1s + swz(4 * p4, cc, 0), A1b + (size_t)cc * lda1 + 4 * p4);
  }
  cp_commit();
}

// Waits (all threads) for the loads prefetch_block or the A2 load issued:
// the TMA mbarrier phase (bounded), or every cp.async group and a CTA barrier.
__device__ __forceinline__ bool loads_wait(const TcMaps *mp, uint64_t *bar, uint32_t *phase) {
  if (mp) return wait_phase(bar, phase);
  prefetch_wait();
  __syncthreads();
  return true;
}

// GEMM1's B operand for rows [r0, r0 + kKc) from Vraw: row-of-operand p, K =
// r.  Lanes take 8 p by 4 K runs, so the 16-byte reads (swizzled) and the
// core-matrix stores each spread over all banks.
__device__ __forceinline__ void stage_vb1(const unsigned char *Vraw, int r0, unsigned char *hi, unsigned char *lo,
                                          int vmode, int d0) {
  constexpr uint32_t SB = (kKc / 4) * 128;
#pragma unroll
  for (int u = 0; u < kIb * kKc / 4 / TQR_THREADS; ++u) {
    const int idx = threadIdx.x + u * TQR_THREADS;
    const int rest = idx >> 5;
    const int p = 8 * (rest & 3) + (idx & 7), k4 = 4 * (rest >> 2) + ((idx >> 3) & 3);
    float4 x = *reinterpret_cast<const float4 *>(Vraw + swz(r0 + 4 * k4, p, kVBox));
    if (vmode != kVFull) {
      const int r = r0 + 4 * k4, dg = d0 + p;
      x.x = vmask(vmode, r, dg, x.x); x.y = vmask(vmode, r + 1, dg, x.y);
      x.z = vmask(vmode, r + 2, dg, x.z); x.w = vmask(vmode, r + 3, dg, x.w);
    }
    put_split4(hi, lo, kmaj(p, 4 * k4, SB), x);
  }
}

// Two 32-column TMEM reads of this warp's lane quarter, one wait.
__device__ __forceinline__ void ld32x2(uint32_t ta, uint32_t tb, float (&a)[32], float (&b)[32]) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n"
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,"
      "%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
        "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
        "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(ta), "r"(tb)
      : "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    a[j] = __uint_as_float(r[j]);
    b[j] = __uint_as_float(r[32 + j]);
  }
}

__device__ __forceinline__ void st32(uint32_t taddr, const float (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};"
      ::"r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])),
        "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])), "r"(__float_as_uint(v[20])),
        "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
        "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])),
        "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])),
        "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
}

// [A1; A2] := Q^T [A1; A2] for the 128 columns at A1, A2 (column-major):
// A1 rows [0, k), A2 m2 rows (m2 = 128 or 256), V m2 x k, T 32 x k (blocks of
// 32 columns), k a multiple of 32; A1, A2, V 16-byte aligned with leading
// dimensions multiples of 4.  vmode kVUnitLower: A1 is null and A2 := Q^T A2
// with geqrt!'s V (unmqr!); kVUpper: ttmqr!'s V.  256 threads; all kTmemCols TMEM columns at
// tmem; bars[kBars] mbarriers (count 1) with parities phase[kBars].  Returns
// false if an MMA completion wait timed out (the caller then waits once more
// on every barrier with a pending phase before releasing TMEM).
//
// A2 stays in TMEM for the whole chunk, transposed: TMEM lane c (the chunk
// column) holds A2[0:m2, c] in columns [kA2Col, kA2Col + m2).  So GEMM2 is
// taken transposed, D2 = W^T V_b^T (M = 128 columns, N = m2 rows, K = 32),
// and GEMM1's K-major operand A2^T (row c, K = r) is read back from
// TMEM one lane per thread: 16 consecutive r of one c are four 16-byte K
// runs, stored without any transpose.  The subtraction A2^T -= D2 is fused
// into the next block's staging pass (and into the final write-back) and runs
// on the FP32 pipe: the tensor core's own accumulation is not IEEE
// round-to-nearest, so accumulating A2 through it, block after block and tile
// after tile, lets its rounding drift build up; D2 starts from zero every
// block, as the product alone.  A2 moves through global memory once per chunk
// (in at the start, out at the end) instead of twice per block.
__device__ inline bool tsmqr_chunk(int m2, int k, float *A1, int lda1, float *A2, int lda2, const float *V, int ldv,
                                   const float *T, int ldt, uint32_t tmem, uint64_t *bars, uint32_t *phase,
                                   unsigned char *smem, int vmode = kVFull, const TcMaps *mp = nullptr) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // warps w and w + 4 reach TMEM lanes [32 (w % 4), 32 (w % 4) + 32): this
  // thread's lane is chunk column c; the two warp sets split A2's rows
  const int c = (warp & 3) * 32 + lane, wset = warp >> 2;
  const uint32_t d2t = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  const uint32_t a2t = d2t + kA2Col;
  unsigned char *st_base[2] = {smem, smem + kStage};
  unsigned char *A2raw = smem;                                                     // m2 / 32 boxes
  unsigned char *Vraw = smem + 2 * kStage;                                         // m2 / 32 boxes
  unsigned char *A1s = smem + 2 * kStage + kVraw;                                  // one box
  float *Ts = reinterpret_cast<float *>(smem + 2 * kStage + kVraw + kA1s);         // 32 x kTLd
  // GEMM2 operands in the stage buffers' A regions
  unsigned char *vHi = smem, *vLo = smem + kBufA;                    // V_b^T: m2 x 32, K-major (B)
  unsigned char *wHi = smem + kStage, *wLo = smem + kStage + kBufA;  // W^T: 128 x 32, K-major (A)
  const uint32_t id1 = idesc_tf32(128, 2 * kIb), id2 = idesc_tf32(128, m2);
  const uint32_t d1 = tmem;
  const int nq = m2 / kKc, half = m2 / 2, per_col = m2 / 4, nblk = k / kIb;
  constexpr uint32_t SB = (kKc / 4) * 128;
  bool loads_pending = false;
  auto fail = [&]() {
    // no copy into shared memory outlives the routine
    if (mp) {
      if (loads_pending) bar_wait(&bars[3], phase[3]);
    } else {
      prefetch_wait();
    }
    return false;
  };
  // ---- A2 into TMEM as A2^T: the chunk into the stage buffers (TMA boxes, or
  //      coalesced cp.async), with block 0's operands; then thread c moves its
  //      column (16-byte runs along r) with tcgen05.st ----
  if (mp) {
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      arm_tx(&bars[3], (uint32_t)m2 * kChunk * 4 + (nblk > 0 ? block_bytes(m2, A1 != nullptr) : 0u));
      for (int q = 0; q < m2 / 32; ++q) tma_load2d(A2raw + q * kA2Box, mp->a2, mp->a2r + 32 * q, mp->a2c, &bars[3]);
      if (nblk > 0) tma_block(mp, 0, m2, Vraw, A1 != nullptr, A1s, &bars[3]);
    }
  } else {
    for (int idx = tid; idx < kChunk * per_col; idx += TQR_THREADS) {
      const int cc = idx / per_col, r4 = idx % per_col;
      cp16(A2raw + swz(4 * r4, cc, kA2Box), A2 + (size_t)cc * lda2 + 4 * r4);
    }
    cp_commit();
    if (nblk > 0) prefetch_block(nullptr, 0, V, ldv, m2, Vraw, A1, lda1, A1s, &bars[3]);
  }
  loads_pending = true;
  if (!loads_wait(mp, &bars[3], &phase[3])) return fail();
  loads_pending = false;
#pragma unroll 1
  for (int r0 = wset * half; r0 < (wset + 1) * half; r0 += 32) {
    float v[32];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const float4 x = *reinterpret_cast<const float4 *>(A2raw + swz(r0 + 4 * u, c, kA2Box));
      v[4 * u] = x.x; v[4 * u + 1] = x.y; v[4 * u + 2] = x.z; v[4 * u + 3] = x.w;
    }
    st32(a2t + (uint32_t)r0, v);
  }
  wait_st();
  tmem_sync();
  for (int b = 0; b < nblk; ++b) {
    // this block's T (upper triangle), fetched now and used after GEMM1
    float tv[kIb * kIb / TQR_THREADS];
#pragma unroll
    for (int u = 0; u < kIb * kIb / TQR_THREADS; ++u) {
      const int idx = tid + u * TQR_THREADS, r = idx % kIb, cc = idx / kIb;
      tv[u] = (r <= cc) ? __ldcg(T + (size_t)r + (size_t)(b * kIb + cc) * ldt) : 0.0f;
    }
    if (b > 0) {   // V_b, A1_b in Vraw, A1s
      if (!loads_wait(mp, &bars[3], &phase[3])) return fail();
      loads_pending = false;
    }
    // ---- GEMM1: D1[c][p] = sum_r A2^T[c][r] V_b[r][p], K chunks of 64 rows,
    //      staging of chunk q + 1 overlapping the MMAs of chunk q ----
    for (int q = 0; q < nq; ++q) {
      const int sbuf = q & 1;
      if (q >= 2 && !wait_phase(&bars[sbuf], &phase[sbuf])) return fail();   // chunk q - 2 done with it
      unsigned char *aHi = st_base[sbuf], *aLo = aHi + kBufA, *bHi = aHi + 2 * kBufA, *bLo = bHi + kBufB;
      // A operand from TMEM: warp set s takes rows [32 s, 32 s + 32) of the
      // chunk, first finishing the previous block's A2^T -= D2 on them (chunk
      // 0's D2 columns, [0, 64), are read before this block's GEMM1 writes D1
      // there; chunk 1's, [64, 128), are disjoint from D1)
      {
        const int r = q * kKc + wset * 32;
        float v[32];
        if (b > 0) {
          float d[32];
          ld32x2(a2t + (uint32_t)r, d2t + (uint32_t)r, v, d);
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] -= d[j];
          st32(a2t + (uint32_t)r, v);
        } else {
          ld32(a2t + (uint32_t)r, v);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          put_split4(aHi, aLo, kmaj(c, wset * 32 + 4 * u, SB),
                     make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]));
        if (b > 0) wait_st();
      }
      stage_vb1(Vraw, q * kKc, bHi, bLo, vmode, b * kIb);
      to_async_proxy();
      if (tid == 0) {
        for (int ks = 0; ks < kKc / 8; ++ks) {
          const uint32_t o = ks * 256;
          const uint64_t ah = sdesc(saddr(aHi) + o, 128, SB), al = sdesc(saddr(aLo) + o, 128, SB);
          // rows 32..63 of this N = 64 operand are V_lo: bLo sits 4 row groups after bHi
          const uint64_t bb = sdesc(saddr(bHi) + o, 128, SB);
          mma(d1, ah, bb, id1, (q == 0 && ks == 0) ? 0u : 1u);
          mma(d1, al, bb, id1, 1u);
        }
        commit(&bars[sbuf]);
      }
    }
    // the last two chunks' commits (one per stage buffer) are still pending
    for (int q = (nq >= 2 ? nq - 2 : 0); q < nq; ++q)
      if (!wait_phase(&bars[q & 1], &phase[q & 1])) return fail();
    // T block (upper triangle, zeros below) to shared memory
#pragma unroll
    for (int u = 0; u < kIb * kIb / TQR_THREADS; ++u) {
      const int idx = tid + u * TQR_THREADS, r = idx % kIb, cc = idx / kIb;
      Ts[r + cc * kTLd] = tv[u];
    }
    __syncthreads();
    if (warp < 4) {
      // ---- W = T^T (A1_b + D1^T); A1_b -= W (in A1s); W (split) -> A operand of GEMM2 ----
      float w[32];
      {
        float wl[32];
        ld32x2(d1 + ((uint32_t)(warp * 32) << 16), d1 + ((uint32_t)(warp * 32) << 16) + kIb, w, wl);
#pragma unroll
        for (int p = 0; p < 32; ++p) w[p] += wl[p];   // (A_hi + A_lo) V_hi + (A_hi + A_lo) V_lo
      }
      if (A1) {
#pragma unroll
        for (int p4 = 0; p4 < 8; ++p4) {
          const float4 x = *reinterpret_cast<const float4 *>(A1s + swz(4 * p4, c, 0));
          w[4 * p4] += x.x; w[4 * p4 + 1] += x.y; w[4 * p4 + 2] += x.z; w[4 * p4 + 3] += x.w;
        }
      }
      // W := T^T W in place, last row first (row p reads rows q <= p, not yet
      // overwritten; the zeros of T below its diagonal cover the rest of the
      // 16-byte group)
#pragma unroll
      for (int p = 31; p >= 0; --p) {
        float s = 0.0f;
#pragma unroll
        for (int q4 = 0; q4 <= p / 4; ++q4) {
          const float4 t = *reinterpret_cast<const float4 *>(Ts + p * kTLd + 4 * q4);
          s = fmaf(t.x, w[4 * q4], s);
          s = fmaf(t.y, w[4 * q4 + 1], s);
          s = fmaf(t.z, w[4 * q4 + 2], s);
          s = fmaf(t.w, w[4 * q4 + 3], s);
        }
        w[p] = s;
      }
#pragma unroll
      for (int p4 = 0; p4 < 8; ++p4) {
        if (A1) {
          float4 *xa = reinterpret_cast<float4 *>(A1s + swz(4 * p4, c, 0));
          float4 x = *xa;
          x.x -= w[4 * p4]; x.y -= w[4 * p4 + 1]; x.z -= w[4 * p4 + 2]; x.w -= w[4 * p4 + 3];
          *xa = x;
        }
        put_split4(wHi, wLo, kmaj(c, 4 * p4, (kIb / 4) * 128), make_float4(w[4 * p4], w[4 * p4 + 1],
                                                                          w[4 * p4 + 2], w[4 * p4 + 3]));
      }
    } else {
      // ---- meanwhile V_b^T as the B operand of GEMM2 from Vraw: row r, K = p;
      //      four reads along p (consecutive r across the warp), one 16-byte store ----
      const int t = tid - 128;
#pragma unroll 4
      for (int idx = t; idx < m2 * (kIb / 4); idx += 128) {
        const int r = idx % m2, p4 = idx / m2;
        auto vat = [&](int p) { return *reinterpret_cast<const float *>(Vraw + swz(r, p, kVBox)); };
        float4 x = make_float4(vat(4 * p4), vat(4 * p4 + 1), vat(4 * p4 + 2), vat(4 * p4 + 3));
        if (vmode != kVFull) {
          const int dg = b * kIb + 4 * p4;
          x.x = vmask(vmode, r, dg, x.x); x.y = vmask(vmode, r, dg + 1, x.y);
          x.z = vmask(vmode, r, dg + 2, x.z); x.w = vmask(vmode, r, dg + 3, x.w);
        }
        put_split4(vHi, vLo, kmaj(r, 4 * p4, (kIb / 4) * 128), x);
      }
    }
    to_async_proxy();
    // ---- GEMM2 over all m2 rows at once: D2[c][r] = sum_p W[p][c] V_b[r][p] ----
    if (tid == 0) {
      for (int ks = 0; ks < kIb / 8; ++ks) {
        const uint32_t o = ks * 256;
        const uint64_t ah = sdesc(saddr(wHi) + o, 128, 1024), al = sdesc(saddr(wLo) + o, 128, 1024);
        const uint64_t bh = sdesc(saddr(vHi) + o, 128, 1024), bl = sdesc(saddr(vLo) + o, 128, 1024);
        mma(tmem, ah, bh, id2, ks == 0 ? 0u : 1u);
        mma(tmem, ah, bl, id2, 1u);
        mma(tmem, al, bh, id2, 1u);
      }
      commit(&bars[2]);
    }
    // while the MMAs run: the updated A1_b back to global (coalesced), then
    // the next block's V_b and A1_b into Vraw, A1s
    if (A1) {
      float *A1b = A1 + (size_t)b * kIb;
      for (int idx = tid; idx < kChunk * (kIb / 4); idx += TQR_THREADS) {
        const int cc = idx / (kIb / 4), p4 = idx % (kIb / 4);
        *reinterpret_cast<float4 *>(A1b + (size_t)cc * lda1 + 4 * p4) =
            *reinterpret_cast<const float4 *>(A1s + swz(4 * p4, cc, 0));
      }
    }
    __syncthreads();
    if (b + 1 < nblk) {
      prefetch_block(mp, b + 1, V + (size_t)(b + 1) * kIb * ldv, ldv, m2, Vraw,
                     A1 ? A1 + (size_t)(b + 1) * kIb : nullptr, lda1, A1s, &bars[3]);
      loads_pending = true;
    }
    if (!wait_phase(&bars[2], &phase[2])) return fail();
  }
  // ---- A2 = A2^T - D2 out of TMEM through the stage buffers (coalesced) ----
#pragma unroll 1
  for (int r0 = wset * half; r0 < (wset + 1) * half; r0 += 32) {
    float v[32];
    if (nblk > 0) {   // the last block's D2 is pending
      float d[32];
      ld32x2(a2t + (uint32_t)r0, d2t + (uint32_t)r0, v, d);
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] -= d[j];
    } else {
      ld32(a2t + (uint32_t)r0, v);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
      *reinterpret_cast<float4 *>(A2raw + swz(r0 + 4 * u, c, kA2Box)) =
          make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
  }
  __syncthreads();
  for (int idx = tid; idx < kChunk * per_col; idx += TQR_THREADS) {
    const int cc = idx / per_col, r4 = idx % per_col;
    *reinterpret_cast<float4 *>(A2 + (size_t)cc * lda2 + 4 * r4) =
        *reinterpret_cast<const float4 *>(A2raw + swz(4 * r4, cc, kA2Box));
  }
  tmem_sync();
  return true;
}

}  // namespace tc
}  // namespace tqr
