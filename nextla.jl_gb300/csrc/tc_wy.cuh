// tc_wy.cuh -- the tensor-core FP32 trailing update in compact-WY form.
//
// tsmqr!, unmqr! and ttmqr! apply a tile's k reflectors in ib = 32 blocks, one
// after another (src/tsmqr.jl:47-146 through pamm!/parfb!, src/unmqr.jl:99-148,
// src/ttmqr.jl:1-95), each block Q_b = I - V_b T_b V_b^T.  The product of the
// blocks is one compact-WY transformation Q = Q_0 Q_1 ... = I - V T V^T whose
// k-by-k upper triangular T has the blocks T_b on its diagonal and, above it,
// larft!'s forward recursion (src/larft.jl:53-86) taken over whole blocks:
//
//   T[0:j, J] = -T[0:j, 0:j] (V[:, 0:j]^T V_J) T_J         (J: block j's columns)
//
// (Q_a Q_b = I - [V_a V_b] [[T_a, -T_a V_a^T V_b T_b], [0, T_b]] [V_a V_b]^T).
// The update Q^T [A1; A2] of one 128-column chunk is then three large products
// instead of a chain of eight small ones:
//
//   Y^T = A2^T V                GEMM1  M = 128 (chunk columns), N = k,  K = m2
//   W^T = (A1^T + Y^T) T        GEMM2  M = 128, N = k - 16 s, K = k (T upper:
//                                      K step s only meets columns >= 16 s)
//   D   = W^T V^T               GEMM3  M = 128, N = m2, K = k
//   A1 -= W,  A2 -= D^T         FP32 pipe, IEEE
//
// (For unmqr! there is no A1 and V is geqrt!'s unit lower triangle, whose ones
// stand in for the identity rows of A1.)
//
// wy_build forms, once per tile's V, what every chunk of that tile shares: the
// B operands of the three products -- V (masked by VMode), V^T and T -- each
// split x = hi + lo for TF32x3 and stored as the exact shared-memory image of
// a 16-wide K stage (256 rows of 64 bytes in the tensor cores' 64-byte swizzle,
// hi and lo side by side), 1.5 MB per slot.  Its Gram blocks V_a^T V_b run on
// the tensor cores (TF32x3), the recursion on the FP32 pipe.
//
// wy_chunk streams K through a ring of four 48 KB stage buffers with warp
// roles: lane 0 of warp 0 issues every load (one bulk copy of a stage's B
// image, one tensor-map box of A2 or A1) as soon as the stage's buffer is free
// and every MMA as soon as the stage is ready, testing its mbarriers without
// blocking; warps 1..7 turn each stage's A operand into hi and lo in place
// (A2's raw box; A1^T + Y^T or W^T read back from TMEM) and hand it over
// through an mbarrier.  No CTA-wide barrier separates stages; every wait is
// bounded.
#pragma once
#include "tc_apply.cuh"

namespace tqr {
namespace tc {
namespace wy {

constexpr int kKs = 16;                                  // K per stage: one 64-byte swizzle row of FP32
constexpr int kRing = 4;                                 // stage buffers
constexpr int kDim = 256;                                // rows of a stage image
constexpr int kStagesMax = kDim / kKs;
constexpr uint32_t kABox = 128 * kKs * 4;                // A operand of a stage: 128 rows x 16 K (8 KB)
constexpr uint32_t kImg = kDim * kKs * 4;                // B operand of a stage: 256 rows x 16 K (16 KB)
constexpr uint32_t kStage = 2 * kABox + 2 * kImg;        // A hi, A lo, B hi, B lo
constexpr size_t kSmem = kRing * (size_t)kStage + 1024;
constexpr int kWorkers = 7;                              // warps 1..7 stage the A operands
// mbarriers: loads[kRing], MMAs[kRing], A operands ready[kRing], epilogue loads, teardown
constexpr int kBars = 3 * kRing + 2;
constexpr int kEpiBar = 3 * kRing, kDownBar = 3 * kRing + 1;
constexpr int kPh = 3 * kRing + 1;                       // parities kept by the caller
// slot: stage images of V (GEMM1 and Gram: row p, K = r), V^T (GEMM3: row r,
// K = p) and T (GEMM2, stage s: row p' - 16 s, K = p), hi then lo.  A T
// image keeps only its k - 16 s live rows, hi rows then lo rows back to back,
// so one bulk copy moves just those.
enum : int { kImgV = 0, kImgVT = 1, kImgT = 2 };
constexpr size_t kSlotBytes = (size_t)3 * kStagesMax * 2 * kImg;
__host__ __device__ constexpr size_t img_off(int which, int s) { return ((size_t)which * kStagesMax + s) * 2 * kImg; }
constexpr uint32_t kYCol = 0, kWCol = 256;               // TMEM: Y^T (later D) and W^T
// the recursion's storage, in the ring once the Gram blocks are in TMEM:
// block column q of T (rows [0, 32 (q + 1)), ld 32 (q + 1)) at tf_off(q),
// then X (224 rows of 32, ld kXLd), then T_J row-major (32 x 32)
constexpr int kXLd = 36;
__host__ __device__ constexpr int tf_off(int q) { return 512 * q * (q + 1); }
static_assert(((size_t)tf_off(8) + 224 * kXLd + 1024) * 4 <= kRing * (size_t)kStage, "recursion fits the ring");
static_assert(kStage % 1024 == 0 && kABox % 1024 == 0 && kImg % 1024 == 0, "swizzle atoms stay aligned");
static_assert(kSlotBytes == (size_t)6 * 256 * 256 * 4, "slot size");

// tcgen05 shared-memory descriptor of a K-major operand in the 64-byte
// swizzle: rows of 64 bytes (16 FP32 of K), 8-row atoms 512 bytes apart, the
// leading offset unused (one atom spans the MMA's K), version 1.
__device__ __forceinline__ uint64_t sdesc64(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

// Byte offset of (row, k), k in [0, 16), in a 64-byte-swizzled box: the 16-byte
// chunk k / 4 of row `row` sits at position (k / 4) ^ ((row / 2) % 4), the
// tensor memory accelerator's SWIZZLE_64B placement (box base 512-byte aligned).
__host__ __device__ __forceinline__ uint32_t swz64(int row, int k) {
  return (uint32_t)row * 64u + ((uint32_t)((k >> 2) ^ ((row >> 1) & 3)) << 4) + (uint32_t)(k & 3) * 4u;
}

// A1 and A2 through the tensor memory accelerator (boxes of 16 rows x 128
// columns, 64-byte swizzle) and their element coordinates.
struct WyMaps {
  const CUtensorMap *a1, *a2;
  int a1r, a1c, a2r, a2c;
};

__device__ __forceinline__ unsigned char *ring(unsigned char *smem, int g) { return smem + (size_t)(g % kRing) * kStage; }

// Parity of stage g's phase of a ring barrier (which: 0 loads, 1 MMAs, 2 A
// ready); ph holds each barrier's next phase at the routine's start.
__device__ __forceinline__ uint32_t par(const uint32_t *ph, int which, int g) {
  return ph[which * kRing + g % kRing] ^ (uint32_t)((g / kRing) & 1);
}

// After S stages every buffer's barriers have advanced once per use.
__device__ __forceinline__ void advance(uint32_t *ph, int S, bool a_ready) {
#pragma unroll
  for (int b = 0; b < kRing; ++b) {
    const uint32_t f = (uint32_t)((S > b ? (S - 1 - b) / kRing + 1 : 0) & 1);
    ph[b] ^= f;
    ph[kRing + b] ^= f;
    if (a_ready) ph[2 * kRing + b] ^= f;
  }
}

__device__ __forceinline__ void fence_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

// One bulk copy of contiguous global bytes into shared memory, completing on
// the mbarrier (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void *sdst, const void *gsrc, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(saddr(sdst)), "l"(gsrc), "r"(bytes), "r"(saddr(bar))
               : "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap *m) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}

__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}

// Whether the mbarrier phase with parity `parity` has completed (no waiting).
__device__ __forceinline__ bool bar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(saddr(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// bar_wait that also gives up once another role has flagged a failure.
__device__ __forceinline__ bool bar_wait_f(uint64_t *bar, uint32_t parity, const volatile int *fail) {
  for (long it = 0; it < kWaitLimit; ++it) {
    uint32_t ok;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(saddr(bar)), "r"(parity) : "memory");
    if (ok) return true;
    if ((it & 31) == 31 && *fail) return false;
  }
  return false;
}

// The three split MMAs of one 16-wide K stage (two K = 8 steps) into D, with
// the operands' hi and lo boxes at the given shared-memory addresses.
__device__ __forceinline__ void mma_split(uint32_t d, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t id,
                                          bool acc0) {
#pragma unroll
  for (int ks = 0; ks < 2; ++ks) {
    const uint32_t o = 32u * ks;
    mma(d, sdesc64(ah + o), sdesc64(bh + o), id, (acc0 || ks) ? 1u : 0u);
    mma(d, sdesc64(ah + o), sdesc64(bl + o), id, 1u);
    mma(d, sdesc64(al + o), sdesc64(bh + o), id, 1u);
  }
}

// A stage buffer: A hi, A lo, B hi, B lo.
__device__ __forceinline__ void mma_stage(uint32_t d, const unsigned char *st, uint32_t id, bool acc0) {
  const uint32_t ah = saddr(st);
  mma_split(d, ah, ah + kABox, ah + 2 * kABox, ah + 2 * kABox + kImg, id, acc0);
}

__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// x split into hi and lo at byte offset off of the stage's A hi / A lo boxes.
__device__ __forceinline__ void put_a(unsigned char *st, uint32_t off, float4 x) {
  put_split4(st, st + kABox, (int)off, x);
}

__device__ __forceinline__ float4 split_hi(float4 x, float4 &lo) {
  float4 h;
  h.x = tf32_round(x.x); lo.x = tf32_round(x.x - h.x);
  h.y = tf32_round(x.y); lo.y = tf32_round(x.y - h.y);
  h.z = tf32_round(x.z); lo.z = tf32_round(x.z - h.z);
  h.w = tf32_round(x.w); lo.w = tf32_round(x.w - h.w);
  return h;
}

// Worker share of a GEMM2 stage: NV K values from p0 of row c, W0^T = Y^T
// (TMEM at taddr) + A1^T (the raw box in the A hi slot, when there is one),
// split in place.
template <int NV>
__device__ __forceinline__ void stage_w0(unsigned char *st, int c, int p0, uint32_t taddr, bool has_a1) {
  float y[NV];
  if constexpr (NV == 16) ld16(taddr, y); else ld8(taddr, y);
#pragma unroll
  for (int u = 0; u < NV / 4; ++u) {
    float4 x = make_float4(y[4 * u], y[4 * u + 1], y[4 * u + 2], y[4 * u + 3]);
    const uint32_t off = swz64(c, p0 + 4 * u);
    if (has_a1) {
      const float4 a = *reinterpret_cast<const float4 *>(st + off);
      x.x += a.x; x.y += a.y; x.z += a.z; x.w += a.w;
    }
    put_a(st, off, x);
  }
}

// Worker share of a GEMM3 stage: NV K values from p0 of row c, W^T from TMEM,
// split in place; with A1 (a1p: its values of this row and stage, in global
// memory) A1 -= W from the raw box in the A lo slot, which each thread reads
// before its lo values overwrite it.
template <int NV>
__device__ __forceinline__ void stage_w(unsigned char *st, int c, int p0, uint32_t taddr, float *a1p) {
  float w[NV];
  if constexpr (NV == 16) ld16(taddr, w); else ld8(taddr, w);
#pragma unroll
  for (int u = 0; u < NV / 4; ++u) {
    const float4 x = make_float4(w[4 * u], w[4 * u + 1], w[4 * u + 2], w[4 * u + 3]);
    const uint32_t off = swz64(c, p0 + 4 * u);
    if (a1p) {
      const float4 a = *reinterpret_cast<const float4 *>(st + kABox + off);
      *reinterpret_cast<float4 *>(a1p + 4 * u) = make_float4(a.x - x.x, a.y - x.y, a.z - x.z, a.w - x.w);
    }
    put_a(st, off, x);
  }
}

// [A1; A2] := Q^T [A1; A2] for the 128 columns at A1, A2 (column-major) with
// the slot that wy_build made for Q: A1 rows [0, k) (null: unmqr!, no A1), A2
// m2 rows (128 or 256), k a multiple of 32, A1 and A2 16-byte aligned with
// leading dimensions multiples of 4, the slot 16-byte aligned.  256 threads;
// all 512 TMEM columns at tmem; bars[kBars] mbarriers (loads, MMAs, epilogue
// and teardown with count 1, A-ready with count kWorkers) with their parities
// in ph[kPh].  Returns false if a wait gave up (no load is then in flight;
// MMAs may be, and the caller commits once more on bars[kDownBar] and waits
// before releasing TMEM).
__device__ inline bool wy_chunk(int m2, int k, float *A1, int lda1, float *A2, int lda2, const unsigned char *slot,
                                const WyMaps &mp, uint32_t tmem, uint64_t *bars, uint32_t *ph, unsigned char *smem) {
  __shared__ int s_fail, s_issued, s_consumed, s_eissued;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool has_a1 = A1 != nullptr;
  const int S1 = m2 / kKs, S2 = k / kKs, S = S1 + 2 * S2;
  uint64_t *lb = bars, *mb = bars + kRing, *ab = bars + 2 * kRing, *eb = bars + kEpiBar;
  // shared memory last written by this CTA's threads, and global data written
  // by other tasks, before the tensor memory accelerator touches them
  fence_async_all();
  if (tid == 0) { s_fail = 0; s_issued = 0; s_consumed = 0; s_eissued = 0; }
  __syncthreads();
  auto loads = [&](int g) {   // the loader lane
    unsigned char *st = ring(smem, g);
    uint64_t *bar = &lb[g % kRing];
    if (g < S1) {
      arm_tx(bar, kABox + 2 * kImg);
      tma_load2d(st, mp.a2, mp.a2r + kKs * g, mp.a2c, bar);
      bulk_load(st + 2 * kABox, slot + img_off(kImgV, g), 2 * kImg, bar);
    } else if (g < S1 + S2) {
      const int s = g - S1;
      arm_tx(bar, (has_a1 ? kABox : 0u) + 2 * 64u * (uint32_t)(k - kKs * s));
      if (has_a1) tma_load2d(st, mp.a1, mp.a1r + kKs * s, mp.a1c, bar);
      bulk_load(st + 2 * kABox, slot + img_off(kImgT, s), 2 * 64u * (uint32_t)(k - kKs * s), bar);
    } else {
      const int s = g - S1 - S2;
      arm_tx(bar, (has_a1 ? kABox : 0u) + 2 * kImg);
      if (has_a1) tma_load2d(st + kABox, mp.a1, mp.a1r + kKs * s, mp.a1c, bar);   // A1's raw box: the A lo slot
      bulk_load(st + 2 * kABox, slot + img_off(kImgVT, s), 2 * kImg, bar);
    }
  };
  bool ok = true;
  if (warp == 0) {
    // ---- control, lane 0: never blocks on one condition while another can
    //      proceed -- a stage's loads go out as soon as its buffer's last MMAs
    //      are done, its MMAs as soon as its A operand and loads are in ----
    if (lane == 0) {
      if (has_a1) prefetch_map(mp.a1);
      prefetch_map(mp.a2);
      int issued = min(kRing, S), g = 0;
      for (int x = 0; x < issued; ++x) loads(x);
      const uint32_t idY = idesc_tf32(128, k), idD = idesc_tf32(128, m2);
      long idle = 0;
      while (g < S) {
        bool moved = false;
        if (issued < S && bar_test(&mb[issued % kRing], par(ph, 1, issued - kRing))) {
          loads(issued);
          ++issued;
          moved = true;
        }
        const int b = g % kRing;
        if (bar_test(&ab[b], par(ph, 2, g)) && bar_test(&lb[b], par(ph, 0, g))) {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const unsigned char *st = ring(smem, g);
          if (g < S1) {
            mma_stage(tmem + kYCol, st, idY, g > 0);
          } else if (g < S1 + S2) {
            const int s = g - S1;
            const uint32_t ah = saddr(st), bh = ah + 2 * kABox;   // T's lo rows follow its k - 16 s hi rows
            mma_split(tmem + kWCol + (uint32_t)(kKs * s), ah, ah + kABox, bh, bh + 64u * (uint32_t)(k - kKs * s),
                      idesc_tf32(128, k - kKs * s), s > 0);
          } else {
            mma_stage(tmem + kYCol, st, idD, g > S1 + S2);
          }
          commit(&mb[b]);
          ++g;
          moved = true;
        }
        if (moved) {
          idle = 0;
        } else if (++idle > kWaitLimit || ((idle & 31) == 31 && s_fail)) {
          ok = false;
          break;
        }
      }
      if (!ok) atomicExch(&s_fail, 1);
      s_issued = issued;
      s_consumed = g;
    }
    __syncwarp();
  } else {
    // ---- workers (warps 1..7): each stage's A operand, split in place; warp
    //      4 alone serves TMEM lanes 0..31 and takes all 16 K values there ----
    const int q = warp & 3, c = 32 * q + lane, h = warp >> 2;
    const uint32_t lt = tmem + ((uint32_t)(32 * q) << 16);
    for (int g = 0; g < S; ++g) {
      const int b = g % kRing;
      if (g == S1 || g == S1 + S2) {   // the accumulator read back in this phase is complete
        ok = bar_wait_f(&mb[(g - 1) % kRing], par(ph, 1, g - 1), &s_fail);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      }
      if (ok) ok = bar_wait_f(&lb[b], par(ph, 0, g), &s_fail);
      ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
      if (!ok) break;
      unsigned char *st = ring(smem, g);
      if (g < S1) {
        // GEMM1's A: A2's raw box, hi over the raw values
        for (int i = (warp - 1) * 32 + lane; i < (int)(kABox / 16); i += kWorkers * 32)
          put_a(st, 16u * i, *reinterpret_cast<const float4 *>(st + 16u * i));
      } else if (g < S1 + S2) {
        // GEMM2's A: W0^T = A1^T + Y^T
        const uint32_t col = kYCol + (uint32_t)(kKs * (g - S1));
        if (q == 0) stage_w0<16>(st, c, 0, lt + col, has_a1);
        else stage_w0<8>(st, c, 8 * h, lt + col + 8u * h, has_a1);
      } else {
        // GEMM3's A: W^T; A1 -= W on the way
        const int s = g - S1 - S2;
        const uint32_t col = kWCol + (uint32_t)(kKs * s);
        float *a1p = has_a1 ? A1 + (size_t)c * lda1 + kKs * s : nullptr;
        if (q == 0) stage_w<16>(st, c, 0, lt + col, a1p);
        else stage_w<8>(st, c, 8 * h, lt + col + 8u * h, a1p ? a1p + 8 * h : nullptr);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) arrive(&ab[b]);
    }
    if (!ok && lane == 0) atomicExch(&s_fail, 1);
  }
  // ---- A2 -= D^T once GEMM3 is complete: A2's boxes into the (now idle)
  //      ring through the tensor memory accelerator; thread (c, h) takes rows
  //      [32 q + 16 h, +16) of column c ----
  __syncthreads();
  ok = s_fail == 0;
  if (ok && tid == 0) {
    ok = bar_wait_f(&mb[(S - 1) % kRing], par(ph, 1, S - 1), &s_fail);
    if (ok) {
      arm_tx(eb, (uint32_t)(m2 / kKs) * kABox);
      for (int q = 0; q < m2 / kKs; ++q) tma_load2d(smem + (size_t)q * kABox, mp.a2, mp.a2r + kKs * q, mp.a2c, eb);
      s_eissued = 1;
    } else {
      atomicExch(&s_fail, 1);
    }
  }
  if (ok) {
    ok = bar_wait_f(&mb[(S - 1) % kRing], par(ph, 1, S - 1), &s_fail) && bar_wait_f(eb, ph[kEpiBar], &s_fail);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  ok = __all_sync(0xffffffffu, ok);
  if (ok) {
    const int c = (warp & 3) * 32 + lane, h = warp >> 2;
    const uint32_t lt = tmem + ((uint32_t)((warp & 3) * 32) << 16);
#pragma unroll 1
    for (int q = 0; q < m2 / 32; ++q) {
      float d[16];
      ld16(lt + kYCol + (uint32_t)(32 * q + 16 * h), d);
      const unsigned char *box = smem + (size_t)(2 * q + h) * kABox;
      float *a2p = A2 + (size_t)c * lda2 + 32 * q + 16 * h;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float4 x = *reinterpret_cast<const float4 *>(box + swz64(c, 4 * u));
        x.x -= d[4 * u]; x.y -= d[4 * u + 1]; x.z -= d[4 * u + 2]; x.w -= d[4 * u + 3];
        *reinterpret_cast<float4 *>(a2p + 4 * u) = x;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  ok = __syncthreads_and(ok) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!ok) {
    // every load still in flight lands before the buffers are given up
    if (tid == 0) {
      for (int g = s_consumed; g < s_issued; ++g) bar_wait(&lb[g % kRing], par(ph, 0, g));
      if (s_eissued) bar_wait(eb, ph[kEpiBar]);
    }
    __syncthreads();
    return false;
  }
  advance(ph, S, true);
  ph[kEpiBar] ^= 1u;
  return true;
}

// acc[i][:] += sum over 32 rows qq of T[32 i + lane][32 (NI - 1) + qq] X[qq][:]
// for the NI row blocks a block column of T meets (tq: that block column at
// this lane's row, ld 32 NI; xq: X's rows of the block at this warp's columns).
template <int NI>
__device__ __forceinline__ void trmm_rows(const float *tq, const float *xq, float (&acc)[7][4]) {
#pragma unroll 4
  for (int qq = 0; qq < 32; ++qq) {
    const float4 x = *reinterpret_cast<const float4 *>(xq + qq * kXLd);
    const float *tr = tq + qq * 32 * NI;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      const float t = tr[32 * i];
      acc[i][0] = fmaf(t, x.x, acc[i][0]);
      acc[i][1] = fmaf(t, x.y, acc[i][1]);
      acc[i][2] = fmaf(t, x.z, acc[i][2]);
      acc[i][3] = fmaf(t, x.w, acc[i][3]);
    }
  }
}

// The slot of one tile's reflectors: V (m2 x k, column-major, 16-byte aligned,
// ldv a multiple of 4, masked by vmode with the reflector's diagonal row p)
// and the k x k compact-WY T built from the blocked T (32 x k, blocks of 32
// columns), as the stage images described above, into slot (kSlotBytes,
// 16-byte aligned).  Same resources and failure contract as wy_chunk (the
// A-ready barriers are not used).
__device__ inline bool wy_build(int m2, int k, const float *V, int ldv, const float *T, int ldt, int vmode,
                                unsigned char *slot, uint32_t tmem, uint64_t *bars, uint32_t *ph, unsigned char *smem) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // ---- 1. stage images of V (row p, K = r) and V^T (row r, K = p).  Work
  //      item e is the 16-byte chunk t = e % 1024 of stage e / 1024's image,
  //      so a warp stores 512 contiguous bytes: image row n = t / 4 holds
  //      logical chunk (t % 4) ^ ((n / 2) % 4) there ----
#pragma unroll 4
  for (int e = tid; e < (m2 / kKs) * 1024; e += TQR_THREADS) {
    const int t = e & 1023, s = e >> 10, p = t >> 2, r = kKs * s + 4 * ((t & 3) ^ ((p >> 1) & 3));
    unsigned char *img = slot + img_off(kImgV, s) + 16 * t;
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p < k) {
      x = __ldcg(reinterpret_cast<const float4 *>(V + r + (size_t)p * ldv));
      x.x = vmask(vmode, r, p, x.x); x.y = vmask(vmode, r + 1, p, x.y);
      x.z = vmask(vmode, r + 2, p, x.z); x.w = vmask(vmode, r + 3, p, x.w);
    }
    float4 lo;
    const float4 hi = split_hi(x, lo);
    *reinterpret_cast<float4 *>(img) = hi;
    *reinterpret_cast<float4 *>(img + kImg) = lo;
  }
#pragma unroll 4
  for (int e = tid; e < (k / kKs) * 1024; e += TQR_THREADS) {
    const int t = e & 1023, s = e >> 10, r = t >> 2, p = kKs * s + 4 * ((t & 3) ^ ((r >> 1) & 3));
    unsigned char *img = slot + img_off(kImgVT, s) + 16 * t;
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    if (r < m2) {
      const float *src = V + r + (size_t)p * ldv;
      x.x = vmask(vmode, r, p, __ldcg(src));
      x.y = vmask(vmode, r, p + 1, __ldcg(src + ldv));
      x.z = vmask(vmode, r, p + 2, __ldcg(src + 2 * (size_t)ldv));
      x.w = vmask(vmode, r, p + 3, __ldcg(src + 3 * (size_t)ldv));
    }
    float4 lo;
    const float4 hi = split_hi(x, lo);
    *reinterpret_cast<float4 *>(img) = hi;
    *reinterpret_cast<float4 *>(img + kImg) = lo;
  }
  fence_async_all();
  __syncthreads();
  // ---- 2. Gram blocks on the tensor cores: half hf takes rows p in
  //      [128 hf, +128) against columns q in [128 hf + 32, k), into TMEM
  //      lane p - 128 hf, column 256 hf + q.  A stage is one V image (hi and
  //      lo, one bulk copy); A starts at its row 128 hf, B at row q0 (whole
  //      8-row swizzle atoms) ----
  const int SK = m2 / kKs;
  const int nh = (k > 32 ? 1 : 0) + (k > 160 ? 1 : 0);
  const int S = nh * SK;
  uint64_t *lb = bars, *mb = bars + kRing;
  int issued = 0, consumed = 0;   // thread 0
  auto loads = [&](int g) {       // thread 0
    uint64_t *bar = &lb[g % kRing];
    arm_tx(bar, 2 * kImg);
    bulk_load(ring(smem, g), slot + img_off(kImgV, g % SK), 2 * kImg, bar);
  };
  bool ok = true;
  if (tid == 0 && S > 0) {
    // loads as buffers free up, MMAs as loads land (never blocking on one)
    issued = min(kRing, S);
    for (int x = 0; x < issued; ++x) loads(x);
    int g = 0;
    long idle = 0;
    while (g < S) {
      bool moved = false;
      if (issued < S && bar_test(&mb[issued % kRing], par(ph, 1, issued - kRing))) {
        loads(issued);
        ++issued;
        moved = true;
      }
      if (bar_test(&lb[g % kRing], par(ph, 0, g))) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int hf = g / SK, s = g % SK, q0 = 128 * hf + 32;
        const uint32_t xh = saddr(ring(smem, g)), xl = xh + kImg;
        mma_split(tmem + (uint32_t)(256 * hf + q0), xh + 8192u * hf, xl + 8192u * hf, xh + 64u * q0, xl + 64u * q0,
                  idesc_tf32(128, k - q0), s > 0);
        commit(&mb[g % kRing]);
        ++g;
        moved = true;
      }
      if (moved) {
        idle = 0;
      } else if (++idle > kWaitLimit) {
        ok = false;
        break;
      }
    }
    consumed = g;
  }
  if (S > 0 && ok) ok = bar_wait(&mb[(S - 1) % kRing], par(ph, 1, S - 1));
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  ok = __syncthreads_and(ok) != 0;
  if (!ok) {
    // every load thread 0 issued and did not consume lands first
    if (tid == 0)
      for (int g = consumed; g < issued; ++g) bar_wait(&lb[g % kRing], par(ph, 0, g));
    __syncthreads();
    return false;
  }
  // ---- 3. T by block columns, in the ring (the Gram blocks stay in TMEM) ----
  float *Tf = reinterpret_cast<float *>(smem);
  float *X = Tf + tf_off(8);
  float *TjR = X + 224 * kXLd;   // T_J row-major: TjR[q * 32 + cc]
  const int nbk = k / 32;
  for (int idx = tid; idx < nbk * 1024; idx += TQR_THREADS) {
    const int q = idx >> 10, e = idx & 1023, rr = e & 31, cc = e >> 5;
    Tf[tf_off(q) + cc * 32 * (q + 1) + 32 * q + rr] = rr <= cc ? __ldcg(T + rr + (size_t)(32 * q + cc) * ldt) : 0.0f;
  }
  __syncthreads();
  const uint32_t lt = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  for (int j = 1; j < nbk; ++j) {
    const int ldj = 32 * (j + 1);
    for (int idx = tid; idx < 1024; idx += TQR_THREADS) {
      const int q = idx >> 5, cc = idx & 31;
      TjR[idx] = Tf[tf_off(j) + cc * ldj + 32 * j + q];
    }
    __syncthreads();
    // (a) X[p][:] = G[p][J] T_J for p < 32 j: thread (TMEM lane L, half hh) is row p = L + 128 hh
    {
      const int hh = warp >> 2, p = (warp & 3) * 32 + lane + 128 * hh;
      float gv[32];
      ld32(lt + (uint32_t)(256 * hh + 32 * j), gv);
      if (p < 32 * j) {
#pragma unroll
        for (int c4 = 0; c4 < 8; ++c4) {
          float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
          for (int q = 0; q < 4 * c4 + 4; ++q) {   // T_J[q][cc] = 0 for q > cc
            const float4 t = *reinterpret_cast<const float4 *>(TjR + q * 32 + 4 * c4);
            s0 = fmaf(gv[q], t.x, s0); s1 = fmaf(gv[q], t.y, s1);
            s2 = fmaf(gv[q], t.z, s2); s3 = fmaf(gv[q], t.w, s3);
          }
          *reinterpret_cast<float4 *>(X + p * kXLd + 4 * c4) = make_float4(s0, s1, s2, s3);
        }
      }
    }
    __syncthreads();
    // (b) T[0:32 j, J] = -T[0:32 j, 0:32 j] X: lane -> row 32 i + lane of row block
    //     i < j, warp -> columns [4 warp, +4) of block J
    {
      const int cb = 4 * warp;
      float acc[7][4];
#pragma unroll
      for (int i = 0; i < 7; ++i)
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[i][u] = 0.0f;
      for (int qb = 0; qb < j; ++qb) {
        const float *tq = Tf + tf_off(qb) + lane;
        const float *xq = X + 32 * qb * kXLd + cb;
        switch (qb) {   // block column qb meets row blocks 0..qb
          case 0: trmm_rows<1>(tq, xq, acc); break;
          case 1: trmm_rows<2>(tq, xq, acc); break;
          case 2: trmm_rows<3>(tq, xq, acc); break;
          case 3: trmm_rows<4>(tq, xq, acc); break;
          case 4: trmm_rows<5>(tq, xq, acc); break;
          case 5: trmm_rows<6>(tq, xq, acc); break;
          default: trmm_rows<7>(tq, xq, acc); break;
        }
      }
      float *tJ = Tf + tf_off(j);
#pragma unroll
      for (int i = 0; i < 7; ++i)
        if (i < j)
#pragma unroll
          for (int u = 0; u < 4; ++u) tJ[(cb + u) * ldj + 32 * i + lane] = -acc[i][u];
    }
    __syncthreads();
  }
  // ---- 4. stage images of T (stage s: row n = p' - 16 s, K = p - 16 s; zeros
  //      below the diagonal): the k - 16 s live rows of hi, then of lo,
  //      chunk by chunk as in 1 ----
#pragma unroll 4
  for (int e = tid; e < (k / kKs) * 1024; e += TQR_THREADS) {
    const int t = e & 1023, s = e >> 10, n = t >> 2, pc = kKs * s + n, live = k - kKs * s;
    if (n >= live) continue;
    const int p = kKs * s + 4 * ((t & 3) ^ ((n >> 1) & 3));
    unsigned char *img = slot + img_off(kImgT, s) + 16 * t;
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    {
      const int qb = pc >> 5;
      // rows [p, p + 4) of column pc lie in its stored block column: p + 3 <= 16 s + 15 < 32 (qb + 1)
      x = *reinterpret_cast<const float4 *>(Tf + tf_off(qb) + (pc - 32 * qb) * 32 * (qb + 1) + p);
      if (p > pc) x.x = 0.f;
      if (p + 1 > pc) x.y = 0.f;
      if (p + 2 > pc) x.z = 0.f;
      if (p + 3 > pc) x.w = 0.f;
    }
    float4 lo;
    const float4 hi = split_hi(x, lo);
    *reinterpret_cast<float4 *>(img) = hi;
    *reinterpret_cast<float4 *>(img + 64 * live) = lo;
  }
  // the slot is read next through bulk copies
  fence_async_all();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  advance(ph, S, false);
  return true;
}

}  // namespace wy
}  // namespace tc
}  // namespace tqr
