/*
 * tileqr.h -- C ABI of libtileqr.so, the GB300 (sm_103a) tile-QR library that
 * stands in for NextLA.jl's in-place tile kernels.
 *
 * Conventions shared by every entry point
 *   - Matrices are column-major with an explicit leading dimension; indices are
 *     0-based.  A Julia caller passes pointer(A) and stride(A, 2) of its (view
 *     of a) CuArray, exactly the storage NextLA's kernels index.
 *   - All pointers are device pointers.  The tile kernels, the stream tile
 *     driver and the solves allocate no device memory per call; scratch is
 *     the caller's `work`.  What the library does allocate:
 *       * the autotuners (tqr_tile_autotune, tqr_batched_autotune) cudaMalloc
 *         their timing matrices and free them before returning;
 *       * tqr_batched_graph creates a stream and instantiates a CUDA graph;
 *       * the persistent drivers (tqr_?tile_geqrf_dag, tqr_?tile_gels_dag,
 *         tqr_?tile_geqrf_{tree,hqr}_dag, tqr_dsgels) keep a pinned host
 *         image of each shape's schedule (cudaMallocHost on the first call
 *         for that shape, cached until exit);
 *       * the stream tile driver creates two streams and four events per
 *         device on its first call (kept until exit); tqr_dsgels creates
 *         four timing events per call.
 *     tqr_dtile_geqrf_noalloc allocates nothing, on the host or the device.
 *   - `work` / `lwork` / `ldwork` arguments exist for signature parity with
 *     NextLA and may be NULL: the W blocks live in on-chip shared memory.
 *   - Return value: 0 on success; -i when argument i (1-based position in the
 *     C signature) is illegal, which is where NextLA throws ArgumentError;
 *     a positive cudaError_t value when a launch failed.
 *   - Calls are asynchronous on `stream`.  NextLA's kernels block until done;
 *     a binding that keeps that behaviour synchronises the stream afterwards.
 *   - Flags are the ASCII characters NextLA uses ('L'/'R', 'N'/'C'/'T',
 *     'F'/'B', 'C'/'R').  'T' means the same as 'C' for real types.
 *   - Each routine exists for double (tqr_d...) and float (tqr_s...); the
 *     tile kernels and the flat tile QR also for ComplexF64 (tqr_z...) and
 *     ComplexF32 (tqr_c...), declared together further down.
 */
#ifndef TILEQR_H
#define TILEQR_H

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Complex elements: real part first, the layout of Julia's ComplexF64 /
 * ComplexF32 and of C99's double _Complex / float _Complex.  Pointers to them
 * must be aligned to the element size (16 / 8 bytes; a CuArray's are). */
typedef struct { double re, im; } tqr_zcomplex;
typedef struct { float re, im; } tqr_ccomplex;

/* geqr2!(m, n, A, tau, work) -- src/geqr2.jl:107-121.
 * Unblocked Householder QR of the m-by-n A; tau has min(m, n) entries. */
int tqr_dgeqr2(int m, int n, double *A, int lda, double *tau, double *work, cudaStream_t stream);
int tqr_sgeqr2(int m, int n, float *A, int lda, float *tau, float *work, cudaStream_t stream);

/* larft!(direct, storev, n, k, V, tau, T) -- src/larft.jl:205-213.
 * k-by-k triangular factor of H = I - V T V^H (all four direct/storev forms). */
int tqr_dlarft(char direct, char storev, int n, int k, const double *V, int ldv, const double *tau,
               double *T, int ldt, cudaStream_t stream);
int tqr_slarft(char direct, char storev, int n, int k, const float *V, int ldv, const float *tau,
               float *T, int ldt, cudaStream_t stream);

/* larfb!(side, trans, direct, storev, m, n, k, V, ldv, T, C, work) -- src/larfb.jl:37-142.
 * C := op(H) C or C op(H); direct 'F' and storev 'C' only, as in the reference. */
int tqr_dlarfb(char side, char trans, char direct, char storev, int m, int n, int k,
               const double *V, int ldv, const double *T, int ldt, double *C, int ldc,
               double *work, int ldwork, cudaStream_t stream);
int tqr_slarfb(char side, char trans, char direct, char storev, int m, int n, int k,
               const float *V, int ldv, const float *T, int ldt, float *C, int ldc,
               float *work, int ldwork, cudaStream_t stream);

/* geqrt!(m, n, ib, A, T, tau, work) -- src/geqrt.jl:22-68.
 * Blocked QR of an m-by-n tile: R above the diagonal, V below, T is ib-by-min(m,n)
 * (block starting at column i in T[0:sb, i:i+sb]), tau has min(m, n) entries. */
int tqr_dgeqrt(int m, int n, int ib, double *A, int lda, double *T, int ldt, double *tau,
               double *work, cudaStream_t stream);
int tqr_sgeqrt(int m, int n, int ib, float *A, int lda, float *T, int ldt, float *tau,
               float *work, cudaStream_t stream);

/* unmqr!(side, trans, m, n, k, ib, A, lda, T, C, work) -- src/unmqr.jl:52-149.
 * C := op(Q) C or C op(Q) with Q from geqrt.  k is clamped to the order of Q;
 * the reference also clamps to size(A, 2), which a binding applies before the call. */
int tqr_dunmqr(char side, char trans, int m, int n, int k, int ib, const double *A, int lda,
               const double *T, int ldt, double *C, int ldc, double *work, int ldwork,
               cudaStream_t stream);
int tqr_sunmqr(char side, char trans, int m, int n, int k, int ib, const float *A, int lda,
               const float *T, int ldt, float *C, int ldc, float *work, int ldwork,
               cudaStream_t stream);

/* tsqrt!(m, n, ib, A1, A2, T, tau, work) -- src/tsqrt.jl:128-156.
 * QR of [A1 (upper triangular); A2 (m-by-n)].  m1 = size(A1, 1), which the
 * reference reads from the array (k = min(m1, n), src/tsqrt.jl:139-140). */
int tqr_dtsqrt(int m, int n, int ib, int m1, double *A1, int lda1, double *A2, int lda2,
               double *T, int ldt, double *tau, double *work, cudaStream_t stream);
int tqr_stsqrt(int m, int n, int ib, int m1, float *A1, int lda1, float *A2, int lda2,
               float *T, int ldt, float *tau, float *work, cudaStream_t stream);

/* tsmqr!(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work) -- src/tsmqr.jl:47-146.
 * [A1; A2] := op(Q) [A1; A2] (side 'L') or [A1 A2] := [A1 A2] op(Q) (side 'R').
 * k is clamped to m1 ('L') or n1 ('R'); the reference's clamp to the stored
 * columns of V and T (src/tsmqr.jl:94-96) is applied by the binding. */
int tqr_dtsmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, double *A1,
               int lda1, double *A2, int lda2, const double *V, int ldv, const double *T, int ldt,
               double *work, int lwork, cudaStream_t stream);
int tqr_stsmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, float *A1,
               int lda1, float *A2, int lda2, const float *V, int ldv, const float *T, int ldt,
               float *work, int lwork, cudaStream_t stream);

/* parfb!(side, trans, direct, storev, m1, n1, m2, n2, k, l, A1, A2, V, T, work)
 * -- src/parfb.jl:44-191 with pamm! (src/pamm.jl:49-473), every side x trans x
 * direct x storev form, triangular order 0 <= l <= k (V's trapezoid as in
 * tqr_?pamm).  The forward columnwise form (the one tsmqr! and ttmqr! use) runs
 * fused and ignores work; the backward and rowwise forms go through pamm! and
 * need work (k x n2 for side 'L', m2 x k for 'R', ldwork; -20 if missing). */
int tqr_dparfb(char side, char trans, char direct, char storev, int m1, int n1, int m2, int n2,
               int k, int l, double *A1, int lda1, double *A2, int lda2, const double *V, int ldv,
               const double *T, int ldt, double *work, int ldwork, cudaStream_t stream);
int tqr_sparfb(char side, char trans, char direct, char storev, int m1, int n1, int m2, int n2,
               int k, int l, float *A1, int lda1, float *A2, int lda2, const float *V, int ldv,
               const float *T, int ldt, float *work, int ldwork, cudaStream_t stream);

/* pamm!(op, side, storev, direct, m, n, k, l, A1, A2, V, W) -- src/pamm.jl:49-473.
 * Every op / side / storev / direct form.  Ve, the reflector block in its
 * canonical orientation (mv x k, mv = m for side 'L', n for 'R'), is V
 * (storev 'C') or V^T ('R'), with a trapezoid of order l: direct 'F' keeps
 * only the upper triangle of the last l rows of the first l columns, 'B' only
 * the lower triangle of the first l rows of the last l columns.
 *   op 'W': W = A1 + f(Ve)^T A2 ('L', W k x n) or A1 + A2 f(Ve) ('R', W m x k),
 *           f = conjugation for (L, C) and (R, R);
 *   op 'A': A2 -= g(Ve) W ('L') or W g(Ve)^T ('R'), g = conjugation for
 *           (L, R) and (R, C); W's first ('F') or last ('B') l rows ('L') /
 *           columns ('R') are left holding the trapezoid's triangle times W,
 *           as the reference's in-place triangular product leaves them.
 *           A1 is not used (may be NULL).
 * Requires 0 <= l <= min(k, mv) (-8 otherwise). */
int tqr_dpamm(char op, char side, char storev, char direct, int m, int n, int k, int l, const double *A1,
              int lda1, double *A2, int lda2, const double *V, int ldv, double *W, int ldw,
              cudaStream_t stream);
int tqr_spamm(char op, char side, char storev, char direct, int m, int n, int k, int l, const float *A1,
              int lda1, float *A2, int lda2, const float *V, int ldv, float *W, int ldw, cudaStream_t stream);

/* ttqrt!(m, n, ib, A1, A2, T, tau, work) -- src/ttqrt.jl:81-119.
 * QR of [A1 (upper triangular); A2 (upper triangular, m-by-n)], k = min(m, n)
 * reflectors; column r's reflector occupies A2 rows [0, min(r + 1, m)).
 * Reads and writes only the upper triangle of A2 (LAPACK dtpqrt with l = n);
 * the reference's T recursion (src/ttqrt.jl:66-71) also sums A2 entries
 * below the diagonal, which are zero on upper-triangular input.  A zero
 * column leaves tau = 0 and its T column untouched, as the reference does. */
int tqr_dttqrt(int m, int n, int ib, double *A1, int lda1, double *A2, int lda2, double *T, int ldt,
               double *tau, double *work, cudaStream_t stream);
int tqr_sttqrt(int m, int n, int ib, float *A1, int lda1, float *A2, int lda2, float *T, int ldt,
               float *tau, float *work, cudaStream_t stream);

/* ttmqr!(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work) -- src/ttmqr.jl:1-95.
 * As tsmqr! with the reflectors of ttqrt!: reflector q of V holds rows
 * (side 'R': columns) [0, q] of A2's space, so block i touches A2 rows
 * [0, min(i + kb, m2)).  k is clamped to m1 ('L') or n1 ('R'). */
int tqr_dttmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, double *A1,
               int lda1, double *A2, int lda2, const double *V, int ldv, const double *T, int ldt,
               double *work, int lwork, cudaStream_t stream);
int tqr_sttmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, float *A1,
               int lda1, float *A2, int lda2, const float *V, int ldv, const float *T, int ldt,
               float *work, int lwork, cudaStream_t stream);

/* ---- Complex elements (every reference kernel test runs ComplexF32 and
 * ComplexF64, test/lapack_helpers.jl:11).  Same arguments and semantics as
 * the real routines above, with the reference's complex conventions:
 * beta = -copysign(|(alpha, x)|, re(alpha)) is real, tau = ((beta - re)/beta,
 * -im/beta), a column gets tau = 0 only when x = 0 and im(alpha) = 0
 * (src/geqr2.jl:37-68), the updates apply H^H = I - conj(tau) v v^H, op(Q)
 * for trans 'C' is Q^H, and 'T' acts as 'C' (src/tsmqr.jl:20).  As in the
 * reference, geqr2 leaves a one-row column (the last of an m <= n panel)
 * with tau = 0, so R's last diagonal entry may stay complex there.  The
 * triangular solve divides in Smith's scaled form.  A pointer not aligned to
 * the element size returns an argument error. ---- */
int tqr_zgeqr2(int m, int n, tqr_zcomplex *A, int lda, tqr_zcomplex *tau, tqr_zcomplex *work,
               cudaStream_t stream);
int tqr_zlarft(char direct, char storev, int n, int k, const tqr_zcomplex *V, int ldv,
               const tqr_zcomplex *tau, tqr_zcomplex *T, int ldt, cudaStream_t stream);
int tqr_zlarfb(char side, char trans, char direct, char storev, int m, int n, int k,
               const tqr_zcomplex *V, int ldv, const tqr_zcomplex *T, int ldt, tqr_zcomplex *C,
               int ldc, tqr_zcomplex *work, int ldwork, cudaStream_t stream);
int tqr_zgeqrt(int m, int n, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T, int ldt,
               tqr_zcomplex *tau, tqr_zcomplex *work, cudaStream_t stream);
int tqr_zunmqr(char side, char trans, int m, int n, int k, int ib, const tqr_zcomplex *A, int lda,
               const tqr_zcomplex *T, int ldt, tqr_zcomplex *C, int ldc, tqr_zcomplex *work,
               int ldwork, cudaStream_t stream);
int tqr_ztsqrt(int m, int n, int ib, int m1, tqr_zcomplex *A1, int lda1, tqr_zcomplex *A2, int lda2,
               tqr_zcomplex *T, int ldt, tqr_zcomplex *tau, tqr_zcomplex *work,
               cudaStream_t stream);
int tqr_ztsmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib,
               tqr_zcomplex *A1, int lda1, tqr_zcomplex *A2, int lda2, const tqr_zcomplex *V,
               int ldv, const tqr_zcomplex *T, int ldt, tqr_zcomplex *work, int lwork,
               cudaStream_t stream);
int tqr_zparfb(char side, char trans, char direct, char storev, int m1, int n1, int m2, int n2,
               int k, int l, tqr_zcomplex *A1, int lda1, tqr_zcomplex *A2, int lda2,
               const tqr_zcomplex *V, int ldv, const tqr_zcomplex *T, int ldt, tqr_zcomplex *work,
               int ldwork, cudaStream_t stream);
int tqr_zttqrt(int m, int n, int ib, tqr_zcomplex *A1, int lda1, tqr_zcomplex *A2, int lda2,
               tqr_zcomplex *T, int ldt, tqr_zcomplex *tau, tqr_zcomplex *work,
               cudaStream_t stream);
int tqr_zttmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib,
               tqr_zcomplex *A1, int lda1, tqr_zcomplex *A2, int lda2, const tqr_zcomplex *V,
               int ldv, const tqr_zcomplex *T, int ldt, tqr_zcomplex *work, int lwork,
               cudaStream_t stream);
int tqr_ztile_geqrf(int m, int n, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T,
                    int ldt, tqr_zcomplex *tau, int ldtau, cudaStream_t stream);
int tqr_ztile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const tqr_zcomplex *A,
                    int lda, const tqr_zcomplex *T, int ldt, tqr_zcomplex *B, int ldb,
                    cudaStream_t stream);
int tqr_zpamm(char op, char side, char storev, char direct, int m, int n, int k, int l,
              const tqr_zcomplex *A1, int lda1, tqr_zcomplex *A2, int lda2, const tqr_zcomplex *V,
              int ldv, tqr_zcomplex *W, int ldw, cudaStream_t stream);
int tqr_ztrsm_lun(int n, int nrhs, const tqr_zcomplex *R, int ldr, tqr_zcomplex *B, int ldb,
                  cudaStream_t stream);
int tqr_ztile_gels(int m, int n, int nrhs, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T,
                   int ldt, tqr_zcomplex *tau, int ldtau, tqr_zcomplex *B, int ldb, cudaStream_t stream);

int tqr_cgeqr2(int m, int n, tqr_ccomplex *A, int lda, tqr_ccomplex *tau, tqr_ccomplex *work,
               cudaStream_t stream);
int tqr_clarft(char direct, char storev, int n, int k, const tqr_ccomplex *V, int ldv,
               const tqr_ccomplex *tau, tqr_ccomplex *T, int ldt, cudaStream_t stream);
int tqr_clarfb(char side, char trans, char direct, char storev, int m, int n, int k,
               const tqr_ccomplex *V, int ldv, const tqr_ccomplex *T, int ldt, tqr_ccomplex *C,
               int ldc, tqr_ccomplex *work, int ldwork, cudaStream_t stream);
int tqr_cgeqrt(int m, int n, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T, int ldt,
               tqr_ccomplex *tau, tqr_ccomplex *work, cudaStream_t stream);
int tqr_cunmqr(char side, char trans, int m, int n, int k, int ib, const tqr_ccomplex *A, int lda,
               const tqr_ccomplex *T, int ldt, tqr_ccomplex *C, int ldc, tqr_ccomplex *work,
               int ldwork, cudaStream_t stream);
int tqr_ctsqrt(int m, int n, int ib, int m1, tqr_ccomplex *A1, int lda1, tqr_ccomplex *A2, int lda2,
               tqr_ccomplex *T, int ldt, tqr_ccomplex *tau, tqr_ccomplex *work,
               cudaStream_t stream);
int tqr_ctsmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib,
               tqr_ccomplex *A1, int lda1, tqr_ccomplex *A2, int lda2, const tqr_ccomplex *V,
               int ldv, const tqr_ccomplex *T, int ldt, tqr_ccomplex *work, int lwork,
               cudaStream_t stream);
int tqr_cparfb(char side, char trans, char direct, char storev, int m1, int n1, int m2, int n2,
               int k, int l, tqr_ccomplex *A1, int lda1, tqr_ccomplex *A2, int lda2,
               const tqr_ccomplex *V, int ldv, const tqr_ccomplex *T, int ldt, tqr_ccomplex *work,
               int ldwork, cudaStream_t stream);
int tqr_cttqrt(int m, int n, int ib, tqr_ccomplex *A1, int lda1, tqr_ccomplex *A2, int lda2,
               tqr_ccomplex *T, int ldt, tqr_ccomplex *tau, tqr_ccomplex *work,
               cudaStream_t stream);
int tqr_cttmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib,
               tqr_ccomplex *A1, int lda1, tqr_ccomplex *A2, int lda2, const tqr_ccomplex *V,
               int ldv, const tqr_ccomplex *T, int ldt, tqr_ccomplex *work, int lwork,
               cudaStream_t stream);
int tqr_ctile_geqrf(int m, int n, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T,
                    int ldt, tqr_ccomplex *tau, int ldtau, cudaStream_t stream);
int tqr_ctile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const tqr_ccomplex *A,
                    int lda, const tqr_ccomplex *T, int ldt, tqr_ccomplex *B, int ldb,
                    cudaStream_t stream);
int tqr_cpamm(char op, char side, char storev, char direct, int m, int n, int k, int l,
              const tqr_ccomplex *A1, int lda1, tqr_ccomplex *A2, int lda2, const tqr_ccomplex *V,
              int ldv, tqr_ccomplex *W, int ldw, cudaStream_t stream);
int tqr_ctrsm_lun(int n, int nrhs, const tqr_ccomplex *R, int ldr, tqr_ccomplex *B, int ldb,
                  cudaStream_t stream);
int tqr_ctile_gels(int m, int n, int nrhs, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T,
                   int ldt, tqr_ccomplex *tau, int ldtau, tqr_ccomplex *B, int ldb, cudaStream_t stream);

/* ---- Tile QR built from the kernels above (no counterpart in NextLA, which
 * ships only the tile kernels; the composition is the flat-tree order its
 * kernels are designed for). ----
 * tile_geqrf: A (m-by-n, nb-by-nb tiles) := tile QR.  T is (MT*ib)-by-n with
 * ldt >= MT*ib, T_ik in rows [i*ib, i*ib+ib), columns [k*nb, k*nb+nb); tau is
 * n-by-MT with ldtau >= n.  MT = ceil(m / nb). */
int tqr_dtile_geqrf(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt,
                    double *tau, int ldtau, cudaStream_t stream);
int tqr_stile_geqrf(int m, int n, int nb, int ib, float *A, int lda, float *T, int ldt,
                    float *tau, int ldtau, cudaStream_t stream);

/* The same factorisation as one persistent kernel over a task DAG (same
 * results, bit for bit, as tqr_?tile_geqrf).  Needs m and n multiples of nb,
 * nb <= 256 a multiple of ib; otherwise returns -3 (use tqr_?tile_geqrf).
 * `work` is caller-owned device scratch of at least the size
 * tqr_tile_dag_worksize reports, 256-byte aligned; it receives the task
 * schedule and the dependency counters on every call.  Calls that overlap on
 * the GPU need separate work buffers.  Every internal wait is bounded (20 s);
 * tqr_tile_dag_status synchronises `stream` and reports 0 (ok) or 1 (a wait
 * timed out: the result is invalid) with the task index. */
int tqr_tile_dag_worksize(int m, int n, int nb, int ib, size_t *bytes);
int tqr_dtile_geqrf_dag(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt,
                        double *tau, int ldtau, void *work, size_t lwork, cudaStream_t stream);
int tqr_stile_geqrf_dag(int m, int n, int nb, int ib, float *A, int lda, float *T, int ldt,
                        float *tau, int ldtau, void *work, size_t lwork, cudaStream_t stream);
/* ComplexF64 / ComplexF32 forms (bit-identical to tqr_ztile_geqrf / tqr_ctile_geqrf).
 * tqr_tile_dag_worksize covers every element type. */
int tqr_ztile_geqrf_dag(int m, int n, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T,
                        int ldt, tqr_zcomplex *tau, int ldtau, void *work, size_t lwork,
                        cudaStream_t stream);
int tqr_ctile_geqrf_dag(int m, int n, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T,
                        int ldt, tqr_ccomplex *tau, int ldtau, void *work, size_t lwork,
                        cudaStream_t stream);
int tqr_tile_dag_status(const void *work, int *status, int *task, cudaStream_t stream);
/* Failure-detection self-test: the FP64 persistent tile QR with task 0 also
 * waiting for a word nothing writes and every wait bounded by wait_ms
 * (1..5000): the launch ends by itself with status 1 (a wait timed out) and
 * task 0 reported, the CUDA context stays usable.  Arguments as
 * tqr_dtile_geqrf_dag; A, T, tau are left partly factored. */
int tqr_tile_dag_wait_selftest(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt,
                               double *tau, int ldtau, void *work, size_t lwork, int wait_ms,
                               cudaStream_t stream);
/* Statistics of the last run in `work` (synchronises `stream`), nanoseconds
 * summed over CTAs: out[0..5] time running each task type (GB, GA, UN, TB,
 * TA, TM), out[6] time waiting for inputs, out[7]/out[8] first and last
 * %globaltimer stamps of the run. */
int tqr_tile_dag_stats(const void *work, unsigned long long *out, cudaStream_t stream);
/* Host-only self check of the schedule for a shape: replays the task list and
 * confirms every closed-form wait target and the topological sort (0 = ok). */
int tqr_tile_dag_check(int m, int n, int nb, int ib, long long *ntasks);
/* (nb, ib) autotuner of the tile QR (no counterpart in NextLA, whose callers
 * pass nb and ib).  Times the tile QR of a seeded m-by-n matrix (uniform
 * [-1, 1) entries) for each candidate (nb, ib): (256, 32), (256, 16),
 * (256, 64); (128, 32), (128, 16) when max(m, n) <= 16384; (64, 16), (64, 32)
 * when max(m, n) <= 2048 -- through the persistent kernel where m and n are
 * multiples of nb, else the stream driver -- and returns the fastest in
 * *nb, *ib.  The result is cached per (dtype_bytes, m, n); force = 1 times
 * again.  dtype_bytes 8 (Float64) or 4 (Float32).  Allocates, synchronises
 * `stream` and frees before it returns: call it outside any stream capture.
 * Returns TQR_ERR_WAIT_TIMEOUT if a persistent-kernel wait ran out.
 * tqr_tile_tuning reads the cache: 0 and the entry, or 1 if not tuned. */
#define TQR_ERR_WAIT_TIMEOUT (-1001)
int tqr_tile_autotune(int dtype_bytes, int m, int n, int force, int *nb, int *ib, cudaStream_t stream);
int tqr_tile_tuning(int dtype_bytes, int m, int n, int *nb, int *ib);
int tqr_tile_dag_check_rhs(int m, int n, int nrhs, int nb, int ib, long long *ntasks);

/* Least squares in one persistent launch plus a triangular solve (m >= n,
 * same shape rules as tqr_?tile_geqrf_dag, 0 < nrhs <= nb): B (m-by-nrhs)
 * rides along as one more tile column of the factorisation, so it leaves as
 * Q^T B, then R X = (Q^T B)[0:n]; X overwrites B[0:n].  A, T, tau as for
 * tile_geqrf; `work` from tqr_tile_gels_worksize. */
int tqr_tile_gels_worksize(int m, int n, int nrhs, int nb, int ib, size_t *bytes);
int tqr_dtile_gels_dag(int m, int n, int nrhs, int nb, int ib, double *A, int lda, double *T, int ldt,
                       double *tau, int ldtau, double *B, int ldb, void *work, size_t lwork,
                       cudaStream_t stream);
int tqr_stile_gels_dag(int m, int n, int nrhs, int nb, int ib, float *A, int lda, float *T, int ldt,
                       float *tau, int ldtau, float *B, int ldb, void *work, size_t lwork,
                       cudaStream_t stream);

/* Allocation-free tile QR (no counterpart in NextLA).  Same factorisation and
 * the same bits as tqr_dtile_geqrf_dag (each tile strip sees the same
 * operations in the same order; only the order in which CTAs pick up tasks
 * differs: here an order written on the device by key 4 min(column, k+1) +
 * row, which follows the critical path without a sort; longest path first
 * there), but it needs no `work` argument: for
 * callers that cannot hand the library device memory -- code running while a
 * framework's caching allocator owns the device, host code that must not
 * take the implicit synchronisation of cudaMalloc/cudaFree mid-pipeline, or
 * bindings with nowhere to keep a scratch buffer between calls.  The
 * schedule and its counters live in a fixed 4 MiB device array inside this
 * library (held by every GPU that loads it until exit), which covers e.g.
 * every square matrix up to 8192 with nb = 256, ib = 32; larger problems get
 * TQR_ERR_SCRATCH_TOO_SMALL and nothing is launched.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress), so make
 * that first call before any stream capture.  Each call clears the counters
 * it needs; all calls share the one array, so calls whose kernels overlap on
 * the GPU (different streams, several host threads) race and must be
 * serialised by the caller.  No cudaMalloc, cudaFree or other allocation.
 * The array's device address is cached per device for the life of its
 * primary context: do not call this entry point (or its status reader) after
 * a cudaDeviceReset in the same process.
 *
 * tqr_tile_noalloc_status reads the error word of the last launch on the
 * current device, as tqr_tile_dag_status does for a caller's `work`: *status
 * 0 = ok, 1 = a dependency wait ran out (20 s), 2 = the schedule in the array
 * did not match the launch (another call overwrote it); *task is the task
 * index that reported it.  A non-zero status means A, T and tau are only
 * partly factorised.  It synchronises `stream`. */
#define TQR_ERR_SCRATCH_TOO_SMALL (-1000)
int tqr_dtile_geqrf_noalloc(int m, int n, int nb, int ib, double *A, int lda, double *T, int ldt,
                            double *tau, int ldtau, cudaStream_t stream);
int tqr_tile_noalloc_status(int *status, int *task, cudaStream_t stream);
/* Host replay of tqr_dtile_geqrf_noalloc's task order for a shape: every
 * dependency is listed before its task and every task appears once.  0 =
 * consistent (*ntasks the count), -1 = shape outside the kernel, 1-5 = which
 * check failed (1 count, 2 a wait target not yet reached, 3 a panel counter's
 * final value, 4 the device generator's count and list disagree, 5 not the
 * loop order's tasks). */
int tqr_tile_noalloc_check(int m, int n, int nb, int ib, long long *ntasks);
/* Host simulation of the persistent kernel (no GPU): `workers` CTAs take tasks
 * strictly in list order, each waits for the task's producers and then runs
 * it for its modelled duration (FP64 FMAs per task, panel tasks weighted for
 * their serial column steps).  Gives the makespan of tqr_dtile_geqrf_noalloc's
 * order, of tqr_dtile_geqrf_dag's longest-path order and the ideal total /
 * workers, in those units.  0 = ok, -1 = shape outside the kernel, -5
 * workers, 2 = a list that is not topological. */
int tqr_tile_dag_simulate(int m, int n, int nb, int ib, int workers, double *noalloc_span, double *sorted_span,
                          double *ideal_span);

/* Tile QR with a binary reduction tree per panel (no counterpart in NextLA;
 * the composition its TT kernels exist for).  Panel k: geqrt! on every tile
 * (i, k), i >= k, and unmqr! on its row's trailing tiles; then ttqrt!/ttmqr!
 * merge tile pairs at distance 1, 2, 4, ... (a last row tile shorter than the
 * panel is wide is first merged whole into the tile above by tsqrt!/tsmqr!).
 * The serial chain per panel is 1 + ceil(log2(MT - k)) tile steps instead of
 * MT - k.  T, T2 are (MT*ib)-by-n, ldt >= MT*ib (T2 is zeroed by the call);
 * tau, tau2 n-by-MT, ldtau >= n: geqrt's factors of tile (i,k) in T/tau at
 * rows i*ib / column i, the merge factors of tile (i,k), i > k, in T2/tau2.
 * nrhs > 0: B (m-by-nrhs) is overwritten by Q^T B.  nb <= 256, ib <= 32. */
int tqr_dtile_geqrf_tree(int m, int n, int nb, int ib, double *A, int lda, double *T, double *T2,
                         int ldt, double *tau, double *tau2, int ldtau, int nrhs, double *B, int ldb,
                         cudaStream_t stream);
int tqr_stile_geqrf_tree(int m, int n, int nb, int ib, float *A, int lda, float *T, float *T2,
                         int ldt, float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb,
                         cudaStream_t stream);
/* The same tree factorisation (same arithmetic, same results) as one
 * persistent launch over a task graph: tasks per tile / pair and 16-column
 * strip, dependencies from the regions each task reads and writes, taken in
 * longest-path order with bounded waits.  Needs nb and ib multiples of 16,
 * nb <= 256, ib <= 32, nrhs <= 256.  work: 256-byte aligned,
 * tqr_tile_tree_dag_worksize bytes (the task list, built once per shape on the
 * host, and per-task flags); -16/-17 for an unaligned / too small work.
 * tqr_tile_tree_dag_status: error word (0 ok, 1 a wait timed out, 2 schedule
 * mismatch) and the task it stopped at; tqr_tile_tree_dag_check: host check
 * that every dependency precedes its task, and the task count. */
int tqr_tile_tree_dag_worksize(int m, int n, int nb, int ib, int nrhs, size_t *bytes);
int tqr_tile_tree_dag_check(int m, int n, int nb, int ib, int nrhs, long long *ntasks);
int tqr_tile_tree_dag_status(const void *work, int *error, int *item, cudaStream_t stream);
int tqr_dtile_geqrf_tree_dag(int m, int n, int nb, int ib, double *A, int lda, double *T, double *T2,
                             int ldt, double *tau, double *tau2, int ldtau, int nrhs, double *B, int ldb,
                             void *work, size_t lwork, cudaStream_t stream);
int tqr_stile_geqrf_tree_dag(int m, int n, int nb, int ib, float *A, int lda, float *T, float *T2,
                             int ldt, float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb,
                             void *work, size_t lwork, cudaStream_t stream);
/* Hierarchical form (PLASMA's HQR): the tiles of each panel form groups of
 * grp consecutive tiles, each reduced flat into its first tile (geqrt! on the
 * leader, tsqrt!/tsmqr! of the others into it -- their reflectors in the whole
 * tile, with T2 / tau2), then the leaders by the binary ttqrt!/ttmqr! tree at
 * distances grp, 2 grp, ...; a ragged last tile joins the last group.
 * grp = 1 is tqr_?tile_geqrf_tree; a panel's serial chain is grp + log2 of its
 * leader count tile steps.  Same layouts as the tree form; the Q application
 * takes the same grp. */
int tqr_dtile_geqrf_hqr(int m, int n, int nb, int ib, int grp, double *A, int lda, double *T, double *T2,
                        int ldt, double *tau, double *tau2, int ldtau, int nrhs, double *B, int ldb,
                        cudaStream_t stream);
int tqr_stile_geqrf_hqr(int m, int n, int nb, int ib, int grp, float *A, int lda, float *T, float *T2,
                        int ldt, float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb,
                        cudaStream_t stream);
int tqr_tile_hqr_dag_worksize(int m, int n, int nb, int ib, int grp, int nrhs, size_t *bytes);
/* The FP32 hierarchical tree of the mixed solve (no counterpart in NextLA):
 * as tqr_stile_geqrf_hqr_dag, with the panel steps -- geqrt! blocks, the
 * tsqrt! merges into a group leader and the ttqrt! merges of leaders -- in
 * FP64 on widened copies (the leaders' diagonal R triangles kept in FP64 in
 * `work`, reflectors and tau rounded to FP32 as formed).  For 256 x 256 tiles
 * with ib = 32 every trailing update of A (the leaders' unmqr!, the merges'
 * tsmqr! and ttmqr!) runs on the tensor cores (TF32x3, 128-column chunks), as
 * it does in the plain FP32 task graph unless tqr_tile_dag_tensor_cores(0).
 * m and n multiples of nb, ib <= 32.  `work` from tqr_tile_hqr_dag_worksize
 * (it covers this form).  tqr_tile_hqr_dag_check_tc verifies the
 * tensor-core task graph's order on the host and returns its number of
 * tensor-core tasks in *ntasks. */
int tqr_stile_geqrf_hqr_dag_f64p(int m, int n, int nb, int ib, int grp, float *A, int lda, float *T, float *T2,
                                 int ldt, float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb, void *work,
                                 size_t lwork, cudaStream_t stream);
int tqr_tile_hqr_dag_check_tc(int m, int n, int nb, int ib, int grp, int nrhs, long long *ntasks);
int tqr_tile_hqr_dag_check(int m, int n, int nb, int ib, int grp, int nrhs, long long *ntasks);
int tqr_dtile_geqrf_hqr_dag(int m, int n, int nb, int ib, int grp, double *A, int lda, double *T,
                            double *T2, int ldt, double *tau, double *tau2, int ldtau, int nrhs, double *B,
                            int ldb, void *work, size_t lwork, cudaStream_t stream);
int tqr_stile_geqrf_hqr_dag(int m, int n, int nb, int ib, int grp, float *A, int lda, float *T, float *T2,
                            int ldt, float *tau, float *tau2, int ldtau, int nrhs, float *B, int ldb,
                            void *work, size_t lwork, cudaStream_t stream);
int tqr_dtile_unmqr_hqr(char trans, int m, int n, int nrhs, int nb, int ib, int grp, const double *A,
                        int lda, const double *T, const double *T2, int ldt, double *B, int ldb,
                        cudaStream_t stream);
int tqr_stile_unmqr_hqr(char trans, int m, int n, int nrhs, int nb, int ib, int grp, const float *A,
                        int lda, const float *T, const float *T2, int ldt, float *B, int ldb,
                        cudaStream_t stream);

/* B := Q^T B (trans 'C'/'T') or Q B ('N') with Q from tqr_?tile_geqrf_tree. */
int tqr_dtile_unmqr_tree(char trans, int m, int n, int nrhs, int nb, int ib, const double *A, int lda,
                         const double *T, const double *T2, int ldt, double *B, int ldb,
                         cudaStream_t stream);
int tqr_stile_unmqr_tree(char trans, int m, int n, int nrhs, int nb, int ib, const float *A, int lda,
                         const float *T, const float *T2, int ldt, float *B, int ldb, cudaStream_t stream);

/* The tree and hierarchical drivers for ComplexF64 (z) and ComplexF32 (c)
 * elements (no counterpart driver in NextLA; the reference runs its TT
 * kernels on ComplexF64, test/ttqrt.jl:28-66): the same reductions with the
 * complex geqrt!/unmqr!/tsqrt!/tsmqr!/ttqrt!/ttmqr! arithmetic, Q^H where the
 * real forms apply Q^T ('T' acts as 'C').  Same arguments, layouts and
 * errors as the real forms; element pointers aligned to the element size
 * (the position of A otherwise).  ComplexF64 runs 8-column strips (one CTA
 * per SM), ComplexF32 the real geometry; the task-graph forms
 * (..._dag) take `work` from tqr_tile_hqr_dag_worksize /
 * tqr_tile_tree_dag_worksize, which cover every element type.
 * tqr_tile_hqr_dag_check_strips: the host order check of a task graph with
 * strips of nw columns (16, or 8 for ComplexF64). */
int tqr_ztile_geqrf_tree(int m, int n, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T,
                         tqr_zcomplex *T2, int ldt, tqr_zcomplex *tau, tqr_zcomplex *tau2, int ldtau, int nrhs,
                         tqr_zcomplex *B, int ldb, cudaStream_t stream);
int tqr_ctile_geqrf_tree(int m, int n, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T,
                         tqr_ccomplex *T2, int ldt, tqr_ccomplex *tau, tqr_ccomplex *tau2, int ldtau, int nrhs,
                         tqr_ccomplex *B, int ldb, cudaStream_t stream);
int tqr_ztile_unmqr_tree(char trans, int m, int n, int nrhs, int nb, int ib, const tqr_zcomplex *A, int lda,
                         const tqr_zcomplex *T, const tqr_zcomplex *T2, int ldt, tqr_zcomplex *B, int ldb,
                         cudaStream_t stream);
int tqr_ctile_unmqr_tree(char trans, int m, int n, int nrhs, int nb, int ib, const tqr_ccomplex *A, int lda,
                         const tqr_ccomplex *T, const tqr_ccomplex *T2, int ldt, tqr_ccomplex *B, int ldb,
                         cudaStream_t stream);
int tqr_ztile_geqrf_hqr(int m, int n, int nb, int ib, int grp, tqr_zcomplex *A, int lda, tqr_zcomplex *T,
                        tqr_zcomplex *T2, int ldt, tqr_zcomplex *tau, tqr_zcomplex *tau2, int ldtau, int nrhs,
                        tqr_zcomplex *B, int ldb, cudaStream_t stream);
int tqr_ctile_geqrf_hqr(int m, int n, int nb, int ib, int grp, tqr_ccomplex *A, int lda, tqr_ccomplex *T,
                        tqr_ccomplex *T2, int ldt, tqr_ccomplex *tau, tqr_ccomplex *tau2, int ldtau, int nrhs,
                        tqr_ccomplex *B, int ldb, cudaStream_t stream);
int tqr_ztile_unmqr_hqr(char trans, int m, int n, int nrhs, int nb, int ib, int grp, const tqr_zcomplex *A,
                        int lda, const tqr_zcomplex *T, const tqr_zcomplex *T2, int ldt, tqr_zcomplex *B, int ldb,
                        cudaStream_t stream);
int tqr_ctile_unmqr_hqr(char trans, int m, int n, int nrhs, int nb, int ib, int grp, const tqr_ccomplex *A,
                        int lda, const tqr_ccomplex *T, const tqr_ccomplex *T2, int ldt, tqr_ccomplex *B, int ldb,
                        cudaStream_t stream);
int tqr_ztile_geqrf_hqr_dag(int m, int n, int nb, int ib, int grp, tqr_zcomplex *A, int lda, tqr_zcomplex *T,
                            tqr_zcomplex *T2, int ldt, tqr_zcomplex *tau, tqr_zcomplex *tau2, int ldtau,
                            int nrhs, tqr_zcomplex *B, int ldb, void *work, size_t lwork, cudaStream_t stream);
int tqr_ctile_geqrf_hqr_dag(int m, int n, int nb, int ib, int grp, tqr_ccomplex *A, int lda, tqr_ccomplex *T,
                            tqr_ccomplex *T2, int ldt, tqr_ccomplex *tau, tqr_ccomplex *tau2, int ldtau,
                            int nrhs, tqr_ccomplex *B, int ldb, void *work, size_t lwork, cudaStream_t stream);
int tqr_ztile_geqrf_tree_dag(int m, int n, int nb, int ib, tqr_zcomplex *A, int lda, tqr_zcomplex *T,
                             tqr_zcomplex *T2, int ldt, tqr_zcomplex *tau, tqr_zcomplex *tau2, int ldtau,
                             int nrhs, tqr_zcomplex *B, int ldb, void *work, size_t lwork, cudaStream_t stream);
int tqr_ctile_geqrf_tree_dag(int m, int n, int nb, int ib, tqr_ccomplex *A, int lda, tqr_ccomplex *T,
                             tqr_ccomplex *T2, int ldt, tqr_ccomplex *tau, tqr_ccomplex *tau2, int ldtau,
                             int nrhs, tqr_ccomplex *B, int ldb, void *work, size_t lwork, cudaStream_t stream);
int tqr_tile_hqr_dag_check_strips(int m, int n, int nb, int ib, int grp, int nrhs, int nw, long long *ntasks);

/* B (m-by-nrhs) := Q^T B (trans 'C'/'T') or Q B (trans 'N'), Q from tile_geqrf. */
int tqr_dtile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const double *A, int lda,
                    const double *T, int ldt, double *B, int ldb, cudaStream_t stream);
int tqr_stile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const float *A, int lda,
                    const float *T, int ldt, float *B, int ldb, cudaStream_t stream);

/* R X = B for the upper triangle of the n-by-n R; B (n-by-nrhs) is overwritten
 * by X.  Arithmetic of NextLA's LeftUpperTRSM! (src/trsm.jl:38-63, 134-138),
 * blocked so that n is not limited to 1024. */
int tqr_dtrsm_lun(int n, int nrhs, const double *R, int ldr, double *B, int ldb,
                  cudaStream_t stream);
int tqr_strsm_lun(int n, int nrhs, const float *R, int ldr, float *B, int ldb,
                  cudaStream_t stream);

/* Least squares min ||A X - B||, m >= n: tile_geqrf, Q^T B, then R X = B[0:n].
 * A, T, tau as for tile_geqrf; X overwrites B[0:n, 0:nrhs]. */
int tqr_dtile_gels(int m, int n, int nrhs, int nb, int ib, double *A, int lda, double *T, int ldt,
                   double *tau, int ldtau, double *B, int ldb, cudaStream_t stream);
int tqr_stile_gels(int m, int n, int nrhs, int nb, int ib, float *A, int lda, float *T, int ldt,
                   float *tau, int ldtau, float *B, int ldb, cudaStream_t stream);

/* ---- Mixed-precision least squares (no counterpart in NextLA; its poster lists
 * mixed precision as future work) ----
 * min ||A X - B|| for a Float32 A (m-by-n, m >= n, lda) and Float64 B
 * (m-by-nrhs, nrhs <= 16): tile QR of a copy of A (persistent kernel when m,
 * n are multiples of nb) with the trailing tsmqr/unmqr updates in FP32 (TF32x3
 * on the tensor cores) and the panel tasks in FP64 -- the larfg norm and
 * reflector scaling, the larft T build, the tsqrt blocks and the diagonal R
 * triangles they update, on a widened copy of each panel block, V / T / tau
 * rounded to FP32 once for the updates; X0 = R^-1 (Q^T B)[0:n] in FP32, then CGLS
 * with FP64 iterates on the right-preconditioned problem min ||A R^-1 Y - B||
 * (X = R^-1 Y): every product with A uses A's FP32 entries exactly and sums in
 * double-float on the FP32 pipe (~2^-48 relative per 32 terms, flushed to
 * FP64), every solve with R runs in FP64.  Stops when the
 * preconditioned normal-equation residual of every column has dropped by
 * `tol` or after `maxit` iterations; `iters` and `relres` (that ratio) report
 * where it stopped.  A and B are not modified.  `work` (256-byte aligned) holds
 * the FP32 factor and the iteration vectors; its size comes from
 * tqr_dsgels_worksize.  Synchronises `stream` once per iteration.  Returns
 * cudaErrorTimeout (a positive status) if a bounded device wait of the
 * refinement's triangular solves ran out (2 s); X is then not the solution. */
int tqr_dsgels_worksize(int m, int n, int nrhs, int nb, int ib, size_t *bytes);
int tqr_dsgels(int m, int n, int nrhs, int nb, int ib, const float *A, int lda, const double *B,
               int ldb, double *X, int ldx, int maxit, double tol, void *work, size_t lwork,
               int *iters, double *relres, cudaStream_t stream);
/* Device time (ms) of the last tqr_dsgels call's phases: ms[0] FP32 tile QR,
 * ms[1] X0 = R^-1 Q^T B, ms[2] FP64 CGLS refinement; iters its iterations. */
int tqr_dsgels_phases(double *ms, int *iters);
/* tqr_dsgels_fp64_panels(0) makes later tqr_dsgels calls factor with FP32
 * panels instead (for comparison); 1 restores the default.  Returns the
 * previous setting.  Process-wide. */
int tqr_dsgels_fp64_panels(int on);
/* tqr_dsgels_hqr_group(grp): grp > 0 (default 16) makes tqr_dsgels factor
 * with the hierarchical tree (groups of grp tiles reduced flat, leaders by
 * the binary tree; tqr_stile_geqrf_hqr_dag_f64p) when m and n are multiples
 * of nb and A has at least 2 grp tile rows; 0 selects the flat tree always.
 * Returns the previous setting.  Process-wide; tqr_dsgels_worksize depends
 * on it. */
int tqr_dsgels_hqr_group(int grp);
/* The CGLS refinement of tqr_dsgels applies R^-1 and R^-T (R's 256 x 256
 * diagonal blocks inverted once) as a pipelined task list: 8-row tasks, the
 * update of a row block by one solved block (B_t -= op(R)_{t,s} X_s) and the
 * product with an inverted diagonal block (X_t = op(R_tt^-1) B_t), ordered
 * by per-block counters instead of grid-wide barriers; every sum runs in a
 * fixed order.  tqr_dsgels_trsv_pipelined(0) selects the previous form, one
 * cooperative launch with two grid barriers per block (for comparison); 1
 * restores the default.  Returns the previous setting.  Process-wide.
 * tqr_dsgels_trsv_pipe_check: host replay of the task list for order n
 * (every wait on earlier work, each row block's updates in source order,
 * every task once); 0 = consistent, *ntasks the task count. */
int tqr_dsgels_trsv_pipelined(int on);
int tqr_dsgels_trsv_pipe_check(int n, long long *ntasks);
/* The FP32 tile QR with FP64 panels on its own (the factorisation of
 * tqr_dsgels, without B): as tqr_stile_geqrf_dag, same T/tau layouts; `work`
 * from tqr_tile_dag_worksize (which covers this form). */
int tqr_stile_geqrf_dag_f64p(int m, int n, int nb, int ib, float *A, int lda, float *T, int ldt, float *tau,
                             int ldtau, void *work, size_t lwork, cudaStream_t stream);

/* ---- Batched uneven QR + least squares (no counterpart in NextLA, which
 * factors one matrix at a time) ----
 * nprob independent problems min ||A_q X_q - B_q||, A_q m_q-by-n_q with
 * 1 <= n_q <= m_q <= TQR_BATCH_MAX_M and 0 <= k_q <= TQR_BATCH_MAX_K right-hand
 * sides (k_q = 0: QR only).  Each problem is geqrt! on its A_q (the
 * arithmetic of src/geqrt.jl:22-68 with inner block ib_q), the same
 * reflectors applied to B_q (unmqr!, src/unmqr.jl:52-149, 'L','T'), then
 * LeftUpperTRSM! (src/trsm.jl:36-63) on the first n_q rows.  On return A_q
 * holds geqrt!'s R and V, and B_q's rows 0:n_q hold X_q.
 *
 * tqr_batched_plan (host only): from the sizes, fills nprob descriptors of
 * tqr_batched_problem_bytes() bytes each -- int m, n, k, ib, nw, pad;
 * int64 a_off, b_off -- with A_q packed column-major at A + a_off (lda = m_q)
 * and B_q at B + b_off (ldb = m_q), every problem 32-element aligned, ib and
 * the strip width nw taken from the tuning table, and `order`, the problems by
 * decreasing flops; a_elems, b_elems are the packed lengths.  Returns
 * -(1000 + q) if problem q is out of range.
 * tqr_?batched_gels: one persistent launch (plus a counter reset) over the
 * device copies of the descriptors and order; work (256-byte aligned,
 * tqr_batched_worksize bytes) holds the counter and per-CTA scratch.
 * Descriptors the kernel finds out of range are skipped and counted:
 * tqr_batched_status reads that count and the first bad index (synchronises
 * stream).  No allocation, no host synchronisation.
 * tqr_batched_graph: captures the same launch into an instantiated CUDA graph
 * (cudaGraphExec_t) for replay with tqr_batched_graph_launch.
 * tqr_batched_autotune: times every (ib, nw) candidate on synthetic problems
 * of each column-count class and stores the fastest in the table (allocates;
 * call it before planning and outside any capture); tqr_batched_tuning reads
 * the table entry for a column count.
 * tqr_?batched_residual: per problem ||A^T (B - A X)||_F /
 * (||A||_F (||A||_F ||X||_F + ||B||_F)) in FP64 from the original A, B and the
 * solution (in B's layout); -1 marks a rejected descriptor. */
#define TQR_BATCH_MAX_M 512
#define TQR_BATCH_MAX_K 8
int tqr_batched_problem_bytes(void);
int tqr_batched_plan(int dtype_bytes, int nprob, const int *m, const int *n, const int *k, void *problems,
                     int *order, long long *a_elems, long long *b_elems);
int tqr_batched_worksize(int dtype_bytes, size_t *bytes);
int tqr_batched_autotune(int dtype_bytes, int force, cudaStream_t stream);
int tqr_batched_tuning(int dtype_bytes, int n, int *ib, int *nw);
int tqr_dbatched_gels(int nprob, const void *problems, const int *order, double *A, double *B, void *work,
                      size_t lwork, cudaStream_t stream);
int tqr_sbatched_gels(int nprob, const void *problems, const int *order, float *A, float *B, void *work,
                      size_t lwork, cudaStream_t stream);
/* ComplexF64 (z) and ComplexF32 (c) batches: the same solve with the complex
 * geqrt!/unmqr!('L','C') arithmetic and LeftUpperTRSM!'s complex divisions
 * (Smith's method, as the tile back-solve), on A and B of tqr_zcomplex /
 * tqr_ccomplex elements.  Plan with dtype_bytes 16 (ComplexF64: 8-column
 * strips) or 8 (ComplexF32, the FP64 table); tqr_batched_worksize(16) covers
 * ComplexF64 and tqr_batched_worksize(8) both FP64 and ComplexF32.  The
 * autotuner, the residual kernel and the graph capture are real-only. */
int tqr_zbatched_gels(int nprob, const void *problems, const int *order, tqr_zcomplex *A, tqr_zcomplex *B,
                      void *work, size_t lwork, cudaStream_t stream);
int tqr_cbatched_gels(int nprob, const void *problems, const int *order, tqr_ccomplex *A, tqr_ccomplex *B,
                      void *work, size_t lwork, cudaStream_t stream);
int tqr_batched_status(const void *work, int *bad, int *first_bad, cudaStream_t stream);
int tqr_dbatched_residual(int nprob, const void *problems, const double *A0, const double *B0,
                          const double *X, double *res, cudaStream_t stream);
int tqr_sbatched_residual(int nprob, const void *problems, const float *A0, const float *B0,
                          const float *X, double *res, cudaStream_t stream);
int tqr_batched_graph(int dtype_bytes, int nprob, const void *problems, const int *order, void *A, void *B,
                      void *work, size_t lwork, void **graph_exec);
int tqr_batched_graph_launch(void *graph_exec, cudaStream_t stream);
int tqr_batched_graph_destroy(void *graph_exec);

/* ---- Differentiable batched QR (no counterpart in NextLA, which has no
 * derivative rules) ----
 * batch problems of one shape m-by-n, 1 <= n <= 256, m >= n, each stored
 * column-major and packed (problem p at offset p m n, ld m; n-by-n matrices
 * at p n n, ld n; tau at p ceil(m/256) n).  Every problem is a flat-tree tile
 * QR over 256-row tiles -- geqrt! on the top tile (src/geqrt.jl:22-68), tsqrt!
 * of the top triangle against each further tile (src/tsqrt.jl:46-126), inner
 * block ib -- run by one CTA of a persistent launch.
 * tqr_?qr_batched_fwd: F (in: A; out: the packed factor, R on/above the top
 * tile's diagonal and the reflectors V below), tau, the explicit thin Q
 * (m-by-n) and R (n-by-n, zero below the diagonal).
 * tqr_?qr_batched_bwd: the adjoint Abar = (Qbar + Q copyltu(M)) R^-T with
 * M = R Rbar^T - Qbar^T Q and copyltu(M) = tril(M) + tril(M,-1)^T, from the
 * saved F and tau (every T factor is recomputed from V and tau by the larft!
 * recursion, src/larft.jl:53-86, so none is kept between the passes) and the
 * cotangents Qbar (m-by-n) and Rbar (n-by-n; only its upper triangle is read).
 * work: 256-byte aligned, tqr_qr_batched_worksize bytes (per-CTA T and n-by-n
 * scratch), shared by both passes.  Argument errors: -1 batch, -2 m, -3 n,
 * -4 ib, -5.. pointers, -8 work too small. */
int tqr_qr_batched_worksize(int dtype_bytes, int m, int n, int ib, size_t *bytes);
/* ComplexF64 (z) and ComplexF32 (c) forms of the forward and the adjoint:
 * the complex tile QR (R's diagonal real, the Householder beta) and
 *   Abar = (Qbar + Q X) R^-H,  X = tril(M,-1) + tril(M,-1)^H + Re diag(M),
 *   M = R Rbar^H - Qbar^H Q,
 * the gradient of a real loss as dL/dRe(A) + i dL/dIm(A).  The backward needs
 * m > n (-2 otherwise): with m == n the last column has one row, keeps tau = 0
 * (src/geqr2.jl:32-35) and a complex R_nn, outside that formula.  Work:
 * tqr_qr_batched_worksize with dtype_bytes 16 (ComplexF64) or 8 (covers FP64
 * and ComplexF32).  Element pointers aligned to the element size. */
int tqr_zqr_batched_fwd(int batch, int m, int n, int ib, tqr_zcomplex *F, tqr_zcomplex *tau, tqr_zcomplex *Q,
                        tqr_zcomplex *R, void *work, size_t lwork, cudaStream_t stream);
int tqr_cqr_batched_fwd(int batch, int m, int n, int ib, tqr_ccomplex *F, tqr_ccomplex *tau, tqr_ccomplex *Q,
                        tqr_ccomplex *R, void *work, size_t lwork, cudaStream_t stream);
int tqr_zqr_batched_bwd(int batch, int m, int n, int ib, const tqr_zcomplex *F, const tqr_zcomplex *tau,
                        const tqr_zcomplex *Qbar, const tqr_zcomplex *Rbar, tqr_zcomplex *Abar, void *work,
                        size_t lwork, cudaStream_t stream);
int tqr_cqr_batched_bwd(int batch, int m, int n, int ib, const tqr_ccomplex *F, const tqr_ccomplex *tau,
                        const tqr_ccomplex *Qbar, const tqr_ccomplex *Rbar, tqr_ccomplex *Abar, void *work,
                        size_t lwork, cudaStream_t stream);
int tqr_dqr_batched_fwd(int batch, int m, int n, int ib, double *F, double *tau, double *Q, double *R,
                        void *work, size_t lwork, cudaStream_t stream);
int tqr_sqr_batched_fwd(int batch, int m, int n, int ib, float *F, float *tau, float *Q, float *R,
                        void *work, size_t lwork, cudaStream_t stream);
int tqr_dqr_batched_bwd(int batch, int m, int n, int ib, const double *F, const double *tau,
                        const double *Qbar, const double *Rbar, double *Abar, void *work, size_t lwork,
                        cudaStream_t stream);
int tqr_sqr_batched_bwd(int batch, int m, int n, int ib, const float *F, const float *tau,
                        const float *Qbar, const float *Rbar, float *Abar, void *work, size_t lwork,
                        cudaStream_t stream);

/* ---- Tensor-core FP32 trailing update (no counterpart in NextLA) ----
 * tsmqr!('L', 'C', ...) (src/tsmqr.jl:47-146, l = 0, ib = 32) on tcgen05
 * tensor cores: [A1; A2] := Q^T [A1; A2] with Q from a tsqrt! factor V
 * (m2-by-k) and T (32-by-k), A1 rows [0, k), m2 = 128 or 256, k a multiple of
 * 32, n a multiple of 128; A1, A2 and V 16-byte aligned with leading
 * dimensions multiples of 4 (-6, -8 otherwise).  TF32 products split three
 * ways (hi*hi + hi*lo + lo*hi) with FP32 accumulation in TMEM: FP32-level
 * accuracy.  *err (device) is set to 1 if a tensor-core completion wait gave
 * up. */
int tqr_stsmqr_tc(int m1, int n, int m2, int k, float *A1, int lda1, float *A2, int lda2, const float *V,
                  int ldv, const float *T, int ldt, int *err, cudaStream_t stream);

/* The FP32 persistent tile kernel (tqr_stile_geqrf_dag, tqr_stile_gels_dag and
 * the mixed solve's factorisation) runs its tsmqr updates as 128-column
 * tensor-core tasks when nb = 256, ib = 32 and A is 16-byte aligned with lda
 * a multiple of 4; tqr_tile_dag_tensor_cores(0) switches that off (SIMT
 * strips only), (1) back on; returns the previous setting.
 * tqr_tile_dag_check_tc: host replay check of that schedule. */
int tqr_tile_dag_tensor_cores(int on);
/* Order of the flat-tree persistent kernel's task list: by default tasks are
 * sorted by their longest path to the end of the graph.
 * tqr_tile_dag_order_quantum(q), q > 0, sorts by that length in buckets of q
 * full-tile strip updates and keeps the algorithm's loop order inside a
 * bucket, so consecutive tasks share their reflector tile while it is in L2
 * (the order stays topological); 0 restores the exact sort.  Applies to
 * schedules built afterwards (each shape's schedule is cached per setting);
 * returns the previous value.  Process-wide. */
double tqr_tile_dag_order_quantum(double q);
/* The tensor-core updates (tqr_stsmqr_tc and the tensor-core tasks of the
 * FP32 persistent kernels) load A2, A1 and V with the tensor memory
 * accelerator (cp.async.bulk.tensor, 128-byte swizzle, tensor maps encoded on
 * the host per launch); tqr_tile_tc_tma(0) makes them use 16-byte cp.async
 * copies into the same layout instead (the same results bit for bit), (1)
 * restores TMA.  Returns the previous setting.  Process-wide. */
int tqr_tile_tc_tma(int on);

/* The same trailing update in compact-WY form (no counterpart call in NextLA:
 * it replaces the chain of ib-blocks that tsmqr!, src/tsmqr.jl:47-146, unmqr!,
 * src/unmqr.jl:99-148, and ttmqr!, src/ttmqr.jl:1-95, apply one after another
 * by Q = I - V T V^T with the k x k T of all blocks).
 * tqr_swy_build: once per V, fills a slot (tqr_swy_slot_bytes() = 1.5 MB,
 *   256-byte aligned, device memory) with V masked by vmode (0 as stored,
 *   tsmqr!; 1 unit lower triangular, geqrt!'s V for unmqr!; 2 upper
 *   triangular, ttmqr!), V^T and that T (from the blocked T, 32 x k, ldt >= 32),
 *   each split hi + lo for TF32x3.  m2 = 128 or 256, k a multiple of 32, k <= m2.
 * tqr_swy_apply: [A1; A2] := Q^T [A1; A2] for n columns (a multiple of 128)
 *   with a built slot; A1 (k x n, null for vmode 1: A2 := Q^T A2) and A2
 *   (m2 x n) 16-byte aligned with leading dimensions multiples of 4.
 * tqr_stsmqr_wy: build (vmode 0) then apply, the tsmqr!('L','C') of
 *   tqr_stsmqr_tc.
 * Same results as the blocked form to FP32 rounding (the products are
 * regrouped).  *err becomes nonzero if a bounded device wait gave up. */
size_t tqr_swy_slot_bytes(void);
int tqr_swy_build(int m2, int k, const float *V, int ldv, const float *T, int ldt, int vmode, void *slot,
                  size_t lslot, int *err, cudaStream_t stream);
int tqr_swy_apply(int m1, int n, int m2, int k, float *A1, int lda1, float *A2, int lda2, const void *slot, int *err,
                  cudaStream_t stream);
int tqr_stsmqr_wy(int m1, int n, int m2, int k, float *A1, int lda1, float *A2, int lda2, const float *V, int ldv,
                  const float *T, int ldt, void *slot, size_t lslot, int *err, cudaStream_t stream);
/* tqr_tile_tc_wy(1) makes the FP32 hierarchical and binary-tree task graphs
 * (tqr_stile_geqrf_hqr_dag, tqr_stile_geqrf_tree_dag and the mixed solve's
 * factorisation) run their tensor-core updates in this compact-WY form: one
 * slot build per reflector tile (geqrt!'s V for the leaders' unmqr!, a
 * merge's V for its tsmqr! or ttmqr!), then every 128-column chunk through
 * it.  The slots sit in the caller's `work` (4 * (m / 256) slots; the
 * worksize queries include them).  Off by default: the graphs apply ib-block
 * by ib-block (tqr_stsmqr_tc's routine), which is about twice as accurate
 * (the WY form adds a TF32x3 product with the k x k T to every update) and,
 * with the mixed solve's FP64 panel steps, no slower.  Returns the previous
 * setting.  Process-wide. */
int tqr_tile_tc_wy(int on);
/* Host replay of that schedule: topological order, every chunk task waits for
 * its own reflector tile's slot build, and every rebuild of a slot waits for
 * all chunks that read its previous contents.  *nbuild, *nchunk: how many
 * builds and chunk tasks.  0 = consistent, 1-3 = which check failed. */
int tqr_tile_hqr_dag_check_wy(int m, int n, int nb, int ib, int grp, int nrhs, long long *nbuild,
                              long long *nchunk);
/* Resident CTAs per SM and dynamic shared memory of the persistent tile
 * kernel at nb = 256, ib = 32 (dtype_bytes 8 or 4; tensor_cores for FP32). */
int tqr_tile_dag_occupancy(int dtype_bytes, int tensor_cores, int *ctas_per_sm, int *smem_bytes);
int tqr_tile_dag_check_tc(int m, int n, int nrhs, int nb, int ib, long long *ntasks);

/* ---- Measurement hooks (no counterpart in NextLA; used by the benchmark) ----
 * tqr_launch_count: kernels this library has launched since it was loaded.
 * tqr_profile_enable / tqr_profile_read: while enabled, the tile driver brackets
 * each trailing-update launch (the band unmqr and tsmqr calls) with CUDA events
 * on the stream it runs on; read returns their count, summed device time (ms)
 * and summed algorithmic flops (4 m2 k n per tsmqr, 2 n k (2 m - k) per
 * unmqr), then forgets them.
 * tqr_fp64_peak_probe: independent DFMA chains, 16 * iters * blocks * 256
 * flops, writing blocks * 256 doubles to out -- the SIMT FP64 ceiling.
 * tqr_fp64_mma_probe: the FP64 tensor-core counterpart.  CTAs of 256 threads;
 * in each, warps 0 .. dmma_warps-1 run 4 independent mma.sync.m8n8k4.f64
 * accumulator chains for iters steps, the other warps 8 DFMA chains per
 * thread; *dmma_flops / *dfma_flops receive the flops of each part
 * (dmma_warps = 8: DMMA alone, 0: DFMA alone).  out takes blocks * 256
 * doubles. */
unsigned long long tqr_launch_count(void);
void tqr_profile_enable(int on);
int tqr_profile_read(long long *launches, double *device_ms, double *flops);
int tqr_fp64_peak_probe(int blocks, int iters, double *out, cudaStream_t stream);
int tqr_fp64_mma_probe(int blocks, int iters, int dmma_warps, double *out, double *dmma_flops,
                       double *dfma_flops, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* TILEQR_H */
