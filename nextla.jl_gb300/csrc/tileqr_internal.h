// tileqr_internal.h -- launchers shared between the translation units.
#pragma once
#include <cuda_runtime.h>

namespace tqr {

// Measurement hooks (diag.cu): every launcher counts its kernels; the tile
// driver brackets its trailing-update launches with prof_begin/prof_end.
void count_launch(unsigned long long n = 1);
bool profiling();
void *prof_begin(cudaStream_t st);
void prof_end(void *tok, cudaStream_t st, double flops);

// geqr2 (+ T when T != nullptr) on an m-by-nc panel: one CTA, or with
// cluster = true a thread-block cluster splitting the rows when the panel is
// tall enough (panel_cluster.cuh; different summation order, same bar).
template <typename R>
cudaError_t launch_panel_qr(int m, int nc, R *A, int lda, R *tau, R *T, int ldt, cudaStream_t st,
                            bool cluster = false);

// One ib-block of tsqrt (pointers already offset to the block), one CTA or
// (cluster = true) a cluster; tt >= 0: the ttqrt block whose first column is
// column tt of the triangle.
template <typename R>
cudaError_t launch_tsqrt_block(int m, int sb, R *A1, int lda1, R *A2, int lda2, R *T, int ldt,
                               R *tau, cudaStream_t st, int tt = -1, bool cluster = false);

// The C-ABI routines' bodies (capi.cu).  `cluster` selects the cluster panel
// for the panel steps: the entry points use it; the stream tile driver does
// not, so that it stays bit-identical to the persistent schedule.
template <typename R>
int geqrt_impl(int m, int n, int ib, R *A, int lda, R *T, int ldt, R *tau, cudaStream_t st, bool cluster);
template <typename R>
int tsqrt_impl(int m, int n, int ib, int m1, R *A1, int lda1, R *A2, int lda2, R *T, int ldt, R *tau,
               cudaStream_t st, bool cluster);
template <typename R>
int unmqr_impl(char side, char trans, int m, int n, int k, int ib, const R *A, int lda, const R *T, int ldt,
               R *C, int ldc, cudaStream_t st);
template <typename R>
int tsmqr_impl(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib, R *A1, int lda1, R *A2,
               int lda2, const R *V, int ldv, const R *T, int ldt, cudaStream_t st);

template <typename R>
cudaError_t launch_larft(int direct_f, int storev_c, int n, int k, const R *V, int ldv,
                         const R *tau, R *T, int ldt, cudaStream_t st);

// Block-reflector apply.  mode 0: larfb/unmqr on C (m-by-n); mode 1: tsmqr on
// [A1; A2] (side L) or [A1 A2] (side R) with C = A2 (m-by-n); mode 1 with
// tt >= 0: reflector q of V holds rows (columns for side R) [0, tt + q] only
// (ttmqr, parfb with a triangular part).
template <typename R>
cudaError_t launch_apply(int mode, char side, char trans, int m, int n, int k, int ib, R *C,
                         int ldc, R *A1, int lda1, const R *V, int ldv, const R *T, int ldt,
                         cudaStream_t st, int tt = -1);

// parfb! in the forms the fused apply does not cover (direct 'B' or storev
// 'R', pamm.cu): pamm 'W' into the caller's work W, the T product, A1 -= W,
// pamm 'A' (src/parfb.jl:121-189).
template <typename R>
int parfb_general(char side, char trans, char direct, char storev, int m2, int n2, int k, int l, R *A1, int lda1,
                  R *A2, int lda2, const R *V, int ldv, const R *T, int ldt, R *W, int ldw, cudaStream_t st);

// The FP32 least-squares factorisation of the mixed solve (dag.cu): as
// tqr_stile_gels_dag, with the panel tasks (geqr2/larfg, larft, the tsqrt
// blocks and their diagonal triangles) in FP64 unless tqr_dsgels_fp64_panels(0)
// switched that off.  Workspace: tqr_tile_gels_worksize covers it.
int stile_gels_dag_mixed(int m, int n, int nrhs, int nb, int ib, float *A, int lda, float *T, int ldt,
                         float *tau, int ldtau, float *B, int ldb, void *work, size_t lwork, cudaStream_t stream);

// Whether FP32 persistent schedules may use the tensor cores
// (tqr_tile_dag_tensor_cores; dag.cu).
bool tile_tc_enabled();

// Tensor maps for the tensor-core chunk routines' TMA loads (tc.cu): a
// column-major FP32 matrix (rows x cols, leading dimension ld) with boxes of
// box_rows x box_cols elements and the 128-byte (or 64-byte) swizzle; tm
// points to a CUtensorMap.  tc_tma_enabled: whether the blocked chunk routine
// loads through TMA (tqr_tile_tc_tma).
cudaError_t make_tmap_f32(void *tm, const float *base, long long rows, long long cols, long long ld, int box_rows,
                          int box_cols, int swizzle_bytes = 128);
bool tc_tma_enabled();
// Whether FP32 task graphs run their tensor-core updates in compact-WY form
// (tc_wy.cuh: one slot build per reflector tile, then three products per
// chunk) rather than ib-block by ib-block (tqr_tile_tc_wy).
bool tc_wy_enabled();
// Whether tqr_dsgels factors with FP64 panel steps (tqr_dsgels_fp64_panels).
bool dsgels_f64p_enabled();

// The mixed solve's factorisation as the hierarchical tree (tree.cu): groups
// of grp tiles reduced flat, the leaders by the binary tree, FP64 panel steps,
// tensor-core trailing updates; B rides along as extra trailing columns, then
// R X = (Q^T B)[0:n].  T2, tau2 as for tqr_stile_geqrf_hqr_dag; work from
// tree_dag_work_bytes.
int stile_gels_hqr_mixed(int m, int n, int nrhs, int nb, int ib, int grp, float *A, int lda, float *T, float *T2,
                         int ldt, float *tau, float *tau2, int ldtau, float *B, int ldb, void *work, size_t lwork,
                         cudaStream_t stream);
size_t tree_dag_work_bytes(int m, int n, int nb, int ib, int grp, int nrhs);

}  // namespace tqr
