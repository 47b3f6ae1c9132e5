/*
 * CPU oracle for the block-sparse hot path — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's CPU arithmetic
 * (gevtushenko/block_matrix_format_performance). It exists to check the CUDA
 * library, never to be shipped or measured as the product: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * Pinning: the conversion, generator and comparison routines are checked
 * bit-exactly against golden vectors produced by the reference's own headers
 * (common/matrix_converters.h, common/measurement_class.h,
 * fem_2d/golden_gate_bridge.h) compiled in place — see oracle/ref/.
 * The BiCGStab recurrences (gpu/bicgstab.cu) have no reference golden vector
 * (the reference solver only prints residuals); they are pinned against an
 * independent FP64 direct solve in the tests.
 */
#ifndef BMFP_ORACLE_H
#define BMFP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* y = A*x over CSR, one thread; main.cpp:36-45 (the reference also sets
 * x := 1, y := 0 first, main.cpp:27-28 — here x is an input). */
void orc_csr_spmv_f64 (int n_rows, const int *row_ptr, const int *cols,
                       const double *vals, const double *x, double *y);
void orc_csr_spmv_f32 (int n_rows, const int *row_ptr, const int *cols,
                       const float *vals, const float *x, float *y);

/* Same loop, rows split over n_threads POSIX threads. Every row is summed in
 * the same order as the single-thread loop, so results are bit-identical. */
void orc_csr_spmv_mt_f64 (int n_rows, const int *row_ptr, const int *cols,
                          const double *vals, const double *x, double *y, int n_threads);
void orc_csr_spmv_mt_f32 (int n_rows, const int *row_ptr, const int *cols,
                          const float *vals, const float *x, float *y, int n_threads);

/* y = A*x directly over BCSR with row-major bs*bs blocks (definition of the
 * layout in common/matrix_converters.h:13-82); summation order equals the CSR
 * loop over the converted matrix, so it is bit-identical to
 * orc_csr_spmv_* after orc_bcsr_to_csr_*. */
void orc_bcsr_spmv_f64 (int n_block_rows, int bs, const int *row_ptr, const int *cols,
                        const double *vals, const double *x, double *y);
void orc_bcsr_spmv_f32 (int n_block_rows, int bs, const int *row_ptr, const int *cols,
                        const float *vals, const float *x, float *y);

/* BCSR -> CSR, common/matrix_converters.h:88-117. Output arrays sized
 * n_block_rows*bs+1, nnzb*bs*bs, nnzb*bs*bs. */
void orc_bcsr_to_csr_f64 (int n_block_rows, int bs, const int *brow_ptr, const int *bcols,
                          const double *bvals, int *row_ptr, int *cols, double *vals);
void orc_bcsr_to_csr_f32 (int n_block_rows, int bs, const int *brow_ptr, const int *bcols,
                          const float *bvals, int *row_ptr, int *cols, float *vals);

/* CSR -> BCSR (no reference counterpart: inverse of the conversion above).
 * Pass 1 returns nnzb and fills brow_ptr[n_rows/bs+1]; pass 2 fills columns
 * (sorted, distinct) and row-major block values, zero where CSR has no entry.
 * Returns -1 if n_rows is not a multiple of bs or a column is out of range. */
int64_t orc_csr_to_bcsr_count (int n_rows, int n_cols, int bs, const int *row_ptr,
                               const int *cols, int *brow_ptr);
int orc_csr_to_bcsr_fill_f64 (int n_rows, int bs, const int *row_ptr, const int *cols,
                              const double *vals, const int *brow_ptr, int *bcols, double *bvals);
int orc_csr_to_bcsr_fill_f32 (int n_rows, int bs, const int *row_ptr, const int *cols,
                              const float *vals, const int *brow_ptr, int *bcols, float *bvals);

/* Row-major -> column-major per block, common/matrix_converters.h:32-49. */
void orc_transpose_blocks_f64 (int n_block_rows, int bs, const int *row_ptr,
                               const double *vals, double *out);
void orc_transpose_blocks_f32 (int n_block_rows, int bs, const int *row_ptr,
                               const float *vals, float *out);

/* Contiguous band generator, common/matrix_converters.h:157-196. Arrays sized
 * n_rows+1, n_rows*blocks_per_row, n_rows*blocks_per_row*bs*bs. */
void orc_gen_n_diag_bcsr_f64 (int n_rows, int blocks_per_row, int bs,
                              int *row_ptr, int *cols, double *vals);
void orc_gen_n_diag_bcsr_f32 (int n_rows, int blocks_per_row, int bs,
                              int *row_ptr, int *cols, float *vals);

/* compare_results, common/measurement_class.h:58-87: returns
 * sum((a-b)^2)/sum(b^2) computed in the element type; *flagged is set to 1
 * when the reference would print "ERROR" (error > 1e-9). */
double orc_compare_results_f64 (unsigned n, const double *a, const double *b, int *flagged);
double orc_compare_results_f32 (unsigned n, const float *a, const float *b, int *flagged);

/* BiCGStab over CSR, the recurrences of gpu/bicgstab.cu:387-513, with point
 * Jacobi right preconditioning when use_precond (gpu/bicgstab.cu:201-238).
 * Differences from the reference, on purpose: the returned x is the last
 * iterate (the reference copies buffer half 0, bicgstab.cu:515), dot products
 * are sequential (deterministic) and nothing is printed.
 * Returns 0 converged, 1 max iterations, 2 breakdown (rho, (rh,v) or (t,t) = 0).
 * *iters = iterations done; *rel_res = recursive |r|/|b| at exit. */
int orc_bicgstab_f64 (int n, const int *row_ptr, const int *cols, const double *vals,
                      const double *b, double *x, double eps, int max_iterations,
                      int use_precond, int *iters, double *rel_res);

/* Seeded random-band generator (the block-size sweep's workload, restated
 * from its specification): orc_band_blocks gives block row i's block count;
 * orc_gen_band fills BCSR (csr = 0: row_ptr = block-row offsets) or CSR
 * (csr = 1: row_ptr = scalar-row offsets) columns and values (is_f64: double,
 * else float), on `threads` host threads. */
int orc_band_blocks (int nbr, int bpr, int half, int i);
void orc_gen_band (int nbr, int bpr, int half, int bs, uint64_t seed, int is_f64, int csr,
                   const int64_t *row_ptr, int *cols, void *vals, int threads);
void orc_gen_uniform_vector (int64_t n, uint64_t seed, uint64_t stream, int is_f64, void *out);
/* orc_bicgstab_f64's recurrences on `threads` host threads (rows split in
 * contiguous ranges, dot products summed in thread order). */
int orc_bicgstab_mt_f64 (int n, const int *row_ptr, const int *cols, const double *vals, const double *b,
                         double *x, double eps, int max_iterations, int use_precond, int threads, int *iters,
                         double *rel_res);

/* Block Jacobi: the inverses of the bs x bs diagonal blocks of a CSR matrix
 * (n rows = n/bs block rows), and BiCGStab with that right preconditioner. */
void orc_block_jacobi_f64 (int n, int bs, const int *row_ptr, const int *cols, const double *vals, double *Minv);
int orc_bicgstab_bj_f64 (int n, int bs, const int *row_ptr, const int *cols, const double *vals,
                         const double *b, double *x, double eps, int max_iterations, int *iters, double *rel_res);

#ifdef __cplusplus
}
#endif

#endif
