/*
 * bmfp.h — C ABI of the GB300 (sm_103a) block-sparse library.
 *
 * One shared library, libbmfp.so, exports every function below with C
 * linkage: plain pointers and sizes, no C++ or torch types. The C++ headers
 * under include/bmfp/ rebuild the reference's own host API
 * (gpu_csr_spmv / gpu_csr_vector_spmv / gpu_bcsr_spmv, gpu_bicgstab,
 * bcsr_matrix_class / csr_matrix_class, measurement_class) on top of it.
 *
 * Each entry names the reference interface it replaces (paths inside
 * gevtushenko/block_matrix_format_performance).
 *
 * Conventions
 *  - Every function returns an int status (BMFP_SUCCESS == 0). On failure
 *    bmfp_last_error() returns a message for the calling thread. Nothing in
 *    the library prints, exits or resets the device (the reference's
 *    gpuCheck did both, gpu/bicgstab.cu:12-21).
 *  - Indices are 32-bit signed (the reference instantiates index_type=int,
 *    gpu/gpu_matrix_multiplier.cu:1338-1339).
 *  - BCSR values: nnzb blocks of bs*bs, row-major inside a block
 *    (common/matrix_converters.h:26), or column-major where a variant says
 *    so (the transpose_blocks layout, common/matrix_converters.h:32-49).
 *  - "d_" pointers are device memory, "h_" pointers host memory.
 *  - stream is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    Device work is asynchronous on that stream unless a function says
 *    otherwise.
 */
#ifndef BMFP_H
#define BMFP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define BMFP_API __attribute__ ((visibility ("default")))
#else
#define BMFP_API
#endif

/* ----------------------------------------------------------------- status */
enum bmfp_status
{
  BMFP_SUCCESS = 0,
  BMFP_ERROR_INVALID_VALUE = 1, /* bad size, pointer, enum or layout */
  BMFP_ERROR_CUDA = 2,          /* a CUDA runtime / cuSPARSE call failed */
  BMFP_ERROR_OUT_OF_MEMORY = 3, /* device allocation failed */
  BMFP_ERROR_NOT_SUPPORTED = 4, /* valid request this build does not serve */
  BMFP_ERROR_BREAKDOWN = 5,     /* BiCGStab rho, (rh,v) or (t,t) vanished */
  BMFP_ERROR_NOT_CONVERGED = 6, /* iteration limit reached before tolerance */
  BMFP_ERROR_TIMEOUT = 7,       /* a bounded device wait gave up */
  BMFP_ERROR_BUDGET = 8,        /* request does not fit the HBM budget */
  BMFP_PENDING = 9              /* asynchronous request not finished yet */
};

enum bmfp_dtype
{
  BMFP_R32F = 0, /* float  */
  BMFP_R64F = 1  /* double */
};

/* Thread-local message of the last failure on the calling thread. */
BMFP_API const char *bmfp_last_error (void);
/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
BMFP_API int bmfp_version (void);
/* Number of CUDA devices visible (0 on a host without a GPU; never fails). */
BMFP_API int bmfp_device_count (void);

/* ------------------------------------------------------------ SpMV kernels
 * Variants keep the reference's format strings (the keys of its result.json,
 * gpu/gpu_matrix_multiplier.cu and main.cpp). Each is a GB300 kernel written
 * for this library with that variant's thread mapping; BMFP_SPMV_BCSR_NATIVE
 * and BMFP_SPMV_CSR_NATIVE are the tuned sm_103a kernels.
 *
 *  variant                                value layout  reference
 *  CSR_SCALAR     "GPU CSR"                     CSR     csr_spmv_kernel .cu:65-86
 *  CSR_VECTOR     "GPU CSR-Vector"              CSR     csr_spmv_vector_kernel .cu:165-196
 *  CSR_NATIVE     "GPU CSR (GB300 sub-warp)"    CSR     (new)
 *  BCSR_ROW_THREAD "GPU BCSR (row major, thread per row)"        row  .cu:275-304
 *  BCSR_ROW_WARP   "GPU BCSR (row major, warp per row)"          row  .cu:306-339
 *  BCSR_COL_THREAD "GPU BCSR (column major, thread per row)"     col  .cu:341-370
 *  BCSR_COL_THREAD_TEMPLATE "... thread per row, template)"      col  .cu:372-400
 *  BCSR_COL_COAL_X "... thread per row, coal x)"                 col  .cu:402-435
 *  BCSR_COL_COAL_X_TEMPLATE "... coal x, template)"              col  .cu:437-469
 *  BCSR_COL_BY_COL "GPU BCSR (column major, column-by-column)"   col  .cu:485-528
 *  BCSR_COL_BY_COL_FASTDIV "... column-by-column, int fastdiv)"  col  .cu:530-576
 *  BCSR_COL_BY_COL_PO2 "... column-by-column, int po2)"          col  .cu:584-629
 *  BCSR_COL_BY_COL_TEMPLATE "... column-by-column, template)"    col  .cu:631-673
 *  BCSR_JIT        "jit" (bs-specialised column-by-column)       col  main.cpp:178-230
 *  CUSPARSE_ROW    "GPU BSR (cuSPARSE, row major)"               row  .cu:676-734,879
 *  CUSPARSE_COL    "GPU BSR (cuSPARSE, column major)"            col  .cu:927
 *  BCSR_NATIVE     "GPU BCSR (GB300 native)"                     row  (new)
 *
 * Fixes over the reference, on purpose: the coal-x variants stage the x
 * segment of every block row they serve (the reference's only read the first
 * block row's segment, correct only for constant x), and column-by-column
 * handles block sizes that do not divide 32.
 */
enum bmfp_spmv_variant
{
  BMFP_SPMV_CSR_SCALAR = 0,
  BMFP_SPMV_CSR_VECTOR = 1,
  BMFP_SPMV_CSR_NATIVE = 2,
  BMFP_SPMV_BCSR_ROW_THREAD = 3,
  BMFP_SPMV_BCSR_ROW_WARP = 4,
  BMFP_SPMV_BCSR_COL_THREAD = 5,
  BMFP_SPMV_BCSR_COL_THREAD_TEMPLATE = 6,
  BMFP_SPMV_BCSR_COL_COAL_X = 7,
  BMFP_SPMV_BCSR_COL_COAL_X_TEMPLATE = 8,
  BMFP_SPMV_BCSR_COL_BY_COL = 9,
  BMFP_SPMV_BCSR_COL_BY_COL_FASTDIV = 10,
  BMFP_SPMV_BCSR_COL_BY_COL_PO2 = 11,
  BMFP_SPMV_BCSR_COL_BY_COL_TEMPLATE = 12,
  BMFP_SPMV_BCSR_JIT = 13,
  BMFP_SPMV_CUSPARSE_ROW = 14,
  BMFP_SPMV_CUSPARSE_COL = 15,
  BMFP_SPMV_BCSR_NATIVE = 16,
  BMFP_SPMV_VARIANT_COUNT = 17
};

/* Reference format string of a variant ("GPU CSR", ...), or NULL. */
BMFP_API const char *bmfp_spmv_variant_name (int variant);
/* 1 if the variant reads column-major blocks, 0 row-major/CSR, -1 invalid. */
BMFP_API int bmfp_spmv_variant_layout (int variant);
/* 1 if the variant multiplies CSR, 0 BCSR, -1 invalid. */
BMFP_API int bmfp_spmv_variant_is_csr (int variant);

/* y = A x over device CSR arrays (n_rows+1 row offsets, nnz columns/values).
 * Replaces the kernels launched by gpu_csr_spmv / gpu_csr_vector_spmv
 * (gpu/gpu_matrix_multiplier.cu:88-163, 198-273) without their per-call
 * allocation and copies. variant: CSR_SCALAR, CSR_VECTOR or CSR_NATIVE. */
BMFP_API int bmfp_csr_spmv (int dtype, int variant, int n_rows, int n_cols, int64_t nnz,
                            const int *d_row_ptr, const int *d_cols, const void *d_values,
                            const void *d_x, void *d_y, void *stream);

/* y = A x over device BCSR arrays (n_block_rows+1 offsets, nnzb block
 * columns, nnzb*bs*bs values in the variant's layout). Replaces the kernel
 * launches inside gpu_bcsr_spmv (gpu/gpu_matrix_multiplier.cu:736-1331) and
 * the JIT launch (main.cpp:232-294). */
BMFP_API int bmfp_bcsr_spmv (int dtype, int variant, int n_block_rows, int n_block_cols, int bs,
                             int64_t nnzb, const int *d_row_ptr, const int *d_cols,
                             const void *d_values, const void *d_x, void *d_y, void *stream);

/* Lanes per block row the native kernel would use for this shape (0 = the
 * built-in heuristic); lets callers and the autotuner pin the choice.
 * Valid values: 0, 2, 4, 8, 16, 32 (a group of that many lanes walks the
 * block row's values in 16-byte vectors; needs lanes * 16 bytes >= one block
 * line), or BMFP_LANES_ROW_OWNER (bs in {4,8,16,32}: one lane per scalar
 * row, no cross-lane reduction). Affects only BMFP_SPMV_BCSR_NATIVE. */
#define BMFP_LANES_ROW_OWNER 64
/* Matrix handles only (bmfp_matrix_set_lanes / bmfp_matrix_autotune): one lane
 * per scalar row over a column-major copy of the blocks that the handle then
 * keeps, so the lanes of a block read one contiguous column per load. The
 * fastest FP64 mapping from bs 16 on (GB300's FP64 pipe busy most of the
 * time); costs a second copy of the values in HBM. bs in {2,4,8,16,32}. */
#define BMFP_LANES_COL_OWNER 65
BMFP_API int bmfp_bcsr_spmv_native_ex (int dtype, int n_block_rows, int bs, int64_t nnzb,
                                       const int *d_row_ptr, const int *d_cols,
                                       const void *d_values, const void *d_x, void *d_y,
                                       int lanes_per_block_row, void *stream);
BMFP_API int bmfp_bcsr_native_default_lanes (int dtype, int bs, double avg_blocks_per_row);
/* The column-owner product (BMFP_LANES_COL_OWNER) on caller arrays whose
 * blocks are already column-major (the transpose_blocks layout the
 * reference's column-major variants take, gpu/gpu_matrix_multiplier.cu:
 * 341-400). bs in {2,4,8,16,32}. The fastest FP64 product from bs 8 on
 * with the matrix coming from HBM, and at every bs while it stays in L2. */
BMFP_API int bmfp_bcsr_spmv_colmajor (int dtype, int n_block_rows, int bs, int64_t nnzb,
                                      const int *d_row_ptr, const int *d_cols,
                                      const void *d_values_colmajor, const void *d_x, void *d_y,
                                      void *stream);

/* Measured FMA throughput of the current device in GFLOP/s (2 flop per FMA)
 * for dtype R64F or R32F: a few milliseconds of independent FMA chains on
 * every SM. FP64 sparse products are bound by it on GB300 (one FMA per value,
 * so at most 4 bytes per FP64 flop); bench.py reports both rooflines. */
BMFP_API int bmfp_measure_fma_peak (int dtype, double *gflops, void *stream);

/* Launches one plain streaming read of `bytes` device bytes at d_buf (16-byte
 * aligned, bytes a multiple of 16) on `stream`, for the caller to time like a
 * product: the size-matched floor of a small SpMV, whose launch ramp, first
 * DRAM round trips and tail no kernel avoids (no reference counterpart). */
BMFP_API int bmfp_stream_read (const void *d_buf, size_t bytes, void *stream);

/* One-shot product on HOST buffers: y = A x with the BCSR arrays (row-major
 * blocks; bs = 1 is CSR), x and y all in host memory, the call returning when
 * h_y holds the result. Replaces what each gpu_bcsr_spmv / gpu_csr_spmv call
 * of the reference does around its kernels (gpu/gpu_matrix_multiplier.cu:
 * 106-115 and 757-766 allocate and upload, :151-156 download, :158-160 free)
 * for callers that keep their matrices on the host. The upload is split into
 * block-row chunks: the product of chunk k runs while chunk k+1 is still
 * crossing the host link, so the call costs about one transfer of the
 * arrays. Device memory comes from a stream-ordered pool private to the
 * library that keeps up to 16 GiB per device for the next call. Pinned host
 * buffers (cudaHostAlloc / cudaHostRegister) give full link speed; pageable
 * ones work through the driver's staging copies. lanes as for
 * bmfp_bcsr_spmv_native_ex (0 = built-in choice). stream: the stream the
 * copies are ordered on (NULL = legacy default). */
BMFP_API int bmfp_bcsr_spmv_host (int dtype, int n_block_rows, int n_block_cols, int bs,
                                  int64_t nnzb, const int *h_row_ptr, const int *h_cols,
                                  const void *h_values, const void *h_x, void *h_y, int lanes,
                                  void *stream);

/* ------------------------------------------------ device matrix handles ---
 * A device-resident BCSR (or CSR when bs is given as 0 to *_csr) matrix owned
 * by the library: one upload, then any number of products. The reference
 * re-allocated and re-uploaded per call (gpu/gpu_matrix_multiplier.cu:106-115,
 * 757-766). */
typedef struct bmfp_matrix_s *bmfp_matrix_t;

/* Upload a host BCSR matrix with row-major blocks. dtype is the storage and
 * arithmetic type on the device. Synchronous with respect to the host
 * arrays (they may be freed on return). */
BMFP_API int bmfp_matrix_create_bcsr (bmfp_matrix_t *out, int dtype, int n_block_rows,
                                      int n_block_cols, int bs, int64_t nnzb,
                                      const int *h_row_ptr, const int *h_cols,
                                      const void *h_values, void *stream);
/* Upload a host CSR matrix. */
BMFP_API int bmfp_matrix_create_csr (bmfp_matrix_t *out, int dtype, int n_rows, int n_cols,
                                     int64_t nnz, const int *h_row_ptr, const int *h_cols,
                                     const void *h_values, void *stream);
/* Same from arrays already on the device (copied device-to-device). */
BMFP_API int bmfp_matrix_create_bcsr_device (bmfp_matrix_t *out, int dtype, int n_block_rows,
                                             int n_block_cols, int bs, int64_t nnzb,
                                             const int *d_row_ptr, const int *d_cols,
                                             const void *d_values, void *stream);
/* A copy of a matrix converted to another value type on the device
 * (e.g. the FP32 shadow of an FP64 operator for mixed precision). */
BMFP_API int bmfp_matrix_convert (bmfp_matrix_t *out, bmfp_matrix_t src, int dtype, void *stream);
BMFP_API int bmfp_matrix_destroy (bmfp_matrix_t m);
/* Shape query: any output pointer may be NULL. bs = 0 for CSR. */
BMFP_API int bmfp_matrix_info (bmfp_matrix_t m, int *dtype, int *n_rows, int *n_cols, int *bs,
                               int64_t *nnz_blocks, int64_t *bytes_per_spmv);
/* Device pointers of the stored arrays (values in row-major blocks). */
BMFP_API int bmfp_matrix_device_arrays (bmfp_matrix_t m, const int **d_row_ptr,
                                        const int **d_cols, const void **d_values);
/* y = A x with the tuned kernel (native BCSR or native CSR). x and y are
 * device vectors of the matrix dtype, n_cols*bs and n_rows*bs long. */
BMFP_API int bmfp_matrix_spmv (bmfp_matrix_t m, const void *d_x, void *d_y, void *stream);
/* Time candidate lane counts on this matrix (CUDA events, synchronises the
 * stream) and keep the fastest for later bmfp_matrix_spmv calls. x and y are
 * scratch device vectors of the right size. Optional: the default choice is
 * the built-in heuristic. */
BMFP_API int bmfp_matrix_autotune (bmfp_matrix_t m, const void *d_x, void *d_y, void *stream,
                                   int *chosen_lanes);
/* Pin the native kernel's mapping for this handle (values as for
 * bmfp_bcsr_spmv_native_ex, plus BMFP_LANES_COL_OWNER, which builds the
 * column-major copy; any other value releases it). Like bmfp_matrix_autotune
 * it changes the handle: do not call either while another thread multiplies
 * with the same handle. */
BMFP_API int bmfp_matrix_set_lanes (bmfp_matrix_t m, int lanes, void *stream);

/* ------------------------------------------------------------- BiCGStab ---
 * Replaces gpu_bicgstab<T,C> (gpu/bicgstab.h:10-16, gpu/bicgstab.cu:23-526):
 * the same recurrences and optional point-Jacobi right preconditioning, with
 * the scalars kept on the device, the vector updates and dot products fused
 * into five phase kernels per iteration and the iterations launched as CUDA
 * graphs. A solver is bound to one matrix handle; solves may be repeated with
 * different right-hand sides. */
enum bmfp_solve_precision
{
  BMFP_SOLVE_FP64 = 0,  /* FP64 matrix, vectors and recurrences */
  BMFP_SOLVE_FP32 = 1,  /* FP32 matrix (converted if needed), vectors and recurrences */
  BMFP_SOLVE_MIXED = 2  /* FP32 inner BiCGStab on an FP32 copy of the matrix; true
                           residual b - A x, solution update and the outer
                           convergence norm in FP64 (iterative refinement) */
};

enum bmfp_preconditioner
{
  BMFP_PRECOND_NONE = 0,
  BMFP_PRECOND_JACOBI = 1, /* P = 1/a_ii from the diagonal blocks, bicgstab.cu:201-238 */
  BMFP_PRECOND_BLOCK_JACOBI = 2 /* P = inverse of each bs x bs diagonal block (identity where the
                                   block is missing or singular): the block form of the rule above;
                                   single-system solver, bs <= 8 */
};

enum bmfp_launch_mode
{
  BMFP_LAUNCH_AUTO = 0,       /* persistent from 1 000 000 rows up when it can run, else graphs */
  BMFP_LAUNCH_GRAPH = 1,      /* a CUDA graph of five phase kernels per iteration */
  BMFP_LAUNCH_PERSISTENT = 2  /* one cooperative kernel per iterations_per_graph iterations, the
                                 phases separated by grid barriers, over min(ctas_per_sm, 3) CTAs
                                 per SM (no preconditioner or point Jacobi; any bs but 8, 16,
                                 32); BMFP_ERROR_NOT_SUPPORTED where it cannot run */
};

typedef struct bmfp_solver_options
{
  int precision;            /* enum bmfp_solve_precision */
  int preconditioner;       /* enum bmfp_preconditioner */
  double tolerance;         /* target ||b - A x|| / ||b|| */
  int max_iterations;       /* BiCGStab iterations in total (FP64 and FP32) */
  int check_true_residual;  /* 1 (default): at the end verify b - A x in the matrix
                               precision and restart from it while it is above
                               tolerance; 0: stop on the recursive residual only,
                               as gpu/bicgstab.cu:512 does */
  double inner_tolerance;   /* MIXED: residual reduction asked of each FP32 inner solve */
  int inner_max_iterations; /* MIXED: iteration cap of one inner solve */
  int max_refinements;      /* MIXED: outer refinement steps */
  int fallback_fp64;        /* MIXED: when an outer step cuts the FP64 residual by less
                               than 4x, finish with FP64 BiCGStab from the current x */
  int iterations_per_graph; /* BiCGStab iterations per CUDA graph launch */
  int ctas_per_sm;          /* persistent grid of the single-system solver: CTAs of 256
                               threads per SM (default 4); the grid fixes the summation
                               order, so results are bitwise repeatable for a given value */
  int inner_stall_iterations; /* MIXED: an FP32 inner solve whose best recursive residual
                               has not halved within this many iterations (of its start or
                               of its last halving) is stopped there; it is applied if it
                               halved at least once. 0 = never */
  int residual_replacement; /* 1 (default): FP64 BiCGStab replaces its recursive residual
                               by the true one near convergence (van der Vorst and Ye,
                               group update), so stopping on it also meets the tolerance in
                               b - A x; applies when check_true_residual is 1 (with 0 the
                               reference's plain recurrences run) */
  int launch_mode;          /* enum bmfp_launch_mode (default AUTO). On the same grid (ctas_per_sm
                               <= 3) both modes give the same bits. The persistent kernel holds
                               every SM for its launch, so other work on the GPU waits for it
                               (the server's lanes, which share the GPU with the batched
                               solver, use graphs) */
} bmfp_solver_options;

typedef struct bmfp_solve_info
{
  int status;                    /* BMFP_SUCCESS, BMFP_ERROR_NOT_CONVERGED or BMFP_ERROR_BREAKDOWN */
  int iterations;                /* all BiCGStab iterations */
  int iterations_fp32;           /* of which FP32 (inner) iterations */
  int refinements;               /* MIXED outer steps */
  int restarts;                  /* restarts from the true residual */
  int used_fp64_fallback;        /* MIXED finished in FP64 */
  double true_rel_residual;      /* ||b - A x|| / ||b||, computed in the matrix precision */
  double recursive_rel_residual; /* BiCGStab's own residual at exit */
  double seconds;                /* host wall time of the solve */
  int replacements;              /* residual replacements (FP64 iterations) */
  int pad;
} bmfp_solve_info;

typedef struct bmfp_solver_s *bmfp_solver_t;

/* Defaults: FP64, no preconditioner, tolerance 1e-10, 100000 iterations,
 * true-residual check on, inner tolerance 1e-4, 1000 inner iterations,
 * 30 refinements, FP64 fallback on, 16 iterations per graph. */
BMFP_API void bmfp_solver_options_init (bmfp_solver_options *opts);
/* Allocate the Krylov vectors and capture the iteration graph. The matrix must
 * be square and must outlive the solver (for MIXED it must be FP64). This call
 * synchronises the stream; the reference constructor's 80 %-of-memory guard
 * (bicgstab.cu:41-42) becomes BMFP_ERROR_OUT_OF_MEMORY from the allocations.
 * MIXED with fallback_fp64: creation probes the matrix once (the FP32
 * refinement phase on a seeded right-hand side uniform in [-1, 1)); when
 * that phase would fall back to FP64, every solve of this solver runs FP64
 * only (info->used_fp64_fallback = 1, no FP32 iterations). The choice
 * depends on the matrix alone, never on earlier solves. */
BMFP_API int bmfp_solver_create (bmfp_solver_t *out, bmfp_matrix_t A, const bmfp_solver_options *opts,
                                 void *stream);
/* Solve A x = b from x0 = 0. b and x are device vectors of the matrix dtype
 * (FP64 for MIXED). Blocks until the solve ends; x holds the last iterate
 * whatever the status. Returns info->status. */
BMFP_API int bmfp_solver_solve (bmfp_solver_t s, const void *d_b, void *d_x, bmfp_solve_info *info,
                                void *stream);
BMFP_API int bmfp_solver_destroy (bmfp_solver_t s);
/* Failure detection of the persistent iteration kernel, exercised without a
 * fault: one cooperative launch whose grid barrier waits for one CTA more
 * than the grid holds, so every CTA gives up after limit_seconds (0 < limit
 * <= 1), records the fault and returns. *fault receives the flag the solver's
 * host loop reads (1), *elapsed_seconds the launch's duration; the context
 * stays usable. Synchronises the stream. */
BMFP_API int bmfp_selftest_barrier_timeout (double limit_seconds, int *fault, double *elapsed_seconds,
                                            void *stream);

/* -------------------------------------------------------------- batched ---
 * Many independent square systems of uneven size solved by ONE persistent
 * kernel launch, captured with its work-queue reset in a CUDA graph. Teams
 * of 1-8 CTAs (a thread-block cluster on as many SMs) take systems largest
 * first and solve each one alone, with cluster barriers between phases and
 * dot products reduced through distributed shared memory in a fixed order:
 * a system's result is bitwise the same whatever else is in the batch, for a
 * given configuration. Options as for bmfp_solver_create (FP64, FP32 or
 * MIXED; no preconditioner). Matrices must be FP64 handles with bs <= 32 and
 * must outlive the batch. No counterpart in the reference, which solves one
 * CSR system per call (gpu/bicgstab.cu:387-526). */
typedef struct bmfp_batch_s *bmfp_batch_t;

BMFP_API int bmfp_batch_create (bmfp_batch_t *out, int n_systems, const bmfp_matrix_t *matrices,
                                const bmfp_solver_options *opts, void *stream);
/* Cluster size (1, 2, 4, 8) and threads per CTA (multiple of 64, <= 512). */
BMFP_API int bmfp_batch_configure (bmfp_batch_t b, int cluster_size, int threads_per_cta);
/* The project's autotuner: times every (cluster 4, 8) x (threads 256, 512)
 * candidate on this batch with each system capped at probe_iterations and
 * keeps the fastest. The cap decides what is timed: it must reach a good
 * part of the largest systems' iteration counts to rank the candidates as
 * the full solve does (on the uneven elasticity batch 1024; 128 picks a
 * configuration 40 % slower), at about 1.3 s per 256 iterations there.
 * Outputs may be NULL. Synchronises the stream. A new batch starts at
 * cluster 8 x 512 threads, the fastest on that batch. */
BMFP_API int bmfp_batch_autotune (bmfp_batch_t b, const void *const *d_b, void *const *d_x,
                                  int probe_iterations, int *cluster_size, int *threads_per_cta,
                                  void *stream);
/* Solve every system: d_b[i], d_x[i] are FP64 device vectors (host arrays of
 * n_systems device pointers). infos[i] receives each system's result. Blocks
 * until done; returns BMFP_SUCCESS when every system converged, else the
 * first failing system's status. */
BMFP_API int bmfp_batch_solve (bmfp_batch_t b, const void *const *d_b, void *const *d_x,
                               bmfp_solve_info *infos, void *stream);
BMFP_API int bmfp_batch_destroy (bmfp_batch_t b);

/* -------------------------------------------------------------- serving ---
 * Continuous batching of solve requests on one GPU (no counterpart in the
 * reference). Requests (a resident FP64 matrix handle and a host right-hand
 * side) are admitted in arrival order while their device memory fits the HBM
 * budget and the in-flight limit, and launched as a micro-batch of the
 * batched kernel on an idle stream, so new requests start while earlier ones
 * are still on the GPU; while every stream is busy, arrivals wait and the next
 * launch takes up to max_batch of them at once. Requests with more
 * than wide_threshold_rows rows run on whole-GPU engine lanes. Matrices stay
 * resident (the caller keeps the handles alive until the server is
 * destroyed); each request's Krylov state lives on the device from admission
 * to completion. A request's result does not depend on the other requests in
 * flight. Thread-safe: submit, poll and wait may be called from any thread. */
typedef struct bmfp_server_s *bmfp_server_t;

typedef struct bmfp_server_options
{
  size_t hbm_budget_bytes;     /* device bytes for admitted requests (default 120 GiB) */
  int max_in_flight;           /* requests on the device at once (default 4096) */
  int max_batch;               /* requests per micro-batch launch (default 64) */
  int streams;                 /* concurrent micro-batches (default 8) */
  int cluster_size;            /* CTAs per system team (default 4) */
  int threads_per_cta;         /* default 512 */
  int64_t wide_threshold_rows; /* larger requests use the whole-GPU engine (default 200000) */
  int wide_lanes;              /* whole-GPU solves run concurrently (default 8) */
  bmfp_solver_options solver;  /* precision, tolerance, limits; no preconditioner;
                                  ctas_per_sm defaults to 1 here (eight lanes share the SMs) */
} bmfp_server_options;

typedef struct bmfp_server_stats
{
  uint64_t submitted, completed, micro_batches, wide_solves;
  size_t bytes_in_use, peak_bytes;
  int in_flight, pending;
} bmfp_server_stats;

BMFP_API void bmfp_server_options_init (bmfp_server_options *opts);
/* Start the dispatcher on the current device. */
BMFP_API int bmfp_server_create (bmfp_server_t *out, const bmfp_server_options *opts);
/* Queue a request; h_b is copied, h_x (n doubles) is written on completion
 * and must stay valid until then. BMFP_ERROR_BUDGET if the request alone can
 * never fit the budget. */
BMFP_API int bmfp_server_submit (bmfp_server_t s, bmfp_matrix_t A, const double *h_b, double *h_x,
                                 uint64_t *ticket);
/* BMFP_PENDING while running; otherwise the request's final status, with
 * info filled (info->seconds = submit-to-completion latency) and the ticket
 * released. */
BMFP_API int bmfp_server_poll (bmfp_server_t s, uint64_t ticket, bmfp_solve_info *info);
/* As poll, but blocks until the request completes. */
BMFP_API int bmfp_server_wait (bmfp_server_t s, uint64_t ticket, bmfp_solve_info *info);
BMFP_API int bmfp_server_get_stats (bmfp_server_t s, bmfp_server_stats *stats);
/* Finish every queued request, then stop and free the server. */
BMFP_API int bmfp_server_destroy (bmfp_server_t s);

/* BiCGStab that allocates nothing. No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc (a device-memory pool or budget
 * that forbids more allocations, real-time loops that cannot take an
 * allocation's implicit synchronisation, plug-ins whose host owns every
 * allocation). The caller passes the matrix (BCSR with bs >= 1, or CSR with
 * bs = 0 and n_block_rows = rows), b and x; every other vector lives in a
 * fixed file-scope device array of about 11.6 MB that each GPU loading the
 * library holds until exit. Limit: n_block_rows * max(bs,1) <= 131072 rows
 * (larger systems get BMFP_ERROR_NOT_SUPPORTED; use bmfp_solver_create).
 * The first call on a device looks up the array's device address; make that
 * first call before any stream capture, and do not call again after a
 * cudaDeviceReset of that device. All calls share the array: calls
 * that overlap on the GPU (other threads or streams) race and must be
 * serialised by the caller. Stops on the recursive residual
 * ||r_i|| / ||b|| < tolerance (the reference's rule, gpu/bicgstab.cu:512);
 * *iterations and *rel_residual (that recursive value) may be NULL. Blocks
 * until the solve ends (it synchronises the stream). More than 2^31 - 1
 * stored values (nnzb * bs^2) get BMFP_ERROR_NOT_SUPPORTED. */
BMFP_API int bmfp_bicgstab_solve_noalloc (int dtype, int n_block_rows, int bs, int64_t nnzb,
                                          const int *d_row_ptr, const int *d_cols,
                                          const void *d_values, const void *d_b, void *d_x,
                                          double tolerance, int max_iterations,
                                          int preconditioner, int *iterations,
                                          double *rel_residual, void *stream);

/* --------------------------------------------------- host-side utilities ---
 * Pure host functions (no GPU needed). */

/* BCSR -> CSR, common/matrix_converters.h:88-117. Output sizes
 * n_block_rows*bs+1, nnzb*bs*bs, nnzb*bs*bs. */
BMFP_API int bmfp_bcsr_to_csr (int dtype, int n_block_rows, int bs, const int *brow_ptr,
                               const int *bcols, const void *bvals, int *row_ptr, int *cols,
                               void *vals);
/* CSR -> BCSR (new; the inverse of bmfp_bcsr_to_csr, bit-exact on its
 * output). Pass 1: bvals == NULL and bcols == NULL fills brow_ptr
 * (n_rows/bs+1) and *nnzb. Pass 2: fills bcols (sorted) and row-major block
 * values, zero where the CSR holds no entry. */
BMFP_API int bmfp_csr_to_bcsr (int dtype, int n_rows, int n_cols, int bs, const int *row_ptr,
                               const int *cols, const void *vals, int *brow_ptr, int64_t *nnzb,
                               int *bcols, void *bvals);
/* Row-major -> column-major blocks, common/matrix_converters.h:32-49.
 * (Applied twice it is the identity.) */
BMFP_API int bmfp_transpose_blocks (int dtype, int n_block_rows, int bs, const int *row_ptr,
                                    const void *vals, void *out);
/* The reference's contiguous-band generator, common/matrix_converters.h:157-196:
 * sizes n_rows+1, n_rows*blocks_per_row, n_rows*blocks_per_row*bs*bs. */
BMFP_API int bmfp_gen_n_diag_bcsr (int dtype, int n_rows, int blocks_per_row, int bs,
                                   int *row_ptr, int *cols, void *vals);
/* Seeded random-band BCSR (new): block row i holds min(k, W) distinct block
 * columns drawn from [max(0,i-h), min(nbr-1,i+h)] (W wide), sorted, values
 * uniform in [-1,1). Per-row SplitMix64 streams: the output depends only on
 * (seed, shape). Pass 1 (cols == NULL, vals == NULL): row_ptr and *nnzb.
 * Pass 2: cols and vals. */
BMFP_API int bmfp_gen_band_bcsr (int dtype, int n_block_rows, int blocks_per_row, int half_band,
                                 int bs, uint64_t seed, int *row_ptr, int64_t *nnzb, int *cols,
                                 void *vals);
/* x_i uniform in [-1,1) from SplitMix64 of (seed, stream, i). */
BMFP_API int bmfp_gen_uniform_vector (int dtype, int64_t n, uint64_t seed, uint64_t stream,
                                      void *out);
/* Q4 plane-stress elasticity (new): nx*ny node grid of unit squares, E, nu,
 * thickness 1; node (i,j) -> block row j*nx+i with DOFs (ux,uy); left column
 * clamped (unit diagonal, zero rows/columns kept in the pattern); BCSR bs=2
 * with the full 9-node stencil. Pass 1 (cols == NULL): row_ptr, *nnzb.
 * Pass 2: cols, vals (float64 or float32) and, if rhs != NULL, the load
 * f_y = -1 on the right column (2*nx*ny entries). */
BMFP_API int bmfp_gen_q4_elasticity (int dtype, int nx, int ny, double young, double poisson,
                                     int *row_ptr, int64_t *nnzb, int *cols, void *vals,
                                     void *rhs);
/* Truss model of the Golden Gate bridge, fem_2d/golden_gate_bridge.h:101-237
 * and :767-878 (golden_gate_bridge_2d<T, int, false>, the instantiation
 * main.cpp:349-381 builds): BCSR bs=2 stiffness with one block row per node
 * (supported DOFs left as zero rows and columns, as the reference leaves
 * them) and the load vector (0, load_fy) on the deck's top chord within
 * load_window of mid-span, else 0 (the load of main.cpp:356-363). main.cpp
 * uses (main_span, side_span, tower_height, segment_length) = (128000, 345,
 * 260, 7.62), window 450, fy -2e6. Pass 1 (row_ptr == NULL): *n_block_rows
 * and *nnzb. Pass 2: row_ptr (n_block_rows+1), cols (nnzb), values
 * (nnzb*4) and, if rhs != NULL, rhs (2*n_block_rows). Writes no files. */
BMFP_API int bmfp_gen_golden_gate_bridge (int dtype, double main_span, double side_span,
                                          double tower_height, double segment_length,
                                          double load_window, double load_fy, int *n_block_rows,
                                          int64_t *nnzb, int *row_ptr, int *cols, void *values,
                                          void *rhs);
/* Geometry of the same truss: *n_segments deck segments (top-chord nodes 4s
 * and 4s+1 of segment s carry the loads, golden_gate_bridge.h:170-178),
 * node coordinates xs/ys (*n_nodes each) and element end nodes starts/ends
 * (*n_elements each, start < end). NULL arrays are skipped, so one call with
 * all arrays NULL returns the sizes. For loads of any shape and for VTK
 * output (golden_gate_bridge.h:239-282) through the C++ drop-in. */
BMFP_API int bmfp_golden_gate_bridge_geometry (int dtype, double main_span, double side_span,
                                               double tower_height, double segment_length,
                                               int *n_segments, int *n_nodes, int *n_elements,
                                               void *xs, void *ys, int *starts, int *ends);
/* MatrixMarket coordinate file -> CSR (new; the reference only writes such
 * files, csr_matrix_class::write_mm, common/matrix_converters.h:119-144, with
 * common/mmio.c). Fields real, double, integer or pattern (1.0); symmetry
 * general, symmetric or skew-symmetric (the other triangle mirrored);
 * entries in any order, duplicates summed in file order; output rows
 * ascending, columns ascending within a row. Values are parsed as double and
 * rounded once to dtype. Pass 1 (row_ptr == NULL): *n_rows, *n_cols, *nnz.
 * Pass 2: row_ptr (n_rows+1), cols and values (nnz). Together with
 * bmfp_csr_to_bcsr this brings any MatrixMarket matrix to the kernels. */
BMFP_API int bmfp_mm_read_csr (const char *path, int dtype, int *n_rows, int *n_cols, int64_t *nnz,
                               int *row_ptr, int *cols, void *values);
/* Algorithmic bytes of one BCSR SpMV: values + block columns + row offsets +
 * x read once + y written once (value and vector size from dtype). */
BMFP_API int64_t bmfp_bcsr_spmv_bytes (int dtype, int n_block_rows, int n_block_cols, int bs,
                                       int64_t nnzb);
BMFP_API int64_t bmfp_csr_spmv_bytes (int dtype, int n_rows, int n_cols, int64_t nnz);

#ifdef __cplusplus
}
#endif

#endif /* BMFP_H */
