// Internal helpers shared by every translation unit of libbmfp.so.
#pragma once

#include "bmfp.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

// A device-resident matrix owned by the library (bmfp_matrix_t).
struct bmfp_matrix_s
{
  int dtype = BMFP_R64F;
  int n_rows = 0;  // block rows for BCSR, rows for CSR
  int n_cols = 0;  // block columns for BCSR, columns for CSR
  int bs = 0;      // 0 = CSR
  int64_t nnz = 0; // blocks for BCSR, entries for CSR
  int *d_row_ptr = nullptr;
  int *d_cols = nullptr;
  void *d_vals = nullptr;
  void *d_vals_cm = nullptr; // column-major copy of the blocks (BMFP_LANES_COL_OWNER only)
  int lanes = 0;             // tuned lane count, 0 = heuristic
};

namespace bmfp
{
// Records a printf-style message as the calling thread's last error and
// returns status unchanged, so call sites read `return fail (...)`.
int fail (int status, const char *fmt, ...) __attribute__ ((format (printf, 2, 3)));
int cuda_fail (cudaError_t e, const char *what, const char *file, int line);

inline bool dtype_ok (int dtype) { return dtype == BMFP_R32F || dtype == BMFP_R64F; }
inline size_t dtype_size (int dtype) { return dtype == BMFP_R64F ? 8 : 4; }

inline cudaStream_t as_stream (void *s) { return static_cast<cudaStream_t> (s); }

// Raw (caller-owned arrays) kernel entry points, implemented per .cu file.
int spmv_native_bcsr (int dtype, int n_block_rows, int bs, int64_t nnzb, const int *row_ptr,
                      const int *cols, const void *vals, const void *x, void *y, int lanes,
                      cudaStream_t stream);
int spmv_native_csr (int dtype, int n_rows, int64_t nnz, const int *row_ptr, const int *cols,
                     const void *vals, const void *x, void *y, int lanes, cudaStream_t stream);
int spmv_reference_variant (int dtype, int variant, int n_rows, int n_cols, int bs, int64_t nnz,
                            const int *row_ptr, const int *cols, const void *vals, const void *x,
                            void *y, cudaStream_t stream);
int spmv_cusparse (int dtype, bool column_major, int n_block_rows, int n_block_cols, int bs,
                   int64_t nnzb, const int *row_ptr, const int *cols, const void *vals,
                   const void *x, void *y, cudaStream_t stream);
int native_default_lanes (int dtype, int bs, double avg_blocks_per_row);
int convert_values (int src_dtype, int dst_dtype, int64_t n, const void *src, void *dst,
                    cudaStream_t stream);
// Valid lane counts for the native BCSR kernel at this block size, ascending.
int native_lane_candidates (int dtype, int bs, int *out, int max_out);
// Column-owner product over column-major blocks (bs in {4,8,16,32}), and the
// row-major -> column-major copy it reads.
int spmv_native_bcsr_colmajor (int dtype, int n_block_rows, int bs, const int *row_ptr, const int *cols,
                               const void *vals_cm, const void *x, void *y, cudaStream_t stream);
int transpose_blocks_device (int dtype, int64_t nnzb, int bs, const void *in, void *out, cudaStream_t stream);
// Evicts L2 by reading `bytes` (> L2) of scratch; sink is a device int.
int l2_flush (const void *scratch, size_t bytes, int *sink, cudaStream_t stream);
} // namespace bmfp

#define BMFP_CUDA(expr)                                                                  \
  do                                                                                     \
    {                                                                                    \
      cudaError_t bmfp_e_ = (expr);                                                      \
      if (bmfp_e_ != cudaSuccess)                                                        \
        return ::bmfp::cuda_fail (bmfp_e_, #expr, __FILE__, __LINE__);                   \
    }                                                                                    \
  while (0)

// After a <<<>>> launch: launch-configuration errors are not sticky and are
// cleared by cudaGetLastError.
#define BMFP_LAUNCH_CHECK() BMFP_CUDA (cudaGetLastError ())
