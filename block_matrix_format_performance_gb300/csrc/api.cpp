// C ABI glue: status handling, SpMV entry points and device matrix handles.
#include "internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

namespace bmfp
{
namespace
{
thread_local std::string g_last_error;
}

int fail (int status, const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start (ap, fmt);
  std::vsnprintf (buf, sizeof buf, fmt, ap);
  va_end (ap);
  g_last_error = buf;
  return status;
}

int cuda_fail (cudaError_t e, const char *what, const char *file, int line)
{
  const int status = e == cudaErrorMemoryAllocation ? BMFP_ERROR_OUT_OF_MEMORY : BMFP_ERROR_CUDA;
  return fail (status, "%s failed: %s (%s:%d)", what, cudaGetErrorString (e), file, line);
}
} // namespace bmfp

using namespace bmfp;

extern "C" {

const char *bmfp_last_error (void) { return g_last_error.c_str (); }

int bmfp_version (void) { return 10000; }

int bmfp_device_count (void)
{
  int n = 0;
  if (cudaGetDeviceCount (&n) != cudaSuccess)
    {
      cudaGetLastError ();
      return 0;
    }
  return n;
}

static const char *const kVariantNames[BMFP_SPMV_VARIANT_COUNT] = {
  "GPU CSR",
  "GPU CSR-Vector",
  "GPU CSR (GB300 sub-warp)",
  "GPU BCSR (row major, thread per row)",
  "GPU BCSR (row major, warp per row)",
  "GPU BCSR (column major, thread per row)",
  "GPU BCSR (column major, thread per row, template)",
  "GPU BCSR (column major, thread per row, coal x)",
  "GPU BCSR (column major, thread per row, coal x, template)",
  "GPU BCSR (column major, column-by-column)",
  "GPU BCSR (column major, column-by-column, int fastdiv)",
  "GPU BCSR (column major, column-by-column, int po2)",
  "GPU BCSR (column major, column-by-column, template)",
  "jit",
  "GPU BSR (cuSPARSE, row major)",
  "GPU BSR (cuSPARSE, column major)",
  "GPU BCSR (GB300 native)",
};

const char *bmfp_spmv_variant_name (int variant)
{
  if (variant < 0 || variant >= BMFP_SPMV_VARIANT_COUNT)
    return nullptr;
  return kVariantNames[variant];
}

int bmfp_spmv_variant_is_csr (int variant)
{
  if (variant < 0 || variant >= BMFP_SPMV_VARIANT_COUNT)
    return -1;
  return variant <= BMFP_SPMV_CSR_NATIVE ? 1 : 0;
}

int bmfp_spmv_variant_layout (int variant)
{
  if (variant < 0 || variant >= BMFP_SPMV_VARIANT_COUNT)
    return -1;
  switch (variant)
    {
    case BMFP_SPMV_CSR_SCALAR:
    case BMFP_SPMV_CSR_VECTOR:
    case BMFP_SPMV_CSR_NATIVE:
    case BMFP_SPMV_BCSR_ROW_THREAD:
    case BMFP_SPMV_BCSR_ROW_WARP:
    case BMFP_SPMV_CUSPARSE_ROW:
    case BMFP_SPMV_BCSR_NATIVE:
      return 0;
    default:
      return 1;
    }
}

int bmfp_csr_spmv (int dtype, int variant, int n_rows, int n_cols, int64_t nnz,
                   const int *d_row_ptr, const int *d_cols, const void *d_values, const void *d_x,
                   void *d_y, void *stream)
{
  if (!dtype_ok (dtype))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid dtype %d", dtype);
  if (bmfp_spmv_variant_is_csr (variant) != 1)
    return fail (BMFP_ERROR_INVALID_VALUE, "variant %d is not a CSR variant", variant);
  if (n_rows < 0 || n_cols < 0 || nnz < 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "negative size");
  if (n_rows == 0)
    return BMFP_SUCCESS;
  if (!d_row_ptr || !d_y || (nnz > 0 && (!d_cols || !d_values || !d_x)))
    return fail (BMFP_ERROR_INVALID_VALUE, "null device pointer");
  if (variant == BMFP_SPMV_CSR_NATIVE)
    return spmv_native_csr (dtype, n_rows, nnz, d_row_ptr, d_cols, d_values, d_x, d_y, 0,
                            as_stream (stream));
  return spmv_reference_variant (dtype, variant, n_rows, n_cols, 1, nnz, d_row_ptr, d_cols,
                                 d_values, d_x, d_y, as_stream (stream));
}

int bmfp_bcsr_spmv (int dtype, int variant, int n_block_rows, int n_block_cols, int bs,
                    int64_t nnzb, const int *d_row_ptr, const int *d_cols, const void *d_values,
                    const void *d_x, void *d_y, void *stream)
{
  if (!dtype_ok (dtype))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid dtype %d", dtype);
  if (bmfp_spmv_variant_is_csr (variant) != 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "variant %d is not a BCSR variant", variant);
  if (n_block_rows < 0 || n_block_cols < 0 || nnzb < 0 || bs < 1)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid shape (rows %d, cols %d, bs %d, nnzb %lld)",
                 n_block_rows, n_block_cols, bs, (long long) nnzb);
  if (n_block_rows == 0)
    return BMFP_SUCCESS;
  if (!d_row_ptr || !d_y || (nnzb > 0 && (!d_cols || !d_values || !d_x)))
    return fail (BMFP_ERROR_INVALID_VALUE, "null device pointer");
  if (nnzb * (int64_t) bs * bs > INT32_MAX)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "more than 2^31-1 values");
  cudaStream_t s = as_stream (stream);
  switch (variant)
    {
    case BMFP_SPMV_BCSR_NATIVE:
      return spmv_native_bcsr (dtype, n_block_rows, bs, nnzb, d_row_ptr, d_cols, d_values, d_x,
                               d_y, 0, s);
    case BMFP_SPMV_CUSPARSE_ROW:
    case BMFP_SPMV_CUSPARSE_COL:
      return spmv_cusparse (dtype, variant == BMFP_SPMV_CUSPARSE_COL, n_block_rows, n_block_cols,
                            bs, nnzb, d_row_ptr, d_cols, d_values, d_x, d_y, s);
    default:
      return spmv_reference_variant (dtype, variant, n_block_rows, n_block_cols, bs, nnzb,
                                     d_row_ptr, d_cols, d_values, d_x, d_y, s);
    }
}

int bmfp_bcsr_spmv_native_ex (int dtype, int n_block_rows, int bs, int64_t nnzb,
                              const int *d_row_ptr, const int *d_cols, const void *d_values,
                              const void *d_x, void *d_y, int lanes, void *stream)
{
  if (!dtype_ok (dtype))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid dtype %d", dtype);
  if (n_block_rows < 0 || nnzb < 0 || bs < 1 || lanes < 0 || (lanes > 32 && lanes != BMFP_LANES_ROW_OWNER))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if (n_block_rows == 0)
    return BMFP_SUCCESS;
  if (!d_row_ptr || !d_y || (nnzb > 0 && (!d_cols || !d_values || !d_x)))
    return fail (BMFP_ERROR_INVALID_VALUE, "null device pointer");
  return spmv_native_bcsr (dtype, n_block_rows, bs, nnzb, d_row_ptr, d_cols, d_values, d_x, d_y,
                           lanes, as_stream (stream));
}

int bmfp_bcsr_spmv_colmajor (int dtype, int nbr, int bs, int64_t nnzb, const int *d_row_ptr, const int *d_cols,
                              const void *d_vals_cm, const void *d_x, void *d_y, void *stream)
{
  if (!dtype_ok (dtype) || nbr < 0 || nnzb < 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if (nbr > 0 && (!d_row_ptr || !d_x || !d_y || (nnzb > 0 && (!d_cols || !d_vals_cm))))
    return fail (BMFP_ERROR_INVALID_VALUE, "null device array");
  return spmv_native_bcsr_colmajor (dtype, nbr, bs, d_row_ptr, d_cols, d_vals_cm, d_x, d_y, as_stream (stream));
}

int bmfp_bcsr_native_default_lanes (int dtype, int bs, double avg_blocks_per_row)
{
  if (!dtype_ok (dtype) || bs < 1)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments"), 0;
  return native_default_lanes (dtype, bs, avg_blocks_per_row);
}

int64_t bmfp_bcsr_spmv_bytes (int dtype, int n_block_rows, int n_block_cols, int bs, int64_t nnzb)
{
  const int64_t S = (int64_t) dtype_size (dtype);
  return nnzb * bs * bs * S + nnzb * 4 + ((int64_t) n_block_rows + 1) * 4
         + (int64_t) n_block_cols * bs * S + (int64_t) n_block_rows * bs * S;
}

int64_t bmfp_csr_spmv_bytes (int dtype, int n_rows, int n_cols, int64_t nnz)
{
  const int64_t S = (int64_t) dtype_size (dtype);
  return nnz * S + nnz * 4 + ((int64_t) n_rows + 1) * 4 + (int64_t) n_cols * S
         + (int64_t) n_rows * S;
}

// ------------------------------------------------------------ matrices

static int matrix_alloc (bmfp_matrix_s *m)
{
  const size_t S = dtype_size (m->dtype);
  const int64_t rows = m->n_rows;
  const int64_t nvals = m->bs ? m->nnz * m->bs * m->bs : m->nnz;
  BMFP_CUDA (cudaMalloc (&m->d_row_ptr, sizeof (int) * (size_t) (rows + 1)));
  BMFP_CUDA (cudaMalloc (&m->d_cols, sizeof (int) * (size_t) std::max<int64_t> (m->nnz, 1)));
  BMFP_CUDA (cudaMalloc (&m->d_vals, S * (size_t) std::max<int64_t> (nvals, 1)));
  return BMFP_SUCCESS;
}

static void matrix_free (bmfp_matrix_s *m)
{
  if (!m)
    return;
  cudaFree (m->d_row_ptr);
  cudaFree (m->d_cols);
  cudaFree (m->d_vals);
  cudaFree (m->d_vals_cm);
  delete m;
}

static int matrix_create (bmfp_matrix_t *out, int dtype, int n_rows, int n_cols, int bs,
                          int64_t nnz, const int *row_ptr, const int *cols, const void *vals,
                          cudaMemcpyKind kind, void *stream)
{
  if (!out)
    return fail (BMFP_ERROR_INVALID_VALUE, "null output handle");
  *out = nullptr;
  if (!dtype_ok (dtype))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid dtype %d", dtype);
  if (n_rows < 0 || n_cols < 0 || nnz < 0 || bs < 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "negative size");
  if (!row_ptr || (nnz > 0 && (!cols || !vals)))
    return fail (BMFP_ERROR_INVALID_VALUE, "null input array");
  const int64_t nvals = bs ? nnz * bs * bs : nnz;
  if (nvals > INT32_MAX)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "more than 2^31-1 values");
  bmfp_matrix_s *m = new (std::nothrow) bmfp_matrix_s;
  if (!m)
    return fail (BMFP_ERROR_OUT_OF_MEMORY, "host allocation failed");
  m->dtype = dtype;
  m->n_rows = n_rows;
  m->n_cols = n_cols;
  m->bs = bs;
  m->nnz = nnz;
  int st = matrix_alloc (m);
  if (st != BMFP_SUCCESS)
    {
      matrix_free (m);
      return st;
    }
  cudaStream_t s = as_stream (stream);
  const size_t S = dtype_size (dtype);
  cudaError_t e = cudaMemcpyAsync (m->d_row_ptr, row_ptr, sizeof (int) * ((size_t) n_rows + 1), kind, s);
  if (e == cudaSuccess && nnz > 0)
    e = cudaMemcpyAsync (m->d_cols, cols, sizeof (int) * (size_t) nnz, kind, s);
  if (e == cudaSuccess && nnz > 0)
    e = cudaMemcpyAsync (m->d_vals, vals, S * (size_t) nvals, kind, s);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize (s);
  if (e != cudaSuccess)
    {
      matrix_free (m);
      return cuda_fail (e, "matrix upload", __FILE__, __LINE__);
    }
  *out = m;
  return BMFP_SUCCESS;
}

int bmfp_matrix_create_bcsr (bmfp_matrix_t *out, int dtype, int n_block_rows, int n_block_cols,
                             int bs, int64_t nnzb, const int *h_row_ptr, const int *h_cols,
                             const void *h_values, void *stream)
{
  if (bs < 1)
    return fail (BMFP_ERROR_INVALID_VALUE, "bs must be >= 1");
  return matrix_create (out, dtype, n_block_rows, n_block_cols, bs, nnzb, h_row_ptr, h_cols,
                        h_values, cudaMemcpyHostToDevice, stream);
}

int bmfp_matrix_create_csr (bmfp_matrix_t *out, int dtype, int n_rows, int n_cols, int64_t nnz,
                            const int *h_row_ptr, const int *h_cols, const void *h_values,
                            void *stream)
{
  return matrix_create (out, dtype, n_rows, n_cols, 0, nnz, h_row_ptr, h_cols, h_values,
                        cudaMemcpyHostToDevice, stream);
}

int bmfp_matrix_create_bcsr_device (bmfp_matrix_t *out, int dtype, int n_block_rows,
                                    int n_block_cols, int bs, int64_t nnzb, const int *d_row_ptr,
                                    const int *d_cols, const void *d_values, void *stream)
{
  if (bs < 1)
    return fail (BMFP_ERROR_INVALID_VALUE, "bs must be >= 1");
  return matrix_create (out, dtype, n_block_rows, n_block_cols, bs, nnzb, d_row_ptr, d_cols,
                        d_values, cudaMemcpyDeviceToDevice, stream);
}

int bmfp_matrix_convert (bmfp_matrix_t *out, bmfp_matrix_t src, int dtype, void *stream)
{
  if (!out || !src)
    return fail (BMFP_ERROR_INVALID_VALUE, "null handle");
  *out = nullptr;
  if (!dtype_ok (dtype))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid dtype %d", dtype);
  bmfp_matrix_s *m = new (std::nothrow) bmfp_matrix_s (*src);
  if (!m)
    return fail (BMFP_ERROR_OUT_OF_MEMORY, "host allocation failed");
  m->dtype = dtype;
  m->d_row_ptr = nullptr;
  m->d_cols = nullptr;
  m->d_vals = nullptr;
  int st = matrix_alloc (m);
  if (st != BMFP_SUCCESS)
    {
      matrix_free (m);
      return st;
    }
  cudaStream_t s = as_stream (stream);
  const int64_t nvals = m->bs ? m->nnz * m->bs * m->bs : m->nnz;
  cudaError_t e = cudaMemcpyAsync (m->d_row_ptr, src->d_row_ptr,
                                   sizeof (int) * ((size_t) m->n_rows + 1),
                                   cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && m->nnz > 0)
    e = cudaMemcpyAsync (m->d_cols, src->d_cols, sizeof (int) * (size_t) m->nnz,
                         cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess)
    {
      matrix_free (m);
      return cuda_fail (e, "matrix convert copy", __FILE__, __LINE__);
    }
  st = convert_values (src->dtype, dtype, nvals, src->d_vals, m->d_vals, s);
  if (st == BMFP_SUCCESS)
    {
      e = cudaStreamSynchronize (s);
      if (e != cudaSuccess)
        st = cuda_fail (e, "matrix convert", __FILE__, __LINE__);
    }
  if (st != BMFP_SUCCESS)
    {
      matrix_free (m);
      return st;
    }
  m->lanes = 0;
  *out = m;
  return BMFP_SUCCESS;
}

int bmfp_matrix_destroy (bmfp_matrix_t m)
{
  matrix_free (m);
  return BMFP_SUCCESS;
}

int bmfp_matrix_info (bmfp_matrix_t m, int *dtype, int *n_rows, int *n_cols, int *bs,
                      int64_t *nnz_blocks, int64_t *bytes_per_spmv)
{
  if (!m)
    return fail (BMFP_ERROR_INVALID_VALUE, "null handle");
  if (dtype)
    *dtype = m->dtype;
  if (n_rows)
    *n_rows = m->n_rows;
  if (n_cols)
    *n_cols = m->n_cols;
  if (bs)
    *bs = m->bs;
  if (nnz_blocks)
    *nnz_blocks = m->nnz;
  if (bytes_per_spmv)
    *bytes_per_spmv = m->bs ? bmfp_bcsr_spmv_bytes (m->dtype, m->n_rows, m->n_cols, m->bs, m->nnz)
                            : bmfp_csr_spmv_bytes (m->dtype, m->n_rows, m->n_cols, m->nnz);
  return BMFP_SUCCESS;
}

int bmfp_matrix_device_arrays (bmfp_matrix_t m, const int **d_row_ptr, const int **d_cols,
                               const void **d_values)
{
  if (!m)
    return fail (BMFP_ERROR_INVALID_VALUE, "null handle");
  if (d_row_ptr)
    *d_row_ptr = m->d_row_ptr;
  if (d_cols)
    *d_cols = m->d_cols;
  if (d_values)
    *d_values = m->d_vals;
  return BMFP_SUCCESS;
}

static bool col_owner_bs (int bs) { return bs == 2 || bs == 4 || bs == 8 || bs == 16 || bs == 32; }

// Builds (or, for any other mapping, releases) the column-major copy the
// column-owner kernel reads.
static int matrix_apply_lanes (bmfp_matrix_s *m, int lanes, cudaStream_t s)
{
  if (lanes == BMFP_LANES_COL_OWNER)
    {
      if (m->bs == 0 || !col_owner_bs (m->bs))
        return fail (BMFP_ERROR_INVALID_VALUE, "column-owner mapping needs a BCSR handle with bs in {2,4,8,16,32}");
      if (!m->d_vals_cm)
        {
          const size_t bytes = dtype_size (m->dtype) * (size_t) std::max<int64_t> (m->nnz * m->bs * m->bs, 1);
          void *p = nullptr;
          const cudaError_t e = cudaMalloc (&p, bytes);
          if (e != cudaSuccess)
            {
              cudaGetLastError ();
              return fail (BMFP_ERROR_OUT_OF_MEMORY, "no room for the column-major copy (%zu bytes)", bytes);
            }
          const int st = transpose_blocks_device (m->dtype, m->nnz, m->bs, m->d_vals, p, s);
          if (st != BMFP_SUCCESS)
            {
              cudaFree (p);
              return st;
            }
          m->d_vals_cm = p;
        }
    }
  else if (m->d_vals_cm)
    {
      BMFP_CUDA (cudaStreamSynchronize (s)); // no product may still read it
      cudaFree (m->d_vals_cm);
      m->d_vals_cm = nullptr;
    }
  m->lanes = lanes;
  return BMFP_SUCCESS;
}

int bmfp_matrix_set_lanes (bmfp_matrix_t m, int lanes, void *stream)
{
  if (!m)
    return fail (BMFP_ERROR_INVALID_VALUE, "null matrix");
  if (lanes < 0 || (lanes > 32 && lanes != BMFP_LANES_ROW_OWNER && lanes != BMFP_LANES_COL_OWNER))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid lane count %d", lanes);
  if (lanes != 0 && lanes != BMFP_LANES_COL_OWNER)
    {
      // only mappings this matrix's products can run (the autotuner's list)
      int cand[12];
      const int nc = native_lane_candidates (m->dtype, m->bs ? m->bs : 1, cand, 10);
      if (std::find (cand, cand + nc, lanes) == cand + nc)
        return fail (BMFP_ERROR_INVALID_VALUE, "lane count %d not valid for bs=%d", lanes, m->bs);
    }
  return matrix_apply_lanes (m, lanes, as_stream (stream));
}

int bmfp_matrix_spmv (bmfp_matrix_t m, const void *d_x, void *d_y, void *stream)
{
  if (!m || !d_x || !d_y)
    return fail (BMFP_ERROR_INVALID_VALUE, "null argument");
  if (m->lanes == BMFP_LANES_COL_OWNER && m->d_vals_cm)
    return spmv_native_bcsr_colmajor (m->dtype, m->n_rows, m->bs, m->d_row_ptr, m->d_cols, m->d_vals_cm, d_x,
                                      d_y, as_stream (stream));
  if (m->bs == 0)
    return spmv_native_csr (m->dtype, m->n_rows, m->nnz, m->d_row_ptr, m->d_cols, m->d_vals, d_x,
                            d_y, m->lanes, as_stream (stream));
  return spmv_native_bcsr (m->dtype, m->n_rows, m->bs, m->nnz, m->d_row_ptr, m->d_cols, m->d_vals, d_x, d_y,
                           m->lanes == BMFP_LANES_COL_OWNER ? 0 : m->lanes, as_stream (stream));
}

int bmfp_matrix_autotune (bmfp_matrix_t m, const void *d_x, void *d_y, void *stream,
                          int *chosen_lanes)
{
  if (!m || !d_x || !d_y)
    return fail (BMFP_ERROR_INVALID_VALUE, "null argument");
  int cand[12];
  const int bs_eff = m->bs ? m->bs : 1;
  int nc = native_lane_candidates (m->dtype, bs_eff, cand, 10);
  if (m->bs && col_owner_bs (m->bs))
    cand[nc++] = BMFP_LANES_COL_OWNER;
  if (nc == 0)
    {
      if (chosen_lanes)
        *chosen_lanes = 0;
      return BMFP_SUCCESS;
    }
  cudaStream_t s = as_stream (stream);
  // Each timed product starts with L2 emptied (a read of twice its size),
  // as in repeated products over matrices that do not stay in L2: products
  // back to back would favour whatever mapping the leftovers suit.
  int dev = 0, l2 = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  BMFP_CUDA (cudaDeviceGetAttribute (&l2, cudaDevAttrL2CacheSize, dev));
  const size_t flush_bytes = 2 * (size_t) std::max (l2, 1 << 20) + 64;
  char *scratch = nullptr;
  if (cudaMalloc (&scratch, flush_bytes) != cudaSuccess)
    {
      cudaGetLastError ();
      scratch = nullptr; // time without flushing rather than fail
    }
  else
    BMFP_CUDA (cudaMemsetAsync (scratch, 0, flush_bytes, s));
  int *sink = scratch ? (int *) (scratch + flush_bytes - 64) : nullptr;
  const size_t read_bytes = flush_bytes - 64;
  cudaEvent_t a, b;
  BMFP_CUDA (cudaEventCreate (&a));
  BMFP_CUDA (cudaEventCreate (&b));
  float best = 1e30f;
  int best_g = 0;
  int st = BMFP_SUCCESS;
  for (int i = 0; i < nc && st == BMFP_SUCCESS; i++)
    {
      if (cand[i] == BMFP_LANES_COL_OWNER)
        {
          if (matrix_apply_lanes (m, cand[i], s) != BMFP_SUCCESS)
            continue; // no room for the copy: not a candidate here
        }
      else
        m->lanes = cand[i];
      for (int w = 0; w < 3 && st == BMFP_SUCCESS; w++)
        st = bmfp_matrix_spmv (m, d_x, d_y, stream);
      if (st != BMFP_SUCCESS)
        break;
      const int reps = 5;
      float ms = 0;
      for (int r = 0; r < reps && st == BMFP_SUCCESS; r++)
        {
          if (scratch)
            st = l2_flush (scratch, read_bytes, sink, s);
          cudaEventRecord (a, s);
          if (st == BMFP_SUCCESS)
            st = bmfp_matrix_spmv (m, d_x, d_y, stream);
          cudaEventRecord (b, s);
          cudaError_t e = cudaEventSynchronize (b);
          if (e != cudaSuccess)
            {
              st = cuda_fail (e, "autotune timing", __FILE__, __LINE__);
              break;
            }
          float one = 0;
          cudaEventElapsedTime (&one, a, b);
          ms += one;
        }
      if (st != BMFP_SUCCESS)
        break;
      if (ms < best)
        {
          best = ms;
          best_g = cand[i];
        }
    }
  cudaEventDestroy (a);
  cudaEventDestroy (b);
  if (scratch)
    {
      cudaStreamSynchronize (s);
      cudaFree (scratch);
    }
  const int keep = matrix_apply_lanes (m, st == BMFP_SUCCESS ? best_g : 0, s); // frees an unused copy
  if (st == BMFP_SUCCESS)
    st = keep;
  if (chosen_lanes)
    *chosen_lanes = m->lanes;
  return st;
}

} // extern "C"
