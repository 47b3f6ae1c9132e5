/*
 * CPU oracle for the block-sparse hot path — TEST INFRASTRUCTURE ONLY.
 * See oracle.h for the pinning story. Compiled with -ffp-contract=off so that
 * x86 and Arm hosts produce identical bits (no fused multiply-add contraction),
 * matching the reference's own x86 host build, which has no FMA either.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- SpMV --- */

/* main.cpp:36-45: for each row, dot += data[e] * x[col_ids[e]] in order. */
#define ORC_CSR_SPMV(T, NAME)                                                  \
  void NAME (int n_rows, const int *row_ptr, const int *cols, const T *vals,   \
             const T *x, T *y)                                                 \
  {                                                                            \
    for (int row = 0; row < n_rows; row++)                                     \
      {                                                                        \
        T dot = 0;                                                             \
        for (int e = row_ptr[row]; e < row_ptr[row + 1]; e++)                  \
          dot += vals[e] * x[cols[e]];                                         \
        y[row] = dot;                                                          \
      }                                                                        \
  }
ORC_CSR_SPMV (double, orc_csr_spmv_f64)
ORC_CSR_SPMV (float, orc_csr_spmv_f32)

typedef struct
{
  int row_begin, row_end;
  const int *row_ptr, *cols;
  const void *vals, *x;
  void *y;
  int is_f64;
} orc_spmv_task;

static void *orc_spmv_worker (void *arg)
{
  const orc_spmv_task *t = (const orc_spmv_task *) arg;
  const int *rp = t->row_ptr + t->row_begin;
  int n = t->row_end - t->row_begin;
  if (t->is_f64)
    {
      /* Shift row_ptr so the shared loop body indexes rows [begin,end). */
      const double *v = (const double *) t->vals;
      const double *x = (const double *) t->x;
      double *y = (double *) t->y + t->row_begin;
      for (int row = 0; row < n; row++)
        {
          double dot = 0;
          for (int e = rp[row]; e < rp[row + 1]; e++)
            dot += v[e] * x[t->cols[e]];
          y[row] = dot;
        }
    }
  else
    {
      const float *v = (const float *) t->vals;
      const float *x = (const float *) t->x;
      float *y = (float *) t->y + t->row_begin;
      for (int row = 0; row < n; row++)
        {
          float dot = 0;
          for (int e = rp[row]; e < rp[row + 1]; e++)
            dot += v[e] * x[t->cols[e]];
          y[row] = dot;
        }
    }
  return NULL;
}

static void orc_spmv_mt (int n_rows, const int *row_ptr, const int *cols, const void *vals,
                         const void *x, void *y, int n_threads, int is_f64)
{
  if (n_threads < 1)
    n_threads = 1;
  if (n_threads > 256)
    n_threads = 256;
  pthread_t th[256];
  orc_spmv_task tasks[256];
  int started[256];
  for (int i = 0; i < n_threads; i++)
    {
      tasks[i].row_begin = (int) ((int64_t) n_rows * i / n_threads);
      tasks[i].row_end = (int) ((int64_t) n_rows * (i + 1) / n_threads);
      tasks[i].row_ptr = row_ptr;
      tasks[i].cols = cols;
      tasks[i].vals = vals;
      tasks[i].x = x;
      tasks[i].y = y;
      tasks[i].is_f64 = is_f64;
      started[i] = 0;
      if (i > 0 && pthread_create (&th[i], NULL, orc_spmv_worker, &tasks[i]) == 0)
        started[i] = 1;
    }
  orc_spmv_worker (&tasks[0]);
  for (int i = 1; i < n_threads; i++)
    {
      if (started[i])
        pthread_join (th[i], NULL);
      else
        orc_spmv_worker (&tasks[i]);
    }
}

void orc_csr_spmv_mt_f64 (int n_rows, const int *row_ptr, const int *cols,
                          const double *vals, const double *x, double *y, int n_threads)
{
  orc_spmv_mt (n_rows, row_ptr, cols, vals, x, y, n_threads, 1);
}

void orc_csr_spmv_mt_f32 (int n_rows, const int *row_ptr, const int *cols,
                          const float *vals, const float *x, float *y, int n_threads)
{
  orc_spmv_mt (n_rows, row_ptr, cols, vals, x, y, n_threads, 0);
}

/* Scalar row r of block row i visits blocks in order and, inside each block,
 * columns 0..bs-1 — the same order as the CSR row produced by
 * matrix_converters.h:97-113, hence the same bits. */
#define ORC_BCSR_SPMV(T, NAME)                                                 \
  void NAME (int n_block_rows, int bs, const int *row_ptr, const int *cols,    \
             const T *vals, const T *x, T *y)                                  \
  {                                                                            \
    for (int br = 0; br < n_block_rows; br++)                                  \
      for (int r = 0; r < bs; r++)                                             \
        {                                                                      \
          T dot = 0;                                                           \
          for (int b = row_ptr[br]; b < row_ptr[br + 1]; b++)                  \
            {                                                                  \
              const T *blk = vals + (int64_t) b * bs * bs + (int64_t) r * bs;  \
              const T *xb = x + (int64_t) cols[b] * bs;                        \
              for (int c = 0; c < bs; c++)                                     \
                dot += blk[c] * xb[c];                                         \
            }                                                                  \
          y[(int64_t) br * bs + r] = dot;                                      \
        }                                                                      \
  }
ORC_BCSR_SPMV (double, orc_bcsr_spmv_f64)
ORC_BCSR_SPMV (float, orc_bcsr_spmv_f32)

/* --------------------------------------------------------- conversions --- */

/* common/matrix_converters.h:88-117 */
#define ORC_BCSR_TO_CSR(T, NAME)                                               \
  void NAME (int n_block_rows, int bs, const int *brow_ptr, const int *bcols,  \
             const T *bvals, int *row_ptr, int *cols, T *vals)                 \
  {                                                                            \
    int64_t offset = 0;                                                        \
    for (int br = 0; br < n_block_rows; br++)                                  \
      for (int r = 0; r < bs; r++)                                             \
        {                                                                      \
          row_ptr[(int64_t) br * bs + r] = (int) offset;                       \
          for (int b = brow_ptr[br]; b < brow_ptr[br + 1]; b++)                \
            for (int c = 0; c < bs; c++)                                       \
              {                                                                \
                cols[offset] = bcols[b] * bs + c;                              \
                vals[offset] = bvals[(int64_t) b * bs * bs + r * bs + c];      \
                offset++;                                                      \
              }                                                                \
        }                                                                      \
    row_ptr[(int64_t) n_block_rows * bs] = (int) offset;                       \
  }
ORC_BCSR_TO_CSR (double, orc_bcsr_to_csr_f64)
ORC_BCSR_TO_CSR (float, orc_bcsr_to_csr_f32)

static int orc_cmp_int (const void *a, const void *b)
{
  int x = *(const int *) a, y = *(const int *) b;
  return (x > y) - (x < y);
}

/* Collect the distinct block columns touched by the bs scalar rows of block
 * row br into buf (sorted); returns how many. */
static int orc_block_cols (int br, int bs, const int *row_ptr, const int *cols, int *buf)
{
  int n = 0;
  for (int r = 0; r < bs; r++)
    {
      int row = br * bs + r;
      for (int e = row_ptr[row]; e < row_ptr[row + 1]; e++)
        buf[n++] = cols[e] / bs;
    }
  qsort (buf, (size_t) n, sizeof (int), orc_cmp_int);
  int m = 0;
  for (int i = 0; i < n; i++)
    if (m == 0 || buf[m - 1] != buf[i])
      buf[m++] = buf[i];
  return m;
}

int64_t orc_csr_to_bcsr_count (int n_rows, int n_cols, int bs, const int *row_ptr,
                               const int *cols, int *brow_ptr)
{
  if (bs <= 0 || n_rows % bs != 0 || n_cols % bs != 0)
    return -1;
  int nbr = n_rows / bs;
  int max_row = 0;
  for (int br = 0; br < nbr; br++)
    {
      int len = row_ptr[(br + 1) * bs] - row_ptr[br * bs];
      if (len > max_row)
        max_row = len;
    }
  for (int64_t e = 0; e < row_ptr[n_rows]; e++)
    if (cols[e] < 0 || cols[e] >= n_cols)
      return -1;
  int *buf = (int *) malloc (sizeof (int) * (size_t) (max_row + 1));
  int64_t nnzb = 0;
  brow_ptr[0] = 0;
  for (int br = 0; br < nbr; br++)
    {
      nnzb += orc_block_cols (br, bs, row_ptr, cols, buf);
      brow_ptr[br + 1] = (int) nnzb;
    }
  free (buf);
  return nnzb;
}

#define ORC_CSR_TO_BCSR_FILL(T, NAME)                                          \
  int NAME (int n_rows, int bs, const int *row_ptr, const int *cols,           \
            const T *vals, const int *brow_ptr, int *bcols, T *bvals)          \
  {                                                                            \
    int nbr = n_rows / bs;                                                     \
    int max_row = 0;                                                           \
    for (int br = 0; br < nbr; br++)                                           \
      {                                                                        \
        int len = row_ptr[(br + 1) * bs] - row_ptr[br * bs];                   \
        if (len > max_row)                                                     \
          max_row = len;                                                       \
      }                                                                        \
    int *buf = (int *) malloc (sizeof (int) * (size_t) (max_row + 1));         \
    memset (bvals, 0, sizeof (T) * (size_t) brow_ptr[nbr] * bs * bs);          \
    for (int br = 0; br < nbr; br++)                                           \
      {                                                                        \
        int m = orc_block_cols (br, bs, row_ptr, cols, buf);                   \
        if (m != brow_ptr[br + 1] - brow_ptr[br])                              \
          {                                                                    \
            free (buf);                                                        \
            return -1;                                                         \
          }                                                                    \
        memcpy (bcols + brow_ptr[br], buf, sizeof (int) * (size_t) m);         \
        for (int r = 0; r < bs; r++)                                           \
          {                                                                    \
            int row = br * bs + r;                                             \
            for (int e = row_ptr[row]; e < row_ptr[row + 1]; e++)              \
              {                                                                \
                int bc = cols[e] / bs, c = cols[e] % bs;                       \
                /* binary search of bc among this block row's columns */       \
                int lo = 0, hi = m;                                            \
                while (lo < hi)                                                \
                  {                                                            \
                    int mid = (lo + hi) / 2;                                   \
                    if (buf[mid] < bc)                                         \
                      lo = mid + 1;                                            \
                    else                                                       \
                      hi = mid;                                                \
                  }                                                            \
                int64_t b = brow_ptr[br] + lo;                                 \
                bvals[b * bs * bs + r * bs + c] = vals[e];                     \
              }                                                                \
          }                                                                    \
      }                                                                        \
    free (buf);                                                                \
    return 0;                                                                  \
  }
ORC_CSR_TO_BCSR_FILL (double, orc_csr_to_bcsr_fill_f64)
ORC_CSR_TO_BCSR_FILL (float, orc_csr_to_bcsr_fill_f32)

/* common/matrix_converters.h:32-49: new[j*bs+i] = old[i*bs+j] per block. */
#define ORC_TRANSPOSE(T, NAME)                                                 \
  void NAME (int n_block_rows, int bs, const int *row_ptr, const T *vals,      \
             T *out)                                                           \
  {                                                                            \
    for (int br = 0; br < n_block_rows; br++)                                  \
      for (int b = row_ptr[br]; b < row_ptr[br + 1]; b++)                      \
        {                                                                      \
          const T *o = vals + (int64_t) b * bs * bs;                           \
          T *n = out + (int64_t) b * bs * bs;                                  \
          for (int i = 0; i < bs; i++)                                         \
            for (int j = 0; j < bs; j++)                                       \
              n[j * bs + i] = o[i * bs + j];                                   \
        }                                                                      \
  }
ORC_TRANSPOSE (double, orc_transpose_blocks_f64)
ORC_TRANSPOSE (float, orc_transpose_blocks_f32)

/* ----------------------------------------------------------- generator --- */

/* common/matrix_converters.h:157-196. The value expression is
 * (data_type(column) + i) / n_rows with i unsigned: in C++ the unsigned is
 * converted to data_type before the add, and n_rows before the divide. */
#define ORC_GEN_N_DIAG(T, NAME)                                                \
  void NAME (int n_rows, int blocks_per_row, int bs, int *row_ptr, int *cols,  \
             T *vals)                                                          \
  {                                                                            \
    int64_t block_id = 0;                                                      \
    for (int row = 0; row < n_rows; row++)                                     \
      {                                                                        \
        row_ptr[row] = row * blocks_per_row;                                   \
        int first_column;                                                      \
        if (row < blocks_per_row / 2)                                          \
          first_column = 0;                                                    \
        else if (row > n_rows - blocks_per_row)                                \
          first_column = n_rows - blocks_per_row;                              \
        else                                                                   \
          first_column = row - blocks_per_row / 2;                             \
        for (int el = 0; el < blocks_per_row; el++)                            \
          {                                                                    \
            int col = first_column + el;                                       \
            T *blk = vals + block_id * bs * bs;                                \
            for (unsigned i = 0; i < (unsigned) (bs * bs); i++)                \
              blk[i] = ((T) col + (T) i) / (T) n_rows;                         \
            cols[block_id++] = col;                                            \
          }                                                                    \
      }                                                                        \
    row_ptr[n_rows] = n_rows * blocks_per_row;                                 \
  }
ORC_GEN_N_DIAG (double, orc_gen_n_diag_bcsr_f64)
ORC_GEN_N_DIAG (float, orc_gen_n_diag_bcsr_f32)

/* ------------------------------------------------------------- compare --- */

/* common/measurement_class.h:58-87 (accumulation in the element type). */
#define ORC_COMPARE(T, NAME)                                                   \
  double NAME (unsigned n, const T *a, const T *b, int *flagged)              \
  {                                                                            \
    T num = 0.0, den = 0.0;                                                    \
    for (unsigned i = 0; i < n; i++)                                           \
      {                                                                        \
        num += (a[i] - b[i]) * (a[i] - b[i]);                                  \
        den += b[i] * b[i];                                                    \
      }                                                                        \
    const T error = num / den;                                                 \
    if (flagged)                                                               \
      *flagged = error > 1e-9 ? 1 : 0;                                         \
    return (double) error;                                                     \
  }
ORC_COMPARE (double, orc_compare_results_f64)
ORC_COMPARE (float, orc_compare_results_f32)

/* ------------------------------------------------------------ BiCGStab --- */

static double orc_dot (int n, const double *a, const double *b)
{
  double s = 0.0;
  for (int i = 0; i < n; i++)
    s += a[i] * b[i];
  return s;
}

int orc_bicgstab_f64 (int n, const int *row_ptr, const int *cols, const double *vals,
                      const double *b, double *x, double eps, int max_iterations,
                      int use_precond, int *iters, double *rel_res)
{
  double *mem = (double *) calloc ((size_t) n * 10, sizeof (double));
  double *r = mem, *rh = mem + n, *p = mem + 2 * n, *v = mem + 3 * n, *h = mem + 4 * n;
  double *s = mem + 5 * n, *t = mem + 6 * n, *P = mem + 7 * n, *q = mem + 8 * n, *z = mem + 9 * n;
  int status = 1;
  *iters = 0;

  /* bicgstab.cu:408-412 */
  const double norm_b = sqrt (orc_dot (n, b, b));
  /* bicgstab.cu:201-225: P[row] = 1/a_rr (1 when |a_rr| < 1e-20); a row
   * without a stored diagonal keeps 1 here (the reference leaves it unset). */
  for (int row = 0; row < n; row++)
    {
      P[row] = 1.0;
      if (use_precond)
        for (int e = row_ptr[row]; e < row_ptr[row + 1]; e++)
          if (cols[e] == row)
            {
              P[row] = fabs (vals[e]) < 1e-20 ? 1.0 : 1.0 / vals[e];
              break;
            }
    }
  /* bicgstab.cu:257-284: x0 = 0, r0 = rh = b */
  for (int i = 0; i < n; i++)
    {
      x[i] = 0.0;
      r[i] = rh[i] = b[i];
    }
  *rel_res = norm_b > 0 ? 1.0 : 0.0;
  if (norm_b == 0.0)
    {
      free (mem);
      return 0;
    }

  double rho_prev = 1.0, omega_prev = 1.0, alpha = 1.0; /* bicgstab.cu:414-420 */
  for (int it = 0; it < max_iterations; it++)
    {
      const double rho = orc_dot (n, rh, r);                 /* :447 */
      if (rho == 0.0)
        {
          status = 2;
          break;
        }
      const double beta = rho / rho_prev * alpha / omega_prev; /* :451 */
      for (int i = 0; i < n; i++)                             /* :452, :286-304 */
        p[i] = r[i] + beta * (p[i] - omega_prev * v[i]);
      for (int i = 0; i < n; i++)                             /* :454-457 */
        q[i] = use_precond ? P[i] * p[i] : p[i];
      orc_csr_spmv_f64 (n, row_ptr, cols, vals, q, v);        /* :460 */
      const double rh_v = orc_dot (n, rh, v);                 /* :463-466 */
      if (rh_v == 0.0)
        {
          status = 2;
          break;
        }
      alpha = rho / rh_v;
      for (int i = 0; i < n; i++)                             /* :470, :306-327 */
        {
          h[i] = x[i] + alpha * q[i];
          s[i] = r[i] - alpha * v[i];
        }
      for (int i = 0; i < n; i++)                             /* :472-475 */
        z[i] = use_precond ? P[i] * s[i] : s[i];
      orc_csr_spmv_f64 (n, row_ptr, cols, vals, z, t);        /* :478 */
      const double ts = orc_dot (n, t, s), tt = orc_dot (n, t, t); /* :483-486 */
      if (tt == 0.0)
        {
          /* t = 0 means s = 0 up to the operator: accept h as the iterate. */
          for (int i = 0; i < n; i++)
            {
              x[i] = h[i];
              r[i] = s[i];
            }
          *iters = it + 1;
          *rel_res = sqrt (orc_dot (n, r, r)) / norm_b;
          status = *rel_res < eps ? 0 : 2;
          break;
        }
      const double omega = ts / tt;                           /* :488 */
      for (int i = 0; i < n; i++)                             /* :491-494 */
        {
          r[i] = s[i] - omega * t[i];
          x[i] = h[i] + omega * z[i];
        }
      *iters = it + 1;
      *rel_res = sqrt (orc_dot (n, r, r)) / norm_b;           /* :497-501 */
      if (*rel_res < eps)                                     /* :512 */
        {
          status = 0;
          break;
        }
      rho_prev = rho;
      omega_prev = omega;
    }
  free (mem);
  return status;
}
