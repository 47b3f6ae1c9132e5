/*
 * CPU oracle for the block-sparse hot path — TEST INFRASTRUCTURE ONLY.
 * See oracle.h for the pinning story. Compiled with -ffp-contract=off so that
 * x86 and Arm hosts produce identical bits (no fused multiply-add contraction),
 * matching the reference's own x86 host build, which has no FMA either.
 */
/* POSIX barriers (the threaded BiCGStab) under -std=c11 */
#define _POSIX_C_SOURCE 200809L
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

/* M^-1 v: point Jacobi (P), block Jacobi (Minv: n/bs blocks of bs x bs,
 * row-major) or none. */
static void orc_apply_precond (int n, int use_precond, const double *P, const double *Minv, int bs,
                               const double *v, double *out)
{
  if (Minv)
    {
      for (int br = 0; br < n / bs; br++)
        for (int r = 0; r < bs; r++)
          {
            double acc = 0.0;
            for (int c = 0; c < bs; c++)
              acc += Minv[((size_t) br * bs + r) * bs + c] * v[br * bs + c];
            out[br * bs + r] = acc;
          }
      return;
    }
  for (int i = 0; i < n; i++)
    out[i] = use_precond ? P[i] * v[i] : v[i];
}

static int orc_bicgstab_core (int n, const int *row_ptr, const int *cols, const double *vals,
                              const double *b, double *x, double eps, int max_iterations,
                              int use_precond, const double *Minv, int bs, int *iters, double *rel_res);

int orc_bicgstab_f64 (int n, const int *row_ptr, const int *cols, const double *vals,
                      const double *b, double *x, double eps, int max_iterations,
                      int use_precond, int *iters, double *rel_res)
{
  return orc_bicgstab_core (n, row_ptr, cols, vals, b, x, eps, max_iterations, use_precond, NULL, 1, iters,
                            rel_res);
}

/* Inverse of each bs x bs diagonal block of a CSR matrix whose rows group
 * into block rows of bs (Gauss-Jordan with partial pivoting), the identity
 * where the block is zero or a pivot falls below 1e-20 times its largest
 * entry: the block form of the point rule of bicgstab.cu:201-225. */
void orc_block_jacobi_f64 (int n, int bs, const int *row_ptr, const int *cols, const double *vals, double *Minv)
{
  double *a = (double *) malloc (sizeof (double) * (size_t) bs * bs);
  for (int br = 0; br < n / bs; br++)
    {
      double *inv = Minv + (size_t) br * bs * bs;
      double amax = 0.0;
      for (int r = 0; r < bs; r++)
        {
          for (int c = 0; c < bs; c++)
            {
              a[r * bs + c] = 0.0;
              inv[r * bs + c] = r == c ? 1.0 : 0.0;
            }
          const int row = br * bs + r;
          for (int e = row_ptr[row]; e < row_ptr[row + 1]; e++)
            if (cols[e] >= br * bs && cols[e] < (br + 1) * bs)
              a[r * bs + cols[e] - br * bs] = vals[e];
        }
      for (int k = 0; k < bs * bs; k++)
        amax = fabs (a[k]) > amax ? fabs (a[k]) : amax;
      int ok = amax > 0.0;
      for (int c = 0; c < bs && ok; c++)
        {
          int piv = c;
          for (int r = c + 1; r < bs; r++)
            if (fabs (a[r * bs + c]) > fabs (a[piv * bs + c]))
              piv = r;
          if (!(fabs (a[piv * bs + c]) >= 1e-20 * amax))
            {
              ok = 0;
              break;
            }
          for (int k = 0; k < bs && piv != c; k++)
            {
              double t = a[c * bs + k];
              a[c * bs + k] = a[piv * bs + k];
              a[piv * bs + k] = t;
              t = inv[c * bs + k];
              inv[c * bs + k] = inv[piv * bs + k];
              inv[piv * bs + k] = t;
            }
          const double d = 1.0 / a[c * bs + c];
          for (int k = 0; k < bs; k++)
            {
              a[c * bs + k] *= d;
              inv[c * bs + k] *= d;
            }
          for (int r = 0; r < bs; r++)
            if (r != c && a[r * bs + c] != 0.0)
              {
                const double f = a[r * bs + c];
                for (int k = 0; k < bs; k++)
                  {
                    a[r * bs + k] -= f * a[c * bs + k];
                    inv[r * bs + k] -= f * inv[c * bs + k];
                  }
              }
        }
      if (!ok)
        for (int k = 0; k < bs * bs; k++)
          inv[k] = k / bs == k % bs ? 1.0 : 0.0;
    }
  free (a);
}

/* The reference recurrences with block-Jacobi right preconditioning
 * (q = Minv p, z = Minv s): the block form of bicgstab.cu:454-475. */
int orc_bicgstab_bj_f64 (int n, int bs, const int *row_ptr, const int *cols, const double *vals,
                         const double *b, double *x, double eps, int max_iterations, int *iters, double *rel_res)
{
  double *Minv = (double *) malloc (sizeof (double) * (size_t) n * bs);
  orc_block_jacobi_f64 (n, bs, row_ptr, cols, vals, Minv);
  const int st = orc_bicgstab_core (n, row_ptr, cols, vals, b, x, eps, max_iterations, 1, Minv, bs, iters,
                                    rel_res);
  free (Minv);
  return st;
}

static int orc_bicgstab_core (int n, const int *row_ptr, const int *cols, const double *vals,
                              const double *b, double *x, double eps, int max_iterations,
                              int use_precond, const double *Minv, int bs, int *iters, double *rel_res)
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
      orc_apply_precond (n, use_precond, P, Minv, bs, p, q);  /* :454-457 */
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
      orc_apply_precond (n, use_precond, P, Minv, bs, s, z);  /* :472-475 */
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

/* ---------------------------------------------- band generator (C) --- */
/* The seeded random-band workload of the block-size sweep, restated from
 * its specification (the same as oracle.py's numpy gen_band_bcsr, which the
 * tests pin to the product's generator): block row i takes min(k, W)
 * distinct block columns from [max(0, i-h), min(nbr-1, i+h)] (W wide) by a
 * partial Fisher-Yates shuffle on a per-row SplitMix64 stream (stream 0),
 * sorted; its k*bs*bs values U[-1, 1) come in storage order from stream 1.
 * No reference counterpart: the reference generates only contiguous bands
 * (gen_n_diag_bcsr). The CSR form expands the blocks directly (the CPU
 * baseline's input, common/matrix_converters.h:88-117 layout), threaded
 * over block rows, whose streams are independent. */

static uint64_t orc_mix64 (uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t orc_next (uint64_t *state)
{
  *state += 0x9E3779B97F4A7C15ull;
  return orc_mix64 (*state);
}

static uint64_t orc_row_state (uint64_t seed, uint64_t stream, uint64_t row)
{
  uint64_t s = row * 0x9E3779B97F4A7C15ull + (seed * 0xD1B54A32D192ED03ull + stream * 0x8CB92BA72F3D8DD7ull);
  return orc_next (&s);
}

static double orc_pm1 (uint64_t z) { return (double) (z >> 11) * (2.0 / 9007199254740992.0) - 1.0; }

static int orc_band_width (int i, int nbr, int half, int *lo)
{
  *lo = i - half > 0 ? i - half : 0;
  const int hi = i + half < nbr - 1 ? i + half : nbr - 1;
  return hi - *lo + 1;
}

int orc_band_blocks (int nbr, int bpr, int half, int i)
{
  int lo;
  const int w = orc_band_width (i, nbr, half, &lo);
  return bpr < w ? bpr : w;
}

/* The sorted block columns of block row i (k of them) into out. */
static void orc_band_cols (int nbr, int bpr, int half, uint64_t seed, int i, int *perm, int *out)
{
  int lo;
  const int w = orc_band_width (i, nbr, half, &lo);
  const int k = bpr < w ? bpr : w;
  for (int j = 0; j < w; j++)
    perm[j] = j;
  uint64_t st = orc_row_state (seed, 0, (uint64_t) i);
  for (int j = 0; j < k; j++)
    {
      const uint64_t z = orc_next (&st);
      const int pick = j + (int) (z % (uint64_t) (w - j));
      const int a = perm[j];
      perm[j] = perm[pick];
      perm[pick] = a;
    }
  for (int j = 0; j < k; j++)
    out[j] = perm[j] + lo;
  qsort (out, (size_t) k, sizeof (int), orc_cmp_int);
}

typedef struct
{
  int nbr, bpr, half, bs, is_f64, csr, begin, end;
  uint64_t seed;
  const int64_t *row_ptr; /* block-row offsets (BCSR) or scalar-row offsets (CSR) */
  int *cols;
  void *vals;
} orc_band_task;

static void *orc_band_worker (void *arg)
{
  const orc_band_task *t = (const orc_band_task *) arg;
  const int bs = t->bs, e = bs * bs;
  int *perm = (int *) malloc (sizeof (int) * (size_t) (2 * t->half + 1));
  int *bc = (int *) malloc (sizeof (int) * (size_t) (t->bpr > 0 ? t->bpr : 1));
  double *blk = (double *) malloc (sizeof (double) * (size_t) t->bpr * e + 1);
  for (int i = t->begin; i < t->end; i++)
    {
      const int k = orc_band_blocks (t->nbr, t->bpr, t->half, i);
      orc_band_cols (t->nbr, t->bpr, t->half, t->seed, i, perm, bc);
      uint64_t vs = orc_row_state (t->seed, 1, (uint64_t) i);
      for (int j = 0; j < k * e; j++)
        blk[j] = orc_pm1 (orc_next (&vs));
      if (!t->csr)
        {
          const int64_t b0 = t->row_ptr[i];
          for (int b = 0; b < k; b++)
            t->cols[b0 + b] = bc[b];
          for (int j = 0; j < k * e; j++)
            {
              if (t->is_f64)
                ((double *) t->vals)[b0 * e + j] = blk[j];
              else
                ((float *) t->vals)[b0 * e + j] = (float) blk[j];
            }
          continue;
        }
      for (int r = 0; r < bs; r++)
        {
          int64_t o = t->row_ptr[(int64_t) i * bs + r];
          for (int b = 0; b < k; b++)
            for (int c = 0; c < bs; c++, o++)
              {
                t->cols[o] = bc[b] * bs + c;
                const double v = blk[(size_t) b * e + (size_t) r * bs + c];
                if (t->is_f64)
                  ((double *) t->vals)[o] = v;
                else
                  ((float *) t->vals)[o] = (float) v;
              }
        }
    }
  free (perm);
  free (bc);
  free (blk);
  return NULL;
}

/* row_ptr: the caller's offsets (int64, from orc_band_blocks); cols and
 * vals: BCSR (csr = 0) or CSR (csr = 1). */
void orc_gen_band (int nbr, int bpr, int half, int bs, uint64_t seed, int is_f64, int csr,
                   const int64_t *row_ptr, int *cols, void *vals, int threads)
{
  if (threads < 1)
    threads = 1;
  if (threads > 256)
    threads = 256;
  pthread_t tid[256];
  orc_band_task task[256];
  for (int t = 0; t < threads; t++)
    {
      orc_band_task *k = &task[t];
      k->nbr = nbr;
      k->bpr = bpr;
      k->half = half;
      k->bs = bs;
      k->is_f64 = is_f64;
      k->csr = csr;
      k->seed = seed;
      k->row_ptr = row_ptr;
      k->cols = cols;
      k->vals = vals;
      k->begin = (int) ((int64_t) nbr * t / threads);
      k->end = (int) ((int64_t) nbr * (t + 1) / threads);
      if (threads > 1)
        pthread_create (&tid[t], NULL, orc_band_worker, k);
      else
        orc_band_worker (k);
    }
  if (threads > 1)
    for (int t = 0; t < threads; t++)
      pthread_join (tid[t], NULL);
}

/* x_i = U[-1, 1) of the row state (seed, stream, i). */
void orc_gen_uniform_vector (int64_t n, uint64_t seed, uint64_t stream, int is_f64, void *out)
{
  for (int64_t i = 0; i < n; i++)
    {
      const double v = orc_pm1 (orc_row_state (seed, stream, (uint64_t) i));
      if (is_f64)
        ((double *) out)[i] = v;
      else
        ((float *) out)[i] = (float) v;
    }
}

/* ------------------------------------------- threaded BiCGStab (CPU) --- */
/* The recurrences of orc_bicgstab_f64 (gpu/bicgstab.cu:426-513, last
 * iterate returned) on `threads` host threads: each owns a contiguous range
 * of rows for every vector update and product; dot products are per-thread
 * partials summed in thread order by every thread. The CPU solve baseline
 * on all host cores; orc_bicgstab_f64 is the single-thread one (and this
 * function with one thread reproduces it bit for bit). */

typedef struct
{
  int n, threads, max_iterations, use_precond;
  const int *row_ptr, *cols;
  const double *vals, *b;
  double *x, *mem, eps, norm_b;
  double *part; /* threads x 4 partial sums */
  pthread_barrier_t *bar;
  int status, iters;
  double rel;
} orc_bicg_shared;

typedef struct
{
  orc_bicg_shared *S;
  int t;
} orc_bicg_arg;

static double orc_sum_part (const orc_bicg_shared *S, int k)
{
  double s = 0.0;
  for (int t = 0; t < S->threads; t++)
    s += S->part[t * 4 + k];
  return s;
}

static void *orc_bicg_worker (void *arg)
{
  orc_bicg_shared *S = ((orc_bicg_arg *) arg)->S;
  const int t = ((orc_bicg_arg *) arg)->t, n = S->n;
  const int lo = (int) ((int64_t) n * t / S->threads), hi = (int) ((int64_t) n * (t + 1) / S->threads);
  double *r = S->mem, *rh = r + n, *p = r + 2 * (size_t) n, *v = r + 3 * (size_t) n, *h = r + 4 * (size_t) n;
  double *s = r + 5 * (size_t) n, *tv = r + 6 * (size_t) n, *P = r + 7 * (size_t) n, *q = r + 8 * (size_t) n;
  double *z = r + 9 * (size_t) n, *x = S->x;
  double *my = S->part + t * 4;
  for (int row = lo; row < hi; row++)
    {
      P[row] = 1.0;
      if (S->use_precond)
        for (int e = S->row_ptr[row]; e < S->row_ptr[row + 1]; e++)
          if (S->cols[e] == row)
            {
              P[row] = fabs (S->vals[e]) < 1e-20 ? 1.0 : 1.0 / S->vals[e];
              break;
            }
      x[row] = 0.0;
      r[row] = rh[row] = S->b[row];
      p[row] = v[row] = 0.0;
    }
  double rho_prev = 1.0, omega_prev = 1.0, alpha = 1.0;
  int status = 1, iters = 0;
  double rel = S->norm_b > 0 ? 1.0 : 0.0;
  for (int it = 0; it < S->max_iterations && S->norm_b > 0; it++)
    {
      double a = 0.0;
      for (int i = lo; i < hi; i++)
        a += rh[i] * r[i];
      my[0] = a;
      pthread_barrier_wait (S->bar);
      const double rho = orc_sum_part (S, 0);
      if (rho == 0.0)
        {
          status = 2;
          break;
        }
      const double beta = rho / rho_prev * alpha / omega_prev;
      for (int i = lo; i < hi; i++)
        {
          p[i] = r[i] + beta * (p[i] - omega_prev * v[i]);
          q[i] = S->use_precond ? P[i] * p[i] : p[i];
        }
      pthread_barrier_wait (S->bar);
      a = 0.0;
      for (int row = lo; row < hi; row++)
        {
          double dot = 0.0;
          for (int e = S->row_ptr[row]; e < S->row_ptr[row + 1]; e++)
            dot += S->vals[e] * q[S->cols[e]];
          v[row] = dot;
          a += rh[row] * dot;
        }
      my[1] = a;
      pthread_barrier_wait (S->bar);
      const double rh_v = orc_sum_part (S, 1);
      if (rh_v == 0.0)
        {
          status = 2;
          break;
        }
      alpha = rho / rh_v;
      for (int i = lo; i < hi; i++)
        {
          h[i] = x[i] + alpha * q[i];
          s[i] = r[i] - alpha * v[i];
          z[i] = S->use_precond ? P[i] * s[i] : s[i];
        }
      pthread_barrier_wait (S->bar);
      double ts = 0.0, tt = 0.0;
      for (int row = lo; row < hi; row++)
        {
          double dot = 0.0;
          for (int e = S->row_ptr[row]; e < S->row_ptr[row + 1]; e++)
            dot += S->vals[e] * z[S->cols[e]];
          tv[row] = dot;
          ts += dot * s[row];
          tt += dot * dot;
        }
      my[2] = ts;
      my[3] = tt;
      pthread_barrier_wait (S->bar);
      const double tsum = orc_sum_part (S, 2), ttsum = orc_sum_part (S, 3);
      if (ttsum == 0.0)
        {
          status = 2;
          break;
        }
      const double omega = tsum / ttsum;
      a = 0.0;
      for (int i = lo; i < hi; i++)
        {
          r[i] = s[i] - omega * tv[i];
          x[i] = h[i] + omega * z[i];
          a += r[i] * r[i];
        }
      /* part 1 was last read after the (rh, v) barrier, two barriers ago:
       * it carries the (r, r) sum now */
      my[1] = a;
      pthread_barrier_wait (S->bar);
      iters = it + 1;
      rel = sqrt (orc_sum_part (S, 1)) / S->norm_b;
      if (rel < S->eps)
        {
          status = 0;
          break;
        }
      rho_prev = rho;
      omega_prev = omega;
    }
  if (t == 0)
    {
      S->status = S->norm_b > 0 ? status : 0;
      S->iters = iters;
      S->rel = rel;
    }
  return NULL;
}

int orc_bicgstab_mt_f64 (int n, const int *row_ptr, const int *cols, const double *vals, const double *b,
                         double *x, double eps, int max_iterations, int use_precond, int threads, int *iters,
                         double *rel_res)
{
  if (threads < 1)
    threads = 1;
  if (threads > 256)
    threads = 256;
  orc_bicg_shared S;
  memset (&S, 0, sizeof S);
  S.n = n;
  S.threads = threads;
  S.max_iterations = max_iterations;
  S.use_precond = use_precond;
  S.row_ptr = row_ptr;
  S.cols = cols;
  S.vals = vals;
  S.b = b;
  S.x = x;
  S.eps = eps;
  S.mem = (double *) calloc ((size_t) n * 10, sizeof (double));
  S.part = (double *) calloc ((size_t) threads * 4, sizeof (double));
  double nb = 0.0;
  for (int i = 0; i < n; i++)
    nb += b[i] * b[i];
  S.norm_b = sqrt (nb);
  pthread_barrier_t bar;
  pthread_barrier_init (&bar, NULL, (unsigned) threads);
  S.bar = &bar;
  pthread_t tid[256];
  orc_bicg_arg args[256];
  for (int t = 0; t < threads; t++)
    {
      args[t].S = &S;
      args[t].t = t;
      if (t > 0)
        pthread_create (&tid[t], NULL, orc_bicg_worker, &args[t]);
    }
  orc_bicg_worker (&args[0]);
  for (int t = 1; t < threads; t++)
    pthread_join (tid[t], NULL);
  pthread_barrier_destroy (&bar);
  free (S.mem);
  free (S.part);
  *iters = S.iters;
  *rel_res = S.rel;
  return S.status;
}
