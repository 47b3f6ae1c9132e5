// The reference's named SpMV variants, as GB300 kernels of this library.
//
// Each kernel keeps the thread mapping that gives the variant its name in
// gpu/gpu_matrix_multiplier.cu (thread per scalar row, warp per row, column
// by column, ...), so the per-variant timings stay comparable with the
// reference's result.json keys. The work inside follows this library's own
// rules: read-only loads for x, streaming loads for values, shuffle instead of
// shared-memory trees. Two reference defects are not carried over:
//  * coal-x (gpu_matrix_multiplier.cu:402-469) staged only the first block
//    row's x segment per 32-thread CTA, right only for x == 1; here every
//    block row stages its own segment.
//  * column-by-column (:485-673) double-counted columns when bs does not
//    divide 32; here the lanes past (32/bs)*bs sit idle.
#include "device_common.cuh"
#include "internal.h"

#include <cstdint>

namespace bmfp
{
namespace
{
constexpr int kThreads = 256;

inline unsigned blocks_for (int64_t threads, int per_block)
{
  return (unsigned) ((threads + per_block - 1) / per_block);
}

template <typename T> __device__ __forceinline__ T warp_sum (T v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    v += __shfl_xor_sync (0xffffffffu, v, off);
  return v;
}

// Tree over the q = lane / bs slots (Q of them) of a warp: after it, lanes
// with q == 0 hold the sum over q of their row r = lane % bs.
template <typename T> __device__ __forceinline__ T slot_tree_sum (T acc, int bs, int q, int Q)
{
  int top = 1;
  while (top < Q)
    top <<= 1;
  for (int s = top >> 1; s > 0; s >>= 1)
    {
      const T other = __shfl_down_sync (0xffffffffu, acc, s * bs);
      if (q < Q && q + s < Q)
        acc += other;
    }
  return acc;
}

// -------------------------------------------------------------------- CSR

// "GPU CSR": one thread per row (gpu_matrix_multiplier.cu:65-86).
template <typename T>
__global__ void __launch_bounds__ (kThreads)
  csr_scalar_kernel (int n_rows, const int *__restrict__ row_ptr, const int *__restrict__ cols,
                     const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t row = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n_rows)
    return;
  T sum = 0;
  for (int e = __ldg (row_ptr + row); e < __ldg (row_ptr + row + 1); e++)
    sum = fma (__ldg (vals + e), __ldg (x + __ldg (cols + e)), sum);
  y[row] = sum;
}

// "GPU CSR-Vector": one warp per row, lanes strided over its entries
// (gpu_matrix_multiplier.cu:165-196).
template <typename T>
__global__ void __launch_bounds__ (kThreads)
  csr_vector_kernel (int n_rows, const int *__restrict__ row_ptr, const int *__restrict__ cols,
                     const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t row = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n_rows)
    return; // whole warp
  T dot = 0;
  for (int e = __ldg (row_ptr + row) + lane; e < __ldg (row_ptr + row + 1); e += 32)
    dot = fma (dev::ld_stream (vals + e), __ldg (x + __ldg (cols + e)), dot);
  dot = warp_sum (dot);
  if (lane == 0)
    y[row] = dot;
}

// ------------------------------------------------------------ row-major BCSR

// "GPU BCSR (row major, thread per row)" (:275-304): thread per scalar row.
template <typename T>
__global__ void __launch_bounds__ (kThreads)
  bcsr_row_thread_kernel (int nbr, int bs, const int *__restrict__ row_ptr,
                          const int *__restrict__ cols, const T *__restrict__ vals,
                          const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t idx = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t br = idx / bs;
  const int r = (int) (idx % bs);
  if (br >= nbr)
    return;
  T acc = 0;
  for (int b = __ldg (row_ptr + br); b < __ldg (row_ptr + br + 1); b++)
    {
      const T *xb = x + (size_t) __ldg (cols + b) * bs;
      const T *a = vals + (size_t) b * bs * bs + (size_t) r * bs;
      for (int c = 0; c < bs; c++)
        acc = fma (__ldg (xb + c), __ldg (a + c), acc);
    }
  y[idx] = acc;
}

// "GPU BCSR (row major, warp per row)" (:306-339): a warp per scalar row,
// lanes strided over the bs*nblk entries of that row.
template <typename T, int BS>
__global__ void __launch_bounds__ (kThreads)
  bcsr_row_warp_kernel (int nbr, const int *__restrict__ row_ptr, const int *__restrict__ cols,
                        const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t wid = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t br = wid / BS;
  const int r = (int) (wid % BS);
  if (br >= nbr)
    return; // whole warp
  const int first = __ldg (row_ptr + br);
  const int len = (__ldg (row_ptr + br + 1) - first) * BS;
  T acc = 0;
  for (int k = lane; k < len; k += 32)
    {
      const int b = first + k / BS, c = k % BS;
      acc = fma (__ldg (x + (size_t) __ldg (cols + b) * BS + c),
                 __ldg (vals + (size_t) b * BS * BS + r * BS + c), acc);
    }
  acc = warp_sum (acc);
  if (lane == 0)
    y[br * BS + r] = acc;
}

// --------------------------------------------------------- column-major BCSR

// "GPU BCSR (column major, thread per row[, template])" (:341-400): thread per
// scalar row over transposed blocks, so the bs threads of a block row read
// consecutive addresses.
template <typename T, int BSC>
__global__ void __launch_bounds__ (kThreads)
  bcsr_col_thread_kernel (int nbr, int bs_rt, const int *__restrict__ row_ptr,
                          const int *__restrict__ cols, const T *__restrict__ vals,
                          const T *__restrict__ x, T *__restrict__ y)
{
  const int bs = BSC ? BSC : bs_rt;
  const int64_t idx = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t br = idx / bs;
  const int r = (int) (idx % bs);
  if (br >= nbr)
    return;
  T acc = 0;
  for (int b = __ldg (row_ptr + br); b < __ldg (row_ptr + br + 1); b++)
    {
      const T *xb = x + (size_t) __ldg (cols + b) * bs;
      const T *a = vals + (size_t) b * bs * bs + r;
      for (int c = 0; c < bs; c++)
        acc = fma (__ldg (xb + c), dev::ld_stream (a + (size_t) c * bs), acc);
    }
  y[idx] = acc;
}

// "GPU BCSR (column major, thread per row, coal x[, template])" (:402-469):
// as above, but the bs threads of a block row first stage the bs entries of x
// for the current block in shared memory with one coalesced load. The CTA is
// a whole number of block rows; all threads step through the CTA's longest
// block row so the barriers are uniform.
template <typename T, int BSC>
__global__ void bcsr_col_coal_x_kernel (int nbr, int bs_rt, const int *__restrict__ row_ptr,
                                        const int *__restrict__ cols,
                                        const T *__restrict__ vals, const T *__restrict__ x,
                                        T *__restrict__ y)
{
  extern __shared__ __align__ (16) unsigned char smem_raw[];
  T *cache = reinterpret_cast<T *> (smem_raw);
  const int bs = BSC ? BSC : bs_rt;
  const int rows_per_cta = blockDim.x / bs;
  const int local_br = threadIdx.x / bs;
  const int r = threadIdx.x % bs;
  const int64_t br = (int64_t) blockIdx.x * rows_per_cta + local_br;
  const bool live = local_br < rows_per_cta && br < nbr;
  const int first = live ? __ldg (row_ptr + br) : 0;
  const int nblk = live ? __ldg (row_ptr + br + 1) - first : 0;
  T *seg = cache + local_br * bs;
  T acc = 0;
  for (int k = 0;; k++)
    {
      const bool active = k < nblk;
      if (active)
        seg[r] = __ldg (x + (size_t) __ldg (cols + first + k) * bs + r);
      __syncthreads ();
      if (active)
        {
          const T *a = vals + (size_t) (first + k) * bs * bs + r;
          for (int c = 0; c < bs; c++)
            acc = fma (seg[c], dev::ld_stream (a + (size_t) c * bs), acc);
        }
      if (!__syncthreads_or (k + 1 < nblk))
        break;
    }
  if (live)
    y[br * bs + r] = acc;
}

// Division by a run-time invariant divisor with a multiply-high (Granlund &
// Montgomery, "Division by invariant integers using multiplication", PLDI
// 1994, fig. 4.1): for 1 <= d < 2^32, l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1, q = (t + ((n - t) >> 1)) >> (l - 1) with
// t = mulhi(m, n); d = 1 is passed as l = 0 and returns n.
struct FastDiv
{
  unsigned m;
  int l;
  unsigned d;
};

__device__ __forceinline__ unsigned fast_div (unsigned n, const FastDiv &f)
{
  if (f.l == 0)
    return n;
  const unsigned t = __umulhi (f.m, n);
  return (t + ((n - t) >> 1)) >> (f.l - 1);
}

FastDiv make_fast_div (unsigned d)
{
  FastDiv f{ 0u, 0, d };
  if (d <= 1)
    return f;
  int l = 0;
  while ((1ull << l) < d)
    l++;
  f.l = l;
  f.m = (unsigned) (((1ull << 32) * ((1ull << l) - d)) / d + 1);
  return f;
}

enum class ColDiv
{
  Plain,
  Fast,
  Po2
};

// "GPU BCSR (column major, column-by-column[, int fastdiv | int po2 |
// template])" (:485-673) and the bs-specialised JIT kernel (main.cpp:178-225):
// a warp per block row; lane (q, r) = (lane / bs, lane % bs) walks the block
// row's columns q, q+Q, ... (Q = 32/bs) reading row r of each column of the
// transposed blocks, then the lanes of each row are summed.
template <typename T, int BSC, ColDiv DIV>
__global__ void __launch_bounds__ (kThreads)
  bcsr_col_by_col_kernel (int nbr, int bs_rt, FastDiv fd, int log2_bs,
                          const int *__restrict__ row_ptr, const int *__restrict__ cols,
                          const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y)
{
  const int bs = BSC ? BSC : bs_rt;
  const int lane = threadIdx.x & 31;
  const int64_t br = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (br >= nbr)
    return; // whole warp
  int q, r, Q;
  if constexpr (DIV == ColDiv::Po2)
    {
      q = lane >> log2_bs;
      r = lane & (bs - 1);
      Q = 32 >> log2_bs;
    }
  else if constexpr (DIV == ColDiv::Fast)
    {
      q = (int) fast_div ((unsigned) lane, fd);
      r = lane - q * bs;
      Q = (int) fast_div (32u, fd);
    }
  else
    {
      q = lane / bs;
      r = lane % bs;
      Q = 32 / bs;
    }
  const int first = __ldg (row_ptr + br), last = __ldg (row_ptr + br + 1);
  T acc = 0;
  if (q < Q)
    for (int col = first * bs + q; col < last * bs; col += Q)
      {
        int b, c;
        if constexpr (DIV == ColDiv::Po2)
          {
            b = col >> log2_bs;
            c = col & (bs - 1);
          }
        else if constexpr (DIV == ColDiv::Fast)
          {
            b = (int) fast_div ((unsigned) col, fd);
            c = col - b * bs;
          }
        else
          {
            b = col / bs;
            c = col % bs;
          }
        acc = fma (dev::ld_stream (vals + (size_t) b * bs * bs + c * bs + r),
                   __ldg (x + (size_t) __ldg (cols + b) * bs + c), acc);
      }
  acc = slot_tree_sum (acc, bs, q, Q);
  if (q == 0)
    y[br * bs + r] = acc;
}

// ---------------------------------------------------------------- dispatch

template <typename T>
int launch_typed (int variant, int n_rows, int bs, const int *rp, const int *c, const T *v,
                  const T *x, T *y, cudaStream_t s)
{
  switch (variant)
    {
    case BMFP_SPMV_CSR_SCALAR:
      csr_scalar_kernel<T><<<blocks_for (n_rows, kThreads), kThreads, 0, s>>> (n_rows, rp, c, v, x, y);
      break;
    case BMFP_SPMV_CSR_VECTOR:
      csr_vector_kernel<T><<<blocks_for ((int64_t) n_rows * 32, kThreads), kThreads, 0, s>>> (
        n_rows, rp, c, v, x, y);
      break;
    case BMFP_SPMV_BCSR_ROW_THREAD:
      bcsr_row_thread_kernel<T><<<blocks_for ((int64_t) n_rows * bs, kThreads), kThreads, 0, s>>> (
        n_rows, bs, rp, c, v, x, y);
      break;
    case BMFP_SPMV_BCSR_ROW_WARP:
      {
        const unsigned g = blocks_for ((int64_t) n_rows * bs * 32, kThreads);
        switch (bs)
          {
#define BMFP_RW(B) case B: bcsr_row_warp_kernel<T, B><<<g, kThreads, 0, s>>> (n_rows, rp, c, v, x, y); break;
            BMFP_RW (1) BMFP_RW (2) BMFP_RW (3) BMFP_RW (4) BMFP_RW (8) BMFP_RW (16) BMFP_RW (32)
#undef BMFP_RW
          default:
            return fail (BMFP_ERROR_NOT_SUPPORTED,
                         "warp-per-row variant is instantiated for bs in {1,2,3,4,8,16,32}, got %d", bs);
          }
        break;
      }
    case BMFP_SPMV_BCSR_COL_THREAD:
      bcsr_col_thread_kernel<T, 0><<<blocks_for ((int64_t) n_rows * bs, kThreads), kThreads, 0, s>>> (
        n_rows, bs, rp, c, v, x, y);
      break;
    case BMFP_SPMV_BCSR_COL_THREAD_TEMPLATE:
      {
        const unsigned g = blocks_for ((int64_t) n_rows * bs, kThreads);
        switch (bs)
          {
#define BMFP_CT(B) case B: bcsr_col_thread_kernel<T, B><<<g, kThreads, 0, s>>> (n_rows, B, rp, c, v, x, y); break;
            BMFP_CT (1) BMFP_CT (2) BMFP_CT (3) BMFP_CT (4) BMFP_CT (8) BMFP_CT (16) BMFP_CT (32)
#undef BMFP_CT
          default:
            return fail (BMFP_ERROR_NOT_SUPPORTED,
                         "template variant is instantiated for bs in {1,2,3,4,8,16,32}, got %d", bs);
          }
        break;
      }
    case BMFP_SPMV_BCSR_COL_COAL_X:
    case BMFP_SPMV_BCSR_COL_COAL_X_TEMPLATE:
      {
        if (bs > 1024)
          return fail (BMFP_ERROR_NOT_SUPPORTED, "coal-x needs bs <= 1024");
        const int rows_per_cta = bs >= kThreads ? 1 : kThreads / bs;
        const int threads = rows_per_cta * bs;
        const unsigned g = blocks_for (n_rows, rows_per_cta);
        const size_t shm = (size_t) threads * sizeof (T);
        if (variant == BMFP_SPMV_BCSR_COL_COAL_X)
          bcsr_col_coal_x_kernel<T, 0><<<g, threads, shm, s>>> (n_rows, bs, rp, c, v, x, y);
        else
          switch (bs)
            {
#define BMFP_CX(B) case B: bcsr_col_coal_x_kernel<T, B><<<g, threads, shm, s>>> (n_rows, B, rp, c, v, x, y); break;
              BMFP_CX (1) BMFP_CX (2) BMFP_CX (3) BMFP_CX (4) BMFP_CX (8) BMFP_CX (16) BMFP_CX (32)
#undef BMFP_CX
            default:
              return fail (BMFP_ERROR_NOT_SUPPORTED,
                           "template variant is instantiated for bs in {1,2,3,4,8,16,32}, got %d", bs);
            }
        break;
      }
    case BMFP_SPMV_BCSR_COL_BY_COL:
    case BMFP_SPMV_BCSR_COL_BY_COL_FASTDIV:
    case BMFP_SPMV_BCSR_COL_BY_COL_PO2:
    case BMFP_SPMV_BCSR_COL_BY_COL_TEMPLATE:
    case BMFP_SPMV_BCSR_JIT:
      {
        if (bs > 32)
          return fail (BMFP_ERROR_NOT_SUPPORTED, "column-by-column needs bs <= 32 (warp per block row)");
        const unsigned g = blocks_for ((int64_t) n_rows * 32, kThreads);
        const FastDiv fd = make_fast_div ((unsigned) bs);
        int lg = 0;
        while ((1 << lg) < bs)
          lg++;
        if (variant == BMFP_SPMV_BCSR_COL_BY_COL)
          bcsr_col_by_col_kernel<T, 0, ColDiv::Plain><<<g, kThreads, 0, s>>> (n_rows, bs, fd, lg, rp, c, v, x, y);
        else if (variant == BMFP_SPMV_BCSR_COL_BY_COL_FASTDIV)
          bcsr_col_by_col_kernel<T, 0, ColDiv::Fast><<<g, kThreads, 0, s>>> (n_rows, bs, fd, lg, rp, c, v, x, y);
        else if (variant == BMFP_SPMV_BCSR_COL_BY_COL_PO2)
          {
            if ((1 << lg) != bs)
              return fail (BMFP_ERROR_NOT_SUPPORTED, "po2 variant needs a power-of-two bs, got %d", bs);
            bcsr_col_by_col_kernel<T, 0, ColDiv::Po2><<<g, kThreads, 0, s>>> (n_rows, bs, fd, lg, rp, c, v, x, y);
          }
        else
          switch (bs)
            {
#define BMFP_CC(B) case B: bcsr_col_by_col_kernel<T, B, ColDiv::Plain><<<g, kThreads, 0, s>>> (n_rows, B, fd, lg, rp, c, v, x, y); break;
              BMFP_CC (1) BMFP_CC (2) BMFP_CC (3) BMFP_CC (4) BMFP_CC (8) BMFP_CC (16) BMFP_CC (32)
#undef BMFP_CC
            default:
              return fail (BMFP_ERROR_NOT_SUPPORTED,
                           "template variant is instantiated for bs in {1,2,3,4,8,16,32}, got %d", bs);
            }
        break;
      }
    default:
      return fail (BMFP_ERROR_INVALID_VALUE, "not a hand-written reference variant: %d", variant);
    }
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}
} // namespace

int spmv_reference_variant (int dtype, int variant, int n_rows, int /*n_cols*/, int bs,
                            int64_t /*nnz*/, const int *row_ptr, const int *cols,
                            const void *vals, const void *x, void *y, cudaStream_t stream)
{
  if (n_rows == 0)
    return BMFP_SUCCESS;
  if (dtype == BMFP_R64F)
    return launch_typed<double> (variant, n_rows, bs, row_ptr, cols, (const double *) vals,
                                 (const double *) x, (double *) y, stream);
  return launch_typed<float> (variant, n_rows, bs, row_ptr, cols, (const float *) vals,
                              (const float *) x, (float *) y, stream);
}

} // namespace bmfp
