// GB300-native sparse matrix-vector products.
//
// y = A x for BCSR with row-major bs x bs blocks (the layout of
// common/matrix_converters.h:13-82) and for CSR. Both are HBM-bound streams:
// every value and block column is read once, x is re-read from L1/L2 by the
// neighbouring block rows, y is written once. The kernels are organised
// around that:
//
//  * bcsr_flat_kernel (bs = 2, 4, 8, 16, 32): an aligned group of G lanes owns
//    one block row. The block row's values are one contiguous run
//    (row_ptr[i]*bs*bs .. row_ptr[i+1]*bs*bs) and the group walks it in
//    16-byte vectors, lane l taking vector l of each G*16-byte chunk, so a
//    warp-wide load is one fully used 512-byte stretch. Because bs*bs and the
//    chunk are both powers of two, every lane keeps a fixed (row, column
//    group) position inside a block (chunk >= block) or a fixed column group
//    and a fixed set of rows per phase (chunk < block). Partial row sums are
//    combined with xor-shuffles over exactly the lane bits that vary the
//    column, so the reduction costs log2 steps and no shared memory.
//  * bcsr_tpr_kernel (any bs <= 32, e.g. 3 for frame elements): a warp owns
//    a block row, lane (q, r) takes scalar row r of blocks q, q+Q, ... with
//    Q = 32/bs, then a shuffle tree sums over q.
//  * bcsr_row_kernel (bs > 32): one thread per scalar row.
//  * csr_subwarp_kernel: G lanes per row, strided over its entries
//    (the bs = 1 case and plain CSR).
//
// Values are loaded with the streaming (evict-first) hint, x through the
// read-only path. No tensor cores: a single-vector product has no reuse of A
// to feed them.
#include "internal.h"
#include "spmv_core.cuh"

#include <algorithm>

namespace bmfp
{
namespace
{
constexpr int kThreads = 256;

// Grid-stride over block rows: group g takes rows g, g + n_groups, ...
template <typename T, int BS, int G, int U>
__global__ void __launch_bounds__ (kThreads)
  bcsr_flat_kernel (int n_block_rows, const int *__restrict__ row_ptr,
                    const int *__restrict__ cols, const T *__restrict__ vals,
                    const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t group = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t n_groups = (int64_t) gridDim.x * blockDim.x / G;
  core::NoEpilogue epi;
  for (int64_t row = group; row < n_block_rows; row += n_groups)
    core::flat_row<T, BS, G, U> ((int) row, row_ptr, cols, vals, x, y, epi);
}

// Row-owner mapping: BS lanes per block row, one per scalar row.
template <typename T, int BS>
__global__ void __launch_bounds__ (kThreads)
  bcsr_rowown_kernel (int n_block_rows, const int *__restrict__ row_ptr, const int *__restrict__ cols,
                      const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t group = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) / BS;
  const int64_t n_groups = (int64_t) gridDim.x * blockDim.x / BS;
  core::NoEpilogue epi;
  for (int64_t row = group; row < n_block_rows; row += n_groups)
    core::rowown_row<T, BS> ((int) row, row_ptr, cols, vals, x, y, epi);
}

// Column-owner mapping over column-major blocks: BS lanes per block row,
// lane r owns scalar row r and walks the columns of each block; for a fixed
// column the BS lanes read BS consecutive values (one contiguous stretch per
// load) and the same x entry (a broadcast). No cross-lane reduction, and
// fewer L1 transactions per FP64 FMA than the row-owner walk of row-major
// lines. One accumulator and scalar x loads measured fastest.
template <typename T, int BS>
__global__ void __launch_bounds__ (kThreads)
  bcsr_colown_kernel (int nbr, const int *__restrict__ row_ptr, const int *__restrict__ cols,
                      const T *__restrict__ vals_cm, const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t idx = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = idx / BS;
  const int r = (int) (idx % BS);
  if (row >= nbr)
    return;
  const int beg = __ldg (row_ptr + row), end = __ldg (row_ptr + row + 1);
  T acc = 0;
  for (int b = beg; b < end; b++)
    {
      const T *a = vals_cm + (size_t) b * BS * BS + r;
      const T *xb = x + (size_t) __ldg (cols + b) * BS;
#pragma unroll
      for (int c = 0; c < BS; c++)
        acc = fma (__ldg (xb + c), dev::ld_stream (a + (size_t) c * BS), acc);
    }
  y[idx] = acc;
}

// Row-major -> column-major blocks: element (r, c) of block b moves from
// b*BS*BS + r*BS + c to b*BS*BS + c*BS + r.
template <typename T>
__global__ void transpose_blocks_kernel (int64_t total, int bs, const T *__restrict__ in, T *__restrict__ out)
{
  const int64_t e2 = (int64_t) bs * bs;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t) gridDim.x * blockDim.x)
    {
      const int64_t b = i / e2;
      const int k = (int) (i - b * e2);
      const int r = k / bs, c = k - (k / bs) * bs;
      out[b * e2 + (int64_t) c * bs + r] = in[i];
    }
}

template <typename T, int BSC>
__global__ void __launch_bounds__ (kThreads)
  bcsr_tpr_kernel (int n_block_rows, int bs_rt, const int *__restrict__ row_ptr,
                   const int *__restrict__ cols, const T *__restrict__ vals,
                   const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t warp = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = (int64_t) gridDim.x * blockDim.x >> 5;
  core::NoEpilogue epi;
  for (int64_t row = warp; row < n_block_rows; row += n_warps)
    core::tpr_row<T, BSC> ((int) row, bs_rt, row_ptr, cols, vals, x, y, epi);
}

// Thread per scalar row (bs > 32).
template <typename T>
__global__ void __launch_bounds__ (kThreads)
  bcsr_row_kernel (int n_block_rows, int bs, const int *__restrict__ row_ptr,
                   const int *__restrict__ cols, const T *__restrict__ vals,
                   const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t idx = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t br = idx / bs;
  const int r = (int) (idx % bs);
  if (br >= n_block_rows)
    return;
  T acc = 0;
  for (int b = __ldg (row_ptr + br); b < __ldg (row_ptr + br + 1); b++)
    {
      const T *a = vals + (size_t) b * bs * bs + (size_t) r * bs;
      const T *xb = x + (size_t) __ldg (cols + b) * bs;
      for (int c = 0; c < bs; c++)
        acc = fma (a[c], dev::ld_cached (xb + c), acc);
    }
  y[idx] = acc;
}

template <typename T, int G>
__global__ void __launch_bounds__ (kThreads)
  csr_subwarp_kernel (int n_rows, const int *__restrict__ row_ptr, const int *__restrict__ cols,
                      const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y)
{
  const int64_t group = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t n_groups = (int64_t) gridDim.x * blockDim.x / G;
  core::NoEpilogue epi;
  for (int64_t row = group; row < n_rows; row += n_groups)
    core::csr_row<T, G> ((int) row, row_ptr, cols, vals, x, y, epi);
}

// ---------------------------------------------------------------- dispatch

inline int vec_elems (int dtype) { return dtype == BMFP_R64F ? 2 : 4; }

inline bool flat_bs (int bs) { return bs == 2 || bs == 4 || bs == 8 || bs == 16 || bs == 32; }

inline bool flat_lanes_ok (int dtype, int bs, int g)
{
  return (g == 2 || g == 4 || g == 8 || g == 16 || g == 32) && g * vec_elems (dtype) >= bs;
}

template <typename T, int BS, int G>
int launch_flat_g (int nbr, const int *rp, const int *c, const T *v, const T *x, T *y,
                   cudaStream_t s)
{
  if constexpr (G * dev::Vec16<T>::N < BS)
    return fail (BMFP_ERROR_INVALID_VALUE, "lane count too small for this block size");
  else
    {
      const int64_t threads = (int64_t) nbr * G;
      const unsigned grid = (unsigned) ((threads + kThreads - 1) / kThreads);
      bcsr_flat_kernel<T, BS, G, 4><<<grid, kThreads, 0, s>>> (nbr, rp, c, v, x, y);
      BMFP_LAUNCH_CHECK ();
      return BMFP_SUCCESS;
    }
}

template <typename T, int BS>
int launch_flat (int nbr, int g, const int *rp, const int *c, const T *v, const T *x, T *y,
                 cudaStream_t s)
{
  switch (g)
    {
    case 2: return launch_flat_g<T, BS, 2> (nbr, rp, c, v, x, y, s);
    case 4: return launch_flat_g<T, BS, 4> (nbr, rp, c, v, x, y, s);
    case 8: return launch_flat_g<T, BS, 8> (nbr, rp, c, v, x, y, s);
    case 16: return launch_flat_g<T, BS, 16> (nbr, rp, c, v, x, y, s);
    case 32: return launch_flat_g<T, BS, 32> (nbr, rp, c, v, x, y, s);
    default: return fail (BMFP_ERROR_INVALID_VALUE, "invalid lane count %d", g);
    }
}

template <typename T, int G>
int launch_csr_g (int n, const int *rp, const int *c, const T *v, const T *x, T *y, cudaStream_t s)
{
  const int64_t threads = (int64_t) n * G;
  const unsigned grid = (unsigned) ((threads + kThreads - 1) / kThreads);
  csr_subwarp_kernel<T, G><<<grid, kThreads, 0, s>>> (n, rp, c, v, x, y);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

template <typename T>
int launch_csr (int n, int g, const int *rp, const int *c, const T *v, const T *x, T *y,
                cudaStream_t s)
{
  switch (g)
    {
    case 1: return launch_csr_g<T, 1> (n, rp, c, v, x, y, s);
    case 2: return launch_csr_g<T, 2> (n, rp, c, v, x, y, s);
    case 4: return launch_csr_g<T, 4> (n, rp, c, v, x, y, s);
    case 8: return launch_csr_g<T, 8> (n, rp, c, v, x, y, s);
    case 16: return launch_csr_g<T, 16> (n, rp, c, v, x, y, s);
    case 32: return launch_csr_g<T, 32> (n, rp, c, v, x, y, s);
    default: return fail (BMFP_ERROR_INVALID_VALUE, "invalid lane count %d", g);
    }
}

inline int csr_default_lanes (double avg_nnz_per_row)
{
  int g = 1;
  while (g < 32 && g < avg_nnz_per_row)
    g <<= 1;
  return g;
}

template <typename T>
int native_bcsr_typed (int nbr, int bs, int64_t nnzb, const int *rp, const int *c, const T *v,
                       const T *x, T *y, int lanes, cudaStream_t s)
{
  const double avg = nbr > 0 ? (double) nnzb / nbr : 0.0;
  const int dtype = sizeof (T) == 8 ? BMFP_R64F : BMFP_R32F;
  if (bs == 1)
    return launch_csr<T> (nbr, lanes ? lanes : native_default_lanes (dtype, 1, avg), rp, c, v, x, y, s);
  if (lanes == 0 && flat_bs (bs))
    {
      lanes = native_default_lanes (dtype, bs, avg);
      const bool ok = (reinterpret_cast<uintptr_t> (v) | reinterpret_cast<uintptr_t> (x)) % 16 == 0;
      if (lanes == BMFP_LANES_ROW_OWNER && (!ok || bs < 4))
        lanes = 0; // misaligned views: the scalar-load kernel below
    }
  if (lanes == BMFP_LANES_ROW_OWNER)
    {
      const bool ok = (reinterpret_cast<uintptr_t> (v) | reinterpret_cast<uintptr_t> (x)) % 16 == 0;
      if (!ok || !(bs == 4 || bs == 8 || bs == 16 || bs == 32))
        return fail (BMFP_ERROR_INVALID_VALUE, "row-owner mapping needs bs in {4,8,16,32} and aligned arrays");
      const int64_t threads = (int64_t) nbr * bs;
      const unsigned grid = (unsigned) ((threads + kThreads - 1) / kThreads);
      switch (bs)
        {
        case 4: bcsr_rowown_kernel<T, 4><<<grid, kThreads, 0, s>>> (nbr, rp, c, v, x, y); break;
        case 8: bcsr_rowown_kernel<T, 8><<<grid, kThreads, 0, s>>> (nbr, rp, c, v, x, y); break;
        case 16: bcsr_rowown_kernel<T, 16><<<grid, kThreads, 0, s>>> (nbr, rp, c, v, x, y); break;
        default: bcsr_rowown_kernel<T, 32><<<grid, kThreads, 0, s>>> (nbr, rp, c, v, x, y); break;
        }
      BMFP_LAUNCH_CHECK ();
      return BMFP_SUCCESS;
    }
  // The flat kernel issues 16-byte vector loads of values and x: it needs
  // both base pointers 16-byte aligned (cudaMalloc gives 256). Misaligned
  // views fall through to the scalar-load kernel below.
  const bool aligned = ((reinterpret_cast<uintptr_t> (v) | reinterpret_cast<uintptr_t> (x)) & 15u) == 0;
  if (flat_bs (bs) && aligned)
    {
      const int g = lanes ? lanes : native_default_lanes (dtype, bs, avg);
      if (!flat_lanes_ok (dtype, bs, g))
        return fail (BMFP_ERROR_INVALID_VALUE, "lane count %d not valid for bs=%d", g, bs);
      switch (bs)
        {
        case 2: return launch_flat<T, 2> (nbr, g, rp, c, v, x, y, s);
        case 4: return launch_flat<T, 4> (nbr, g, rp, c, v, x, y, s);
        case 8: return launch_flat<T, 8> (nbr, g, rp, c, v, x, y, s);
        case 16: return launch_flat<T, 16> (nbr, g, rp, c, v, x, y, s);
        default: return launch_flat<T, 32> (nbr, g, rp, c, v, x, y, s);
        }
    }
  if (bs <= 32)
    {
      const int64_t threads = (int64_t) nbr * 32;
      const unsigned grid = (unsigned) ((threads + kThreads - 1) / kThreads);
      if (bs == 3)
        bcsr_tpr_kernel<T, 3><<<grid, kThreads, 0, s>>> (nbr, bs, rp, c, v, x, y);
      else
        bcsr_tpr_kernel<T, 0><<<grid, kThreads, 0, s>>> (nbr, bs, rp, c, v, x, y);
      BMFP_LAUNCH_CHECK ();
      return BMFP_SUCCESS;
    }
  const int64_t threads = (int64_t) nbr * bs;
  const unsigned grid = (unsigned) ((threads + kThreads - 1) / kThreads);
  bcsr_row_kernel<T><<<grid, kThreads, 0, s>>> (nbr, bs, rp, c, v, x, y);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}
} // namespace

int native_default_lanes (int dtype, int bs, double avg_blocks_per_row)
{
  if (bs == 1)
    {
      // A few lanes per CSR row: the autotuner picked 1-2 on GB300 for eight
      // entries per row.
      int g = 1;
      while (g < 32 && 4 * g < avg_blocks_per_row)
        g <<= 1;
      return g;
    }
  if (!flat_bs (bs))
    return 32;
  // The choices bmfp_matrix_autotune made on GB300 for the block-size sweep
  // (100 000 block rows, 8 blocks per row). FP64 is bound by GB300's narrow
  // FP64 pipe, where a warp instruction costs the same however many lanes are
  // active, so from bs 8 on one lane owns one scalar row (no shuffle adds).
  if (dtype == BMFP_R64F)
    {
      switch (bs)
        {
        case 2:
          // Two lanes own one scalar row each (no shuffle add); four lanes
          // cover two blocks per step and tie only on rows of a multiple of
          // eight blocks (the sweep's 8: 4 lanes picked; the bridge's 5
          // blocks 18.2 vs 22.1 us, Q4 1000x250's 9 blocks 29.5 vs 32.6 us
          // with 2 lanes).
          return avg_blocks_per_row >= 7.5 && avg_blocks_per_row <= 8.5 ? 4 : 2;
        case 4: return 4;
        default: return BMFP_LANES_ROW_OWNER;
        }
    }
  switch (bs)
    {
    case 2: return 2;
    case 4: return BMFP_LANES_ROW_OWNER;
    case 8: return 8;
    default: return 32;
    }
}

int native_lane_candidates (int dtype, int bs, int *out, int max_out)
{
  int n = 0;
  if (bs == 1)
    {
      for (int g = 1; g <= 32 && n < max_out; g <<= 1)
        out[n++] = g;
      return n;
    }
  if (!flat_bs (bs))
    return 0;
  for (int g = 2; g <= 32 && n < max_out; g <<= 1)
    if (flat_lanes_ok (dtype, bs, g))
      out[n++] = g;
  if (bs >= 4 && n < max_out)
    out[n++] = BMFP_LANES_ROW_OWNER;
  return n;
}

int spmv_native_bcsr (int dtype, int nbr, int bs, int64_t nnzb, const int *row_ptr,
                      const int *cols, const void *vals, const void *x, void *y, int lanes,
                      cudaStream_t stream)
{
  if (nbr == 0)
    return BMFP_SUCCESS;
  if (dtype == BMFP_R64F)
    return native_bcsr_typed<double> (nbr, bs, nnzb, row_ptr, cols, (const double *) vals,
                                      (const double *) x, (double *) y, lanes, stream);
  return native_bcsr_typed<float> (nbr, bs, nnzb, row_ptr, cols, (const float *) vals,
                                   (const float *) x, (float *) y, lanes, stream);
}

int spmv_native_bcsr_colmajor (int dtype, int nbr, int bs, const int *rp, const int *c, const void *vals_cm,
                               const void *x, void *y, cudaStream_t s)
{
  if (nbr == 0)
    return BMFP_SUCCESS;
  if (!(bs == 2 || bs == 4 || bs == 8 || bs == 16 || bs == 32))
    return fail (BMFP_ERROR_INVALID_VALUE, "column-owner mapping needs bs in {2,4,8,16,32}");
  const int64_t threads = (int64_t) nbr * bs;
  const unsigned grid = (unsigned) ((threads + kThreads - 1) / kThreads);
#define BMFP_COL(T, B)                                                                                              \
  case B:                                                                                                            \
    bcsr_colown_kernel<T, B><<<grid, kThreads, 0, s>>> (nbr, rp, c, (const T *) vals_cm, (const T *) x, (T *) y); \
    break;
  if (dtype == BMFP_R64F)
    switch (bs)
      {
        BMFP_COL (double, 2) BMFP_COL (double, 4) BMFP_COL (double, 8) BMFP_COL (double, 16) BMFP_COL (double, 32)
      }
  else
    switch (bs)
      {
        BMFP_COL (float, 2) BMFP_COL (float, 4) BMFP_COL (float, 8) BMFP_COL (float, 16) BMFP_COL (float, 32)
      }
#undef BMFP_COL
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int transpose_blocks_device (int dtype, int64_t nnzb, int bs, const void *in, void *out, cudaStream_t s)
{
  const int64_t total = nnzb * bs * bs;
  if (total == 0)
    return BMFP_SUCCESS;
  const unsigned grid = (unsigned) std::min<int64_t> ((total + kThreads - 1) / kThreads, 152 * 32);
  if (dtype == BMFP_R64F)
    transpose_blocks_kernel<double><<<grid, kThreads, 0, s>>> (total, bs, (const double *) in, (double *) out);
  else
    transpose_blocks_kernel<float><<<grid, kThreads, 0, s>>> (total, bs, (const float *) in, (float *) out);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int spmv_native_csr (int dtype, int n_rows, int64_t nnz, const int *row_ptr, const int *cols,
                     const void *vals, const void *x, void *y, int lanes, cudaStream_t stream)
{
  if (n_rows == 0)
    return BMFP_SUCCESS;
  const int g = lanes ? lanes : csr_default_lanes (n_rows ? (double) nnz / n_rows : 0.0);
  if (dtype == BMFP_R64F)
    return launch_csr<double> (n_rows, g, row_ptr, cols, (const double *) vals,
                               (const double *) x, (double *) y, stream);
  return launch_csr<float> (n_rows, g, row_ptr, cols, (const float *) vals, (const float *) x,
                            (float *) y, stream);
}
} // namespace bmfp
