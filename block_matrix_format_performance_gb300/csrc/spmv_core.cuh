// Row-level SpMV device routines shared by the standalone SpMV kernels and
// the solver's fused SpMV + dot-product phases.
//
// Each routine computes the outputs of one block row with an aligned group of
// lanes, stores them to y and hands every stored (index, value) pair to an
// epilogue functor (a no-op for plain SpMV; dot-product accumulators inside
// the solver). The mapping is explained in spmv_native.cu.
#pragma once

#include "device_common.cuh"

namespace bmfp
{
namespace core
{
struct NoEpilogue
{
  template <typename T> __device__ __forceinline__ void operator() (int64_t, T) {}
};

inline constexpr bool flat_block_size (int bs) { return bs == 2 || bs == 4 || bs == 8 || bs == 16 || bs == 32; }

// One block row by an aligned group of G lanes, 16-byte vector loads.
// Requires bs in {2,4,8,16,32}, G*V >= bs and 16-byte aligned vals and x.
template <typename T, int BS, int G, int U, class XL = dev::XNc, class Epi>
__device__ __forceinline__ void flat_row (int row, const int *__restrict__ row_ptr,
                                          const int *__restrict__ cols, const T *__restrict__ vals,
                                          const T *__restrict__ x, T *__restrict__ y, Epi &epi)
{
  using V16 = dev::Vec16<T>;
  constexpr int V = V16::N;
  constexpr int E = BS * BS;
  constexpr int CH = G * V;
  static_assert (E % V == 0, "a block must be a whole number of 16-byte vectors");
  static_assert (CH >= BS, "a group chunk must cover at least one block line");
  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = dev::group_mask<G> ();
  const int beg = __ldg (row_ptr + row);
  const int nblk = __ldg (row_ptr + row + 1) - beg;
  const T *vb = vals + (size_t) beg * E;
  const int *cb = cols + beg;

  if constexpr (CH >= E)
    {
      // Whole groups of U chunks first, with no predicates, then one chunk at
      // a time for the rest: a row of 9 blocks costs 9 block steps rather
      // than 12 (every warp-wide FP64 instruction is paid in full on GB300,
      // active lanes or not). The per-lane accumulation order is the block
      // order either way.
      constexpr int BPI = CH / E;
      const int bl = (gl * V) / E;
      const int o = (gl * V) % E;
      int b0 = 0;
      if constexpr (V <= BS)
        {
          const int c0 = o % BS;
          T acc = 0;
          for (; b0 + BPI * U <= nblk; b0 += BPI * U)
            {
              V16 a[U];
              int c[U];
#pragma unroll
              for (int u = 0; u < U; u++)
                {
                  const int b = b0 + u * BPI + bl;
                  a[u] = dev::ld_stream16 (vb + b * E + o);
                  c[u] = __ldg (cb + b);
                }
#pragma unroll
              for (int u = 0; u < U; u++)
                {
                  const V16 xv = XL::ld16 (x + (size_t) c[u] * BS + c0);
#pragma unroll
                  for (int v = 0; v < V; v++)
                    acc = fma (a[u].v[v], xv.v[v], acc);
                }
            }
          for (; b0 < nblk; b0 += BPI)
            {
              const int b = b0 + bl;
              if (b < nblk)
                {
                  const V16 av = dev::ld_stream16 (vb + b * E + o);
                  const V16 xv = XL::ld16 (x + (size_t) __ldg (cb + b) * BS + c0);
#pragma unroll
                  for (int v = 0; v < V; v++)
                    acc = fma (av.v[v], xv.v[v], acc);
                }
            }
#pragma unroll
          for (int off = 1; off < BS / V; off <<= 1)
            acc += __shfl_xor_sync (mask, acc, off);
#pragma unroll
          for (int off = E / V; off < G; off <<= 1)
            acc += __shfl_xor_sync (mask, acc, off);
          if (gl < E / V && (gl % (BS / V)) == 0)
            {
              const int64_t i = (int64_t) row * BS + gl / (BS / V);
              y[i] = acc;
              epi (i, acc);
            }
        }
      else
        {
          static_assert (V == E, "unexpected vector/block shape");
          T acc0 = 0, acc1 = 0;
          for (; b0 + BPI * U <= nblk; b0 += BPI * U)
            {
              V16 a[U];
              int c[U];
#pragma unroll
              for (int u = 0; u < U; u++)
                {
                  const int b = b0 + u * BPI + bl;
                  a[u] = dev::ld_stream16 (vb + b * E);
                  c[u] = __ldg (cb + b);
                }
#pragma unroll
              for (int u = 0; u < U; u++)
                {
                  T x0, x1;
                  XL::ld2 (x + (size_t) c[u] * 2, x0, x1);
                  acc0 = fma (a[u].v[0], x0, acc0);
                  acc0 = fma (a[u].v[1], x1, acc0);
                  acc1 = fma (a[u].v[2], x0, acc1);
                  acc1 = fma (a[u].v[3], x1, acc1);
                }
            }
          for (; b0 < nblk; b0 += BPI)
            {
              const int b = b0 + bl;
              if (b < nblk)
                {
                  const V16 av = dev::ld_stream16 (vb + b * E);
                  T x0, x1;
                  XL::ld2 (x + (size_t) __ldg (cb + b) * 2, x0, x1);
                  acc0 = fma (av.v[0], x0, acc0);
                  acc0 = fma (av.v[1], x1, acc0);
                  acc1 = fma (av.v[2], x0, acc1);
                  acc1 = fma (av.v[3], x1, acc1);
                }
            }
          acc0 = dev::group_sum<G> (acc0);
          acc1 = dev::group_sum<G> (acc1);
          if (gl == 0)
            {
              const int64_t i = (int64_t) row * 2;
              y[i] = acc0;
              y[i + 1] = acc1;
              epi (i, acc0);
              epi (i + 1, acc1);
            }
        }
    }
  else
    {
      constexpr int NP = E / CH;
      constexpr int RPP = CH / BS;
      const int c0 = (gl * V) % BS;
      const int rl = (gl * V) / BS;
      T acc[NP];
#pragma unroll
      for (int p = 0; p < NP; p++)
        acc[p] = 0;
#pragma unroll 2
      for (int b = 0; b < nblk; b++)
        {
          const T *blk = vb + b * E + gl * V;
          V16 a[NP];
#pragma unroll
          for (int p = 0; p < NP; p++)
            a[p] = dev::ld_stream16 (blk + p * CH);
          const int c = __ldg (cb + b);
          const V16 xv = XL::ld16 (x + (size_t) c * BS + c0);
#pragma unroll
          for (int p = 0; p < NP; p++)
#pragma unroll
            for (int v = 0; v < V; v++)
              acc[p] = fma (a[p].v[v], xv.v[v], acc[p]);
        }
#pragma unroll
      for (int p = 0; p < NP; p++)
#pragma unroll
        for (int off = 1; off < BS / V; off <<= 1)
          acc[p] += __shfl_xor_sync (mask, acc[p], off);
      if ((gl % (BS / V)) == 0)
#pragma unroll
        for (int p = 0; p < NP; p++)
          {
            const int64_t i = (int64_t) row * BS + p * RPP + rl;
            y[i] = acc[p];
            epi (i, acc[p]);
          }
    }
}

// One block row by BS lanes, lane r owning scalar row r: it streams row r of
// every block (BS/V 16-byte vectors, read through L1 so the two halves of a
// sector meet there) against the block's x segment (the same addresses in
// every lane of the group). Each lane finishes its own row: no cross-lane
// reduction, so every FP64 instruction is a useful FMA — what GB300's narrow
// FP64 pipe needs. Requires bs a multiple of V and 16-byte aligned values/x.
template <typename T, int BS, class Epi>
__device__ __forceinline__ void rowown_row (int row, const int *__restrict__ row_ptr,
                                            const int *__restrict__ cols, const T *__restrict__ vals,
                                            const T *__restrict__ x, T *__restrict__ y, Epi &epi)
{
  using V16 = dev::Vec16<T>;
  constexpr int V = V16::N;
  constexpr int NV = BS / V; // vectors per block line
  static_assert (BS % V == 0, "block line must be whole 16-byte vectors");
  const int r = threadIdx.x & (BS - 1);
  const int beg = __ldg (row_ptr + row);
  const int end = __ldg (row_ptr + row + 1);
  T acc0 = 0, acc1 = 0;
  for (int b = beg; b < end; b++)
    {
      const T *line = vals + (size_t) b * BS * BS + (size_t) r * BS;
      const T *xs = x + (size_t) __ldg (cols + b) * BS;
      V16 a[NV];
#pragma unroll
      for (int k = 0; k < NV; k++)
        a[k] = dev::ld_cached16 (line + k * V);
#pragma unroll
      for (int k = 0; k < NV; k++)
        {
          const V16 xv = dev::ld_cached16 (xs + k * V);
#pragma unroll
          for (int v = 0; v < V; v++)
            {
              if ((k * V + v) & 1)
                acc1 = fma (a[k].v[v], xv.v[v], acc1);
              else
                acc0 = fma (a[k].v[v], xv.v[v], acc0);
            }
        }
    }
  const T acc = acc0 + acc1;
  const int64_t i = (int64_t) row * BS + r;
  y[i] = acc;
  epi (i, acc);
}

// One block row by a whole warp, lane (q, r) = (lane / bs, lane % bs), any
// bs <= 32; scalar loads (no alignment requirement).
template <typename T, int BSC, class XL = dev::XNc, class Epi>
__device__ __forceinline__ void tpr_row (int row, int bs_rt, const int *__restrict__ row_ptr,
                                         const int *__restrict__ cols, const T *__restrict__ vals,
                                         const T *__restrict__ x, T *__restrict__ y, Epi &epi)
{
  const int bs = BSC ? BSC : bs_rt;
  const int Q = 32 / bs;
  const int lane = threadIdx.x & 31;
  const int q = lane / bs, r = lane % bs;
  const bool live = q < Q;
  const int beg = __ldg (row_ptr + row), end = __ldg (row_ptr + row + 1);
  T acc = 0;
  if (live)
    for (int b = beg + q; b < end; b += Q)
      {
        const T *a = vals + (size_t) b * bs * bs + r * bs;
        const T *xb = x + (size_t) __ldg (cols + b) * bs;
        for (int c = 0; c < bs; c++)
          acc = fma (dev::ld_stream (a + c), XL::ld (xb + c), acc);
      }
  int top = 1;
  while (top < Q)
    top <<= 1;
  for (int s = top >> 1; s > 0; s >>= 1)
    {
      const T other = __shfl_down_sync (0xffffffffu, acc, s * bs);
      if (live && q + s < Q)
        acc += other;
    }
  if (q == 0)
    {
      const int64_t i = (int64_t) row * bs + r;
      y[i] = acc;
      epi (i, acc);
    }
}

// One CSR row (bs = 1) by an aligned group of G lanes strided over its entries.
template <typename T, int G, class XL = dev::XNc, class Epi>
__device__ __forceinline__ void csr_row (int row, const int *__restrict__ row_ptr,
                                         const int *__restrict__ cols, const T *__restrict__ vals,
                                         const T *__restrict__ x, T *__restrict__ y, Epi &epi)
{
  const int gl = threadIdx.x & (G - 1);
  const int beg = __ldg (row_ptr + row), end = __ldg (row_ptr + row + 1);
  T acc0 = 0, acc1 = 0;
  int e = beg + gl;
  for (; e + G < end; e += 2 * G)
    {
      const T a0 = dev::ld_stream (vals + e), a1 = dev::ld_stream (vals + e + G);
      const int c0 = __ldg (cols + e), c1 = __ldg (cols + e + G);
      acc0 = fma (a0, XL::ld (x + c0), acc0);
      acc1 = fma (a1, XL::ld (x + c1), acc1);
    }
  if (e < end)
    acc0 = fma (dev::ld_stream (vals + e), XL::ld (x + __ldg (cols + e)), acc0);
  const T acc = dev::group_sum<G> (acc0 + acc1);
  if (gl == 0)
    {
      y[row] = acc;
      epi ((int64_t) row, acc);
    }
}
} // namespace core
} // namespace bmfp
