// Device-side helpers: 16-byte vector loads with cache hints, group-wide
// shuffles. Everything here is header-only and inlined into the kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace bmfp
{
namespace dev
{
// One 16-byte vector of T: 2 doubles or 4 floats.
template <typename T> struct Vec16;
template <> struct Vec16<double>
{
  static constexpr int N = 2;
  double v[2];
};
template <> struct Vec16<float>
{
  static constexpr int N = 4;
  float v[4];
};

// Matrix values are read exactly once per product: load them with the
// evict-first (streaming) hint so they do not push x out of L1/L2.
__device__ __forceinline__ Vec16<double> ld_stream16 (const double *p)
{
  double2 t = __ldcs (reinterpret_cast<const double2 *> (p));
  return Vec16<double>{ { t.x, t.y } };
}
__device__ __forceinline__ Vec16<float> ld_stream16 (const float *p)
{
  float4 t = __ldcs (reinterpret_cast<const float4 *> (p));
  return Vec16<float>{ { t.x, t.y, t.z, t.w } };
}

// x is reused by neighbouring block rows: read it through the read-only path.
__device__ __forceinline__ Vec16<double> ld_cached16 (const double *p)
{
  double2 t = __ldg (reinterpret_cast<const double2 *> (p));
  return Vec16<double>{ { t.x, t.y } };
}
__device__ __forceinline__ Vec16<float> ld_cached16 (const float *p)
{
  float4 t = __ldg (reinterpret_cast<const float4 *> (p));
  return Vec16<float>{ { t.x, t.y, t.z, t.w } };
}

// Two consecutive elements (8-byte aligned for float, 16 for double).
__device__ __forceinline__ void ld_cached2 (const float *p, float &a, float &b)
{
  float2 t = __ldg (reinterpret_cast<const float2 *> (p));
  a = t.x;
  b = t.y;
}
__device__ __forceinline__ void ld_cached2 (const double *p, double &a, double &b)
{
  double2 t = __ldg (reinterpret_cast<const double2 *> (p));
  a = t.x;
  b = t.y;
}

template <typename T> __device__ __forceinline__ T ld_stream (const T *p) { return __ldcs (p); }
template <typename T> __device__ __forceinline__ T ld_cached (const T *p) { return __ldg (p); }

// How the row routines load the vector they multiply.
// XNc: the read-only path, for a vector no thread of the running kernel writes.
struct XNc
{
  template <typename T> __device__ static __forceinline__ Vec16<T> ld16 (const T *p) { return ld_cached16 (p); }
  template <typename T> __device__ static __forceinline__ void ld2 (const T *p, T &a, T &b) { ld_cached2 (p, a, b); }
  template <typename T> __device__ static __forceinline__ T ld (const T *p) { return __ldg (p); }
};

// XCoh: plain (weak, L1-cached) global loads, for a vector that other CTAs of
// the same persistent kernel wrote before a grid barrier. The barrier's
// release/acquire pair orders those writes before these loads; the
// read-only path has no such guarantee for data written during the kernel.
// volatile keeps the compiler from merging or moving the loads across the
// barrier between two iterations.
struct XCoh
{
  __device__ static __forceinline__ Vec16<double> ld16 (const double *p)
  {
    Vec16<double> r;
    asm volatile ("ld.global.v2.f64 {%0, %1}, [%2];" : "=d"(r.v[0]), "=d"(r.v[1]) : "l"(p));
    return r;
  }
  __device__ static __forceinline__ Vec16<float> ld16 (const float *p)
  {
    Vec16<float> r;
    asm volatile ("ld.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                  : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3])
                  : "l"(p));
    return r;
  }
  __device__ static __forceinline__ void ld2 (const double *p, double &a, double &b)
  {
    asm volatile ("ld.global.v2.f64 {%0, %1}, [%2];" : "=d"(a), "=d"(b) : "l"(p));
  }
  __device__ static __forceinline__ void ld2 (const float *p, float &a, float &b)
  {
    asm volatile ("ld.global.v2.f32 {%0, %1}, [%2];" : "=f"(a), "=f"(b) : "l"(p));
  }
  __device__ static __forceinline__ double ld (const double *p)
  {
    double r;
    asm volatile ("ld.global.f64 %0, [%1];" : "=d"(r) : "l"(p));
    return r;
  }
  __device__ static __forceinline__ float ld (const float *p)
  {
    float r;
    asm volatile ("ld.global.f32 %0, [%1];" : "=f"(r) : "l"(p));
    return r;
  }
};

// Lane mask of the aligned group of G lanes that contains this lane.
template <int G> __device__ __forceinline__ unsigned group_mask ()
{
  if constexpr (G >= 32)
    return 0xffffffffu;
  else
    {
      const unsigned lane = threadIdx.x & 31u;
      return ((1u << G) - 1u) << (lane & ~(unsigned) (G - 1));
    }
}

template <typename T> __device__ __forceinline__ T shfl_xor (unsigned mask, T v, int off)
{
  return __shfl_xor_sync (mask, v, off);
}

// Sum over all lanes of an aligned G-lane group (butterfly; every lane ends
// with the total, so the result does not depend on which lane reads it).
template <int G, typename T> __device__ __forceinline__ T group_sum (T v)
{
  const unsigned m = group_mask<G> ();
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1)
    v += __shfl_xor_sync (m, v, off);
  return v;
}
} // namespace dev
} // namespace bmfp
