// Arithmetic peak and size-matched read floor of the current device, for
// roofline reporting.
//
// GB300's FP64 FMA rate (about 1.25 TFLOP/s, 1/58 of FP32) bounds every FP64
// sparse product below the HBM roofline: at one FMA per 8-byte value an FP64
// SpMV cannot stream faster than 4 bytes per FP64 flop. bmfp_measure_fma_peak
// measures that rate where the products run, so reports can state both
// bounds. Eight independent FMA chains per thread over a grid of 8 CTAs per
// SM keep every pipe busy; the result is stored so nothing is optimised away.
//
// bmfp_stream_read is the third bound, for small products: a plain streaming
// read of the same number of bytes. Launch ramp, the first DRAM round trips
// and the tail take a few microseconds whatever a kernel does, so a 58 MB
// read after an L2 flush reaches only about 60 % of the copy peak on GB300;
// timing this read beside a product the same way shows how much of a small
// product's time any kernel would spend.
#include "internal.h"

namespace bmfp
{
namespace
{
template <typename T>
__global__ void __launch_bounds__ (256) fma_chains_kernel (T *out, int iters, T a, T b)
{
  T c[8];
#pragma unroll
  for (int k = 0; k < 8; k++)
    c[k] = (T) (threadIdx.x + k);
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++)
      c[k] = fma (c[k], a, b);
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++)
    s += c[k];
  out[(size_t) blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T> int measure (int iters, double *gflops, cudaStream_t s)
{
  int dev = 0, sms = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  BMFP_CUDA (cudaDeviceGetAttribute (&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256;
  T *out = nullptr;
  BMFP_CUDA (cudaMallocAsync (&out, sizeof (T) * (size_t) blocks * threads, s));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate (&e0);
  if (e == cudaSuccess)
    e = cudaEventCreate (&e1);
  float best = 0.0f;
  for (int r = 0; r < 5 && e == cudaSuccess; r++)
    {
      e = cudaEventRecord (e0, s);
      fma_chains_kernel<T><<<blocks, threads, 0, s>>> (out, iters, (T) 0.999, (T) 0.001);
      if (e == cudaSuccess)
        e = cudaGetLastError ();
      if (e == cudaSuccess)
        e = cudaEventRecord (e1, s);
      if (e == cudaSuccess)
        e = cudaEventSynchronize (e1);
      float ms = 0.0f;
      if (e == cudaSuccess)
        e = cudaEventElapsedTime (&ms, e0, e1);
      if (e == cudaSuccess && r >= 2 && (best == 0.0f || ms < best))
        best = ms; // the first two launches warm the clocks up
    }
  cudaFreeAsync (out, s);
  cudaStreamSynchronize (s);
  if (e0)
    cudaEventDestroy (e0);
  if (e1)
    cudaEventDestroy (e1);
  if (e != cudaSuccess)
    return cuda_fail (e, "FMA peak probe", __FILE__, __LINE__);
  *gflops = 2.0 * 8.0 * (double) iters * blocks * threads / (best * 1e-3) / 1e9;
  return BMFP_SUCCESS;
}
// Sink for the read kernel: the sum is stored only if it equals a value no
// finite input reaches in practice, so the loads cannot be elided.
__device__ float g_read_sink;

__global__ void __launch_bounds__ (256) stream_read_kernel (const float4 *__restrict__ p, int64_t n)
{
  float s = 0.0f;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    {
      const float4 v = __ldcs (p + i);
      s += (v.x + v.y) + (v.z + v.w);
    }
  if (s == 1.0e30f)
    g_read_sink = s;
}
} // namespace
} // namespace bmfp

extern "C" int bmfp_measure_fma_peak (int dtype, double *gflops, void *stream)
{
  using namespace bmfp;
  if (!gflops || !dtype_ok (dtype))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  cudaStream_t s = as_stream (stream);
  return dtype == BMFP_R64F ? measure<double> (2048, gflops, s) : measure<float> (16384, gflops, s);
}

extern "C" int bmfp_stream_read (const void *d_buf, size_t bytes, void *stream)
{
  using namespace bmfp;
  if (!d_buf || (reinterpret_cast<uintptr_t> (d_buf) & 15u) != 0 || bytes % 16 != 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "stream_read needs a 16-byte aligned buffer and a multiple of 16 bytes");
  if (bytes == 0)
    return BMFP_SUCCESS;
  int dev = 0, sms = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  BMFP_CUDA (cudaDeviceGetAttribute (&sms, cudaDevAttrMultiProcessorCount, dev));
  // 8 CTAs of 256 threads per SM, one 16-byte load per step: the fastest of
  // the shapes measured for 8-430 MB reads (4 or 8 CTAs per SM, 1 or 4 loads
  // in flight per thread, one element per thread).
  stream_read_kernel<<<(unsigned) sms * 8, 256, 0, as_stream (stream)>>> (static_cast<const float4 *> (d_buf),
                                                                         (int64_t) (bytes / 16));
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}
