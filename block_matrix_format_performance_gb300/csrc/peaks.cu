// Arithmetic peak of the current device, for roofline reporting.
//
// GB300's FP64 FMA rate (about 1.25 TFLOP/s, 1/58 of FP32) bounds every FP64
// sparse product below the HBM roofline: at one FMA per 8-byte value an FP64
// SpMV cannot stream faster than 4 bytes per FP64 flop. bmfp_measure_fma_peak
// measures that rate where the products run, so reports can state both
// bounds. Eight independent FMA chains per thread over a grid of 8 CTAs per
// SM keep every pipe busy; the result is stored so nothing is optimised away.
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
