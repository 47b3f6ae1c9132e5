// Elementwise device helpers shared by the matrix handles and solvers.
#include "internal.h"
#include "solver.h"

namespace bmfp
{
namespace
{
template <typename S, typename D>
__global__ void convert_kernel (int64_t n, const S *__restrict__ src, D *__restrict__ dst)
{
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    dst[i] = (D) src[i];
}

unsigned grid_for (int64_t n)
{
  int64_t g = (n + 255) / 256;
  if (g > 152 * 32)
    g = 152 * 32;
  return (unsigned) (g > 0 ? g : 1);
}
// Reads a scratch buffer larger than L2 so the next kernel finds none of its
// data there; the sum is stored only under a condition the caller makes
// impossible (sink_if == -1), so the reads cannot be optimised away.
__global__ void l2_flush_kernel (const int4 *__restrict__ p, int64_t n, int sink_if, int *__restrict__ sink)
{
  int acc = 0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    {
      const int4 v = p[i]; // default (evict-normal) policy: these lines displace the others
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  if (acc == sink_if)
    *sink = acc;
}

template <typename S, typename D>
__global__ void axpy_convert_kernel (int64_t n, double a, const S *__restrict__ src, D *__restrict__ dst)
{
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    dst[i] = (D) ((double) dst[i] + a * (double) src[i]);
}

template <typename S, typename D>
__global__ void scale_convert_kernel (int64_t n, double a, const S *__restrict__ src, D *__restrict__ dst)
{
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    dst[i] = (D) (a * (double) src[i]);
}

} // namespace

// dst += a * src, with element types converted through double.
int axpy_scaled_convert (int dst_dtype, int src_dtype, int64_t n, double a, const void *src,
                         void *dst, cudaStream_t stream)
{
  if (n == 0)
    return BMFP_SUCCESS;
  const unsigned g = grid_for (n);
  if (dst_dtype == BMFP_R64F && src_dtype == BMFP_R32F)
    axpy_convert_kernel<float, double><<<g, 256, 0, stream>>> (n, a, (const float *) src, (double *) dst);
  else if (dst_dtype == BMFP_R64F)
    axpy_convert_kernel<double, double><<<g, 256, 0, stream>>> (n, a, (const double *) src, (double *) dst);
  else if (src_dtype == BMFP_R32F)
    axpy_convert_kernel<float, float><<<g, 256, 0, stream>>> (n, a, (const float *) src, (float *) dst);
  else
    axpy_convert_kernel<double, float><<<g, 256, 0, stream>>> (n, a, (const double *) src, (float *) dst);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

// dst = a * src, with element types converted through double.
int scale_convert (int dst_dtype, int src_dtype, int64_t n, double a, const void *src, void *dst,
                   cudaStream_t stream)
{
  if (n == 0)
    return BMFP_SUCCESS;
  const unsigned g = grid_for (n);
  if (dst_dtype == BMFP_R32F && src_dtype == BMFP_R64F)
    scale_convert_kernel<double, float><<<g, 256, 0, stream>>> (n, a, (const double *) src, (float *) dst);
  else if (dst_dtype == BMFP_R32F)
    scale_convert_kernel<float, float><<<g, 256, 0, stream>>> (n, a, (const float *) src, (float *) dst);
  else if (src_dtype == BMFP_R64F)
    scale_convert_kernel<double, double><<<g, 256, 0, stream>>> (n, a, (const double *) src, (double *) dst);
  else
    scale_convert_kernel<float, double><<<g, 256, 0, stream>>> (n, a, (const float *) src, (double *) dst);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

// Element type conversion on the device (FP64 -> FP32 rounds to nearest).
int l2_flush (const void *scratch, size_t bytes, int *sink, cudaStream_t s)
{
  const int64_t n = (int64_t) (bytes / 16);
  if (n == 0)
    return BMFP_SUCCESS;
  l2_flush_kernel<<<grid_for (n), 256, 0, s>>> ((const int4 *) scratch, n, -1, sink);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int convert_values (int src_dtype, int dst_dtype, int64_t n, const void *src, void *dst,
                    cudaStream_t stream)
{
  if (n == 0)
    return BMFP_SUCCESS;
  if (src_dtype == dst_dtype)
    {
      BMFP_CUDA (cudaMemcpyAsync (dst, src, (size_t) n * dtype_size (src_dtype),
                                  cudaMemcpyDeviceToDevice, stream));
      return BMFP_SUCCESS;
    }
  if (src_dtype == BMFP_R64F)
    convert_kernel<double, float><<<grid_for (n), 256, 0, stream>>> (n, (const double *) src, (float *) dst);
  else
    convert_kernel<float, double><<<grid_for (n), 256, 0, stream>>> (n, (const float *) src, (double *) dst);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}
} // namespace bmfp
