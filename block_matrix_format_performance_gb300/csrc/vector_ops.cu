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
