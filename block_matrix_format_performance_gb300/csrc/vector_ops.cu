// Elementwise device helpers shared by the matrix handles and solvers.
#include "internal.h"

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
} // namespace

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
