// cuSPARSE bsrmv comparison variants ("GPU BSR (cuSPARSE, row major |
// column major)", gpu/gpu_matrix_multiplier.cu:676-734, 862-957). A closed
// NVIDIA library call kept only as the reference's own comparison point; it is
// never the library's product path.
#define DISABLE_CUSPARSE_DEPRECATED
#include "internal.h"

#include <cusparse.h>

namespace bmfp
{
namespace
{
struct CusparseState
{
  cusparseHandle_t handle = nullptr;
  cusparseMatDescr_t descr = nullptr;
  int device = -1;
};

// One handle per host thread, created on first use and deliberately never
// destroyed: a destructor at thread or process exit could run after the CUDA
// context is gone.
thread_local CusparseState g_cusparse;

int ensure_handle ()
{
  int dev = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  if (g_cusparse.handle && g_cusparse.device == dev)
    return BMFP_SUCCESS;
  if (g_cusparse.descr)
    cusparseDestroyMatDescr (g_cusparse.descr);
  if (g_cusparse.handle)
    cusparseDestroy (g_cusparse.handle);
  g_cusparse.handle = nullptr;
  g_cusparse.descr = nullptr;
  if (cusparseCreate (&g_cusparse.handle) != CUSPARSE_STATUS_SUCCESS)
    return fail (BMFP_ERROR_CUDA, "cusparseCreate failed");
  if (cusparseCreateMatDescr (&g_cusparse.descr) != CUSPARSE_STATUS_SUCCESS)
    return fail (BMFP_ERROR_CUDA, "cusparseCreateMatDescr failed");
  cusparseSetMatType (g_cusparse.descr, CUSPARSE_MATRIX_TYPE_GENERAL);
  cusparseSetMatIndexBase (g_cusparse.descr, CUSPARSE_INDEX_BASE_ZERO);
  g_cusparse.device = dev;
  return BMFP_SUCCESS;
}
} // namespace

int spmv_cusparse (int dtype, bool column_major, int nbr, int nbc, int bs, int64_t nnzb,
                   const int *row_ptr, const int *cols, const void *vals, const void *x, void *y,
                   cudaStream_t stream)
{
  int st = ensure_handle ();
  if (st != BMFP_SUCCESS)
    return st;
  if (bs == 1)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "cuSPARSE bsrmv needs bs > 1");
  cusparseSetStream (g_cusparse.handle, stream);
  const cusparseDirection_t dir = column_major ? CUSPARSE_DIRECTION_COLUMN : CUSPARSE_DIRECTION_ROW;
  cusparseStatus_t s;
  if (dtype == BMFP_R64F)
    {
      const double alpha = 1.0, beta = 0.0;
      s = cusparseDbsrmv (g_cusparse.handle, dir, CUSPARSE_OPERATION_NON_TRANSPOSE, nbr, nbc,
                          (int) nnzb, &alpha, g_cusparse.descr, (const double *) vals, row_ptr,
                          cols, bs, (const double *) x, &beta, (double *) y);
    }
  else
    {
      const float alpha = 1.0f, beta = 0.0f;
      s = cusparseSbsrmv (g_cusparse.handle, dir, CUSPARSE_OPERATION_NON_TRANSPOSE, nbr, nbc,
                          (int) nnzb, &alpha, g_cusparse.descr, (const float *) vals, row_ptr,
                          cols, bs, (const float *) x, &beta, (float *) y);
    }
  if (s != CUSPARSE_STATUS_SUCCESS)
    return fail (BMFP_ERROR_CUDA, "cusparse bsrmv failed: %d", (int) s);
  return BMFP_SUCCESS;
}
} // namespace bmfp
