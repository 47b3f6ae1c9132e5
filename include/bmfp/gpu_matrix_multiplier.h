// Drop-in replacement for the reference's gpu/gpu_matrix_multiplier.h.
//
// gpu_csr_spmv, gpu_csr_vector_spmv and gpu_bcsr_spmv keep the reference's
// signatures and behaviour (gpu/gpu_matrix_multiplier.h:12-26,
// gpu_matrix_multiplier.cu:88-1331): each call uploads the matrix, sets
// x := 1, times every variant's single launch with CUDA events, downloads y,
// checks it with compare_results against reference_y, frees the device
// memory and returns measurement_class objects named by the reference's
// format strings. The kernels are libbmfp.so's sm_103a kernels, reached
// through the C ABI (bmfp_csr_spmv, bmfp_bcsr_spmv). Differences, on purpose:
//  * the measurements carry the algorithmic bytes and flops (the reference
//    passed 0 for GPU runs), so get_effective_bandwidth() is meaningful;
//  * variants a block size has no kernel for (the template variants outside
//    bs in {1,2,3,4,8,16,32}, po2 for non-powers of two, cuSPARSE at bs 1) are
//    left out of the returned vector instead of being timed without a launch;
//  * one extra entry, "GPU BCSR (GB300 native)", times the tuned kernel.
#ifndef BMFP_GPU_MATRIX_MULTIPLIER_H
#define BMFP_GPU_MATRIX_MULTIPLIER_H

#include "bmfp.h"
#include "matrix_converters.h"
#include "measurement_class.h"

#include <cuda_runtime.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace bmfp_detail
{
inline void cuda_throw (cudaError_t e, const char *what)
{
  if (e != cudaSuccess)
    throw std::runtime_error (std::string (what) + ": " + cudaGetErrorString (e));
}

// Device copy of a host array, freed on scope exit.
template <typename T> struct device_array
{
  T *ptr = nullptr;
  explicit device_array (size_t n) { cuda_throw (cudaMalloc (&ptr, sizeof (T) * (n ? n : 1)), "cudaMalloc"); }
  device_array (const T *host, size_t n) : device_array (n)
  {
    if (n)
      cuda_throw (cudaMemcpy (ptr, host, sizeof (T) * n, cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  ~device_array () { cudaFree (ptr); }
  device_array (const device_array &) = delete;
  device_array &operator= (const device_array &) = delete;
};

// Times one launch (returns seconds) and leaves y on the device.
template <typename F> double time_launch (F &&launch, bool &supported)
{
  cudaEvent_t start, stop;
  cuda_throw (cudaEventCreate (&start), "cudaEventCreate");
  cuda_throw (cudaEventCreate (&stop), "cudaEventCreate");
  cuda_throw (cudaDeviceSynchronize (), "cudaDeviceSynchronize");
  cudaEventRecord (start);
  const int st = launch ();
  cudaEventRecord (stop);
  cudaEventSynchronize (stop);
  float ms = 0.0f;
  cudaEventElapsedTime (&ms, start, stop);
  cudaEventDestroy (start);
  cudaEventDestroy (stop);
  supported = st == BMFP_SUCCESS;
  if (st != BMFP_SUCCESS && st != BMFP_ERROR_NOT_SUPPORTED)
    throw std::runtime_error (std::string ("bmfp SpMV: ") + bmfp_last_error ());
  return ms / 1000.0;
}

template <typename T, typename I>
measurement_class run_csr (int variant, const csr_matrix_class<T, I> &m, const T *reference_y)
{
  const size_t n = (size_t) m.n_rows, nnz = (size_t) m.nnz;
  device_array<int> rp (reinterpret_cast<const int *> (m.row_ptr.get ()), n + 1);
  device_array<int> cols (reinterpret_cast<const int *> (m.columns.get ()), nnz);
  device_array<T> vals (m.values.get (), nnz), y (n);
  std::vector<T> ones ((size_t) m.n_cols, (T) 1);
  device_array<T> x (ones.data (), ones.size ());
  bool ok = false;
  const double elapsed = time_launch (
    [&] { return bmfp_csr_spmv (dtype_of<T> (), variant, (int) n, (int) m.n_cols, (int64_t) nnz, rp.ptr, cols.ptr,
                                vals.ptr, x.ptr, y.ptr, nullptr); },
    ok);
  std::unique_ptr<T[]> host_y (new T[n]);
  cuda_throw (cudaMemcpy (host_y.get (), y.ptr, sizeof (T) * n, cudaMemcpyDeviceToHost), "cudaMemcpy");
  compare_results ((unsigned) n, reference_y, host_y.get ());
  return measurement_class (bmfp_spmv_variant_name (variant), elapsed,
                            (double) bmfp_csr_spmv_bytes (dtype_of<T> (), (int) n, (int) m.n_cols, (int64_t) nnz),
                            2.0 * (double) nnz);
}
} // namespace bmfp_detail

// "GPU CSR": thread per row (gpu_matrix_multiplier.cu:65-163).
template <typename data_type, typename index_type>
measurement_class gpu_csr_spmv (const csr_matrix_class<data_type, index_type> &matrix, const data_type *reference_y)
{
  bmfp_detail::check_index<index_type> ();
  return bmfp_detail::run_csr (BMFP_SPMV_CSR_SCALAR, matrix, reference_y);
}

// "GPU CSR-Vector": warp per row (gpu_matrix_multiplier.cu:165-273).
template <typename data_type, typename index_type>
measurement_class gpu_csr_vector_spmv (const csr_matrix_class<data_type, index_type> &matrix,
                                       const data_type *reference_y)
{
  bmfp_detail::check_index<index_type> ();
  return bmfp_detail::run_csr (BMFP_SPMV_CSR_VECTOR, matrix, reference_y);
}

// Every BCSR variant of gpu_matrix_multiplier.cu:736-1331, in the reference's
// order, then the tuned kernel. transpose_matrix_data holds the
// column-major blocks (bcsr_matrix_class::transpose_blocks).
template <typename data_type, typename index_type>
std::vector<measurement_class> gpu_bcsr_spmv (bcsr_matrix_class<data_type, index_type> &matrix,
                                              const data_type *transpose_matrix_data, const data_type *reference_y)
{
  using namespace bmfp_detail;
  check_index<index_type> ();
  const int nbr = (int) matrix.n_rows, nbc = (int) matrix.n_cols, bs = (int) matrix.bs;
  const size_t nnzb = (size_t) matrix.nnzb, nvals = nnzb * bs * bs;
  const size_t nx = (size_t) nbc * bs, ny = (size_t) nbr * bs;
  device_array<int> rp (reinterpret_cast<const int *> (matrix.row_ptr.get ()), (size_t) nbr + 1);
  device_array<int> cols (reinterpret_cast<const int *> (matrix.columns.get ()), nnzb);
  device_array<data_type> row_major (matrix.values.get (), nvals), col_major (transpose_matrix_data, nvals), y (ny);
  std::vector<data_type> ones (nx, (data_type) 1);
  device_array<data_type> x (ones.data (), nx);
  std::unique_ptr<data_type[]> host_y (new data_type[ny]);
  const double bytes = (double) bmfp_bcsr_spmv_bytes (dtype_of<data_type> (), nbr, nbc, bs, (int64_t) nnzb);
  const double flops = 2.0 * (double) nvals;

  static const int order[] = { BMFP_SPMV_BCSR_ROW_THREAD,        BMFP_SPMV_BCSR_ROW_WARP,
                               BMFP_SPMV_CUSPARSE_ROW,           BMFP_SPMV_CUSPARSE_COL,
                               BMFP_SPMV_BCSR_COL_THREAD,        BMFP_SPMV_BCSR_COL_THREAD_TEMPLATE,
                               BMFP_SPMV_BCSR_COL_COAL_X,        BMFP_SPMV_BCSR_COL_COAL_X_TEMPLATE,
                               BMFP_SPMV_BCSR_COL_BY_COL,        BMFP_SPMV_BCSR_COL_BY_COL_FASTDIV,
                               BMFP_SPMV_BCSR_COL_BY_COL_PO2,    BMFP_SPMV_BCSR_COL_BY_COL_TEMPLATE,
                               BMFP_SPMV_BCSR_NATIVE };
  std::vector<measurement_class> results;
  for (int variant : order)
    {
      const data_type *vals = bmfp_spmv_variant_layout (variant) == 1 ? col_major.ptr : row_major.ptr;
      // The native entry takes the column owner on the transposed blocks the
      // caller passes where that is the faster product (FP64, bs 2..32).
      const bool col_owner = variant == BMFP_SPMV_BCSR_NATIVE && sizeof (data_type) == 8
                             && (bs == 2 || bs == 4 || bs == 8 || bs == 16 || bs == 32);
      cuda_throw (cudaMemset (y.ptr, 0, sizeof (data_type) * ny), "cudaMemset");
      bool ok = false;
      const double elapsed = time_launch (
        [&] {
          return col_owner ? bmfp_bcsr_spmv_colmajor (dtype_of<data_type> (), nbr, bs, (int64_t) nnzb, rp.ptr, cols.ptr,
                                                      col_major.ptr, x.ptr, y.ptr, nullptr)
                           : bmfp_bcsr_spmv (dtype_of<data_type> (), variant, nbr, nbc, bs, (int64_t) nnzb, rp.ptr,
                                             cols.ptr, vals, x.ptr, y.ptr, nullptr);
        },
        ok);
      if (!ok)
        continue;
      cuda_throw (cudaMemcpy (host_y.get (), y.ptr, sizeof (data_type) * ny, cudaMemcpyDeviceToHost), "cudaMemcpy");
      compare_results ((unsigned) ny, reference_y, host_y.get ());
      results.emplace_back (bmfp_spmv_variant_name (variant), elapsed, bytes, flops);
    }
  return results;
}

#endif // BMFP_GPU_MATRIX_MULTIPLIER_H
