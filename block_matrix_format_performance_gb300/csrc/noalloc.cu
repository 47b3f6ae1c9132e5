// BiCGStab for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code running under a device-memory
// pool or budget that forbids further allocations, real-time loops where an
// allocation's implicit synchronisation is not acceptable, and plug-ins whose
// host application owns every allocation. bmfp_bicgstab_solve_noalloc takes
// the matrix, the right-hand side and the solution buffer from the caller and
// keeps every other vector of the solve in one file-scope device array,
// g_noalloc_scratch, of fixed size (kNoAllocScratchBytes, about 11.6 MB). Every
// GPU that loads the library holds that array until the process exits.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and caches
// it. That first call should come before any stream capture. The cached
// address belongs to the device's context: a caller that resets the device
// (cudaDeviceReset) after a call must not call this entry point again in the
// same process.
//
// All calls share the one array and it keeps the previous call's contents:
// every solve re-initialises what it reads (the start kernel writes every
// Krylov vector and the scalar state is cleared first). Calls that overlap
// on the GPU — from two host threads, or on two streams — race on the array;
// callers must serialise them.
#include "solver.h"

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

namespace bmfp
{
namespace
{
constexpr int64_t kNoAllocMaxRows = 131072; // scalar rows (DOFs) per solve
constexpr int kNoAllocMaxGrid = 1024;       // CTAs of the phase kernels
constexpr int kNoAllocVectors = 11;         // r, rh, p, v, s, t, q, z, P, g, x'
constexpr size_t kVectorSlot = (size_t) kNoAllocMaxRows * sizeof (double); // 256-byte multiple
constexpr size_t kPartsBytes = (size_t) kRawParts * kNoAllocMaxGrid * sizeof (double);
constexpr size_t kStateSlot = 256;
constexpr size_t kNoAllocScratchBytes = kNoAllocVectors * kVectorSlot + kPartsBytes + kStateSlot;

__device__ __align__ (256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_address[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
int scratch_address (unsigned char **out)
{
  int dev = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "device ordinal %d above %d", dev, kMaxDevices - 1);
  std::lock_guard<std::mutex> lock (g_setup_mutex);
  if (!g_scratch_address[dev])
    {
      void *ptr = nullptr;
      BMFP_CUDA (cudaGetSymbolAddress (&ptr, g_noalloc_scratch));
      g_scratch_address[dev] = static_cast<unsigned char *> (ptr);
    }
  *out = g_scratch_address[dev];
  return BMFP_SUCCESS;
}
} // namespace
} // namespace bmfp

using namespace bmfp;

extern "C" int bmfp_bicgstab_solve_noalloc (int dtype, int n_block_rows, int bs, int64_t nnzb,
                                            const int *d_row_ptr, const int *d_cols,
                                            const void *d_values, const void *d_b, void *d_x,
                                            double tolerance, int max_iterations,
                                            int preconditioner, int *iterations,
                                            double *rel_residual, void *stream)
{
  if (iterations)
    *iterations = 0;
  if (rel_residual)
    *rel_residual = 0.0;
  if (!dtype_ok (dtype))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid dtype %d", dtype);
  if (n_block_rows < 0 || bs < 0 || nnzb < 0 || !(tolerance > 0) || max_iterations < 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid size, tolerance or iteration limit");
  if (preconditioner != BMFP_PRECOND_NONE && preconditioner != BMFP_PRECOND_JACOBI)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid preconditioner %d", preconditioner);
  const int64_t n = (int64_t) n_block_rows * (bs ? bs : 1);
  if (n > kNoAllocMaxRows)
    return fail (BMFP_ERROR_NOT_SUPPORTED,
                 "%lld rows exceed the no-allocation scratch limit of %lld rows; use bmfp_solver_create",
                 (long long) n, (long long) kNoAllocMaxRows);
  // The phase kernels index values with 32-bit block offsets times bs^2, as
  // the matrix handles do (bmfp_matrix_create_bcsr refuses the same).
  const int64_t bsq = (int64_t) (bs ? bs : 1) * (bs ? bs : 1);
  if (nnzb > INT32_MAX || nnzb * bsq > INT32_MAX)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "%lld stored values exceed 2^31 - 1", (long long) (nnzb * bsq));
  if (n == 0)
    return BMFP_SUCCESS;
  if (!d_row_ptr || !d_b || !d_x || (nnzb > 0 && (!d_cols || !d_values)))
    return fail (BMFP_ERROR_INVALID_VALUE, "null device pointer");
  cudaStream_t s = as_stream (stream);

  unsigned char *base = nullptr;
  int rc = scratch_address (&base);
  if (rc != BMFP_SUCCESS)
    return rc;

  RawSolve b;
  b.A.dtype = dtype;
  b.A.n_rows = n_block_rows;
  b.A.n_cols = n_block_rows;
  b.A.bs = bs;
  b.A.nnz = nnzb;
  b.A.d_row_ptr = const_cast<int *> (d_row_ptr);
  b.A.d_cols = const_cast<int *> (d_cols);
  b.A.d_vals = const_cast<void *> (d_values);
  b.n = n;
  b.jacobi = preconditioner == BMFP_PRECOND_JACOBI;
  b.aligned = (reinterpret_cast<uintptr_t> (d_values) & 15u) == 0;
  rc = raw_solve_grid (n, &b.grid);
  if (rc != BMFP_SUCCESS)
    return rc;
  if (b.grid > kNoAllocMaxGrid)
    b.grid = kNoAllocMaxGrid;
  void **vecs[kNoAllocVectors] = { &b.r, &b.rh, &b.p, &b.v, &b.s, &b.t, &b.q, &b.z, &b.P, &b.g, &b.xp };
  for (int i = 0; i < kNoAllocVectors; i++)
    *vecs[i] = base + (size_t) i * kVectorSlot;
  b.part = reinterpret_cast<double *> (base + kNoAllocVectors * kVectorSlot);
  b.st = reinterpret_cast<DevState *> (base + kNoAllocVectors * kVectorSlot + kPartsBytes);
  b.x = d_x;

  // The previous call's state is still in the array: clear the scalars.
  BMFP_CUDA (cudaMemsetAsync (b.st, 0, sizeof (DevState), s));
  if (b.jacobi && (rc = raw_jacobi (b, s)) != BMFP_SUCCESS)
    return rc;
  if ((rc = raw_start (b, d_b, tolerance, max_iterations, s)) != BMFP_SUCCESS)
    return rc;
  DevState h{};
  for (;;)
    {
      for (int it = 0; it < 16 && rc == BMFP_SUCCESS; it++)
        for (int ph = 1; ph <= 5 && rc == BMFP_SUCCESS; ph++)
          rc = raw_phase (b, ph, s);
      if (rc != BMFP_SUCCESS)
        return rc;
      // Read the scalars into this stack frame (no pinned buffer to allocate).
      BMFP_CUDA (cudaMemcpyAsync (&h, b.st, sizeof (DevState), cudaMemcpyDeviceToHost, s));
      BMFP_CUDA (cudaStreamSynchronize (s));
      if (h.done)
        break;
    }
  // The iterate accumulated in the array (x' of the run) into the caller's x.
  if ((rc = raw_finish (b, s)) != BMFP_SUCCESS)
    return rc;
  BMFP_CUDA (cudaStreamSynchronize (s));
  if (iterations)
    *iterations = h.iter;
  if (rel_residual)
    *rel_residual = h.norm_b > 0 ? std::sqrt (h.rr) / h.norm_b : 0.0;
  if (h.status == kStateConverged)
    return BMFP_SUCCESS;
  if (h.status == kStateBreakdown)
    return fail (BMFP_ERROR_BREAKDOWN, "BiCGStab breakdown after %d iterations", h.iter);
  return fail (BMFP_ERROR_NOT_CONVERGED, "no convergence in %d iterations", h.iter);
}
