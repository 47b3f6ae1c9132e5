// Drop-in replacement for the reference's gpu/bicgstab.h.
//
// gpu_bicgstab<T, C> keeps the reference's interface (gpu/bicgstab.h:10-16):
// the constructor takes the CSR matrix and whether to use point-Jacobi
// preconditioning, solve(A, b, epsilon, max_iterations) returns a pointer to
// the solution in pinned host memory owned by the solver (freed by the
// destructor, gpu/bicgstab.cu:66, 97), and the stopping rule is the
// reference's recursive one, ||r_i|| / ||b|| < epsilon (gpu/bicgstab.cu:512).
// The solve runs libbmfp.so's fused, device-resident BiCGStab through the C
// ABI (bmfp_solver_create / bmfp_solver_solve). Differences, on purpose:
//  * the returned solution is the last iterate (the reference copied buffer
//    half 0, gpu/bicgstab.cu:515, which is the previous iterate after an odd
//    number of iterations);
//  * nothing is printed per iteration; last_info() reports iterations and
//    residuals instead;
//  * errors throw std::runtime_error instead of calling exit()
//    (gpu/bicgstab.cu:12-21).
// Index types of any width are accepted (the reference instantiates int and
// unsigned); indices are narrowed to 32 bits for the device.
#ifndef BMFP_BICGSTAB_H
#define BMFP_BICGSTAB_H

#include "bmfp.h"
#include "matrix_converters.h"

#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

template <class T, class C = std::size_t>
class gpu_bicgstab
{
  static_assert (std::is_same<T, float>::value || std::is_same<T, double>::value, "float or double");

public:
  gpu_bicgstab () = delete;

  explicit gpu_bicgstab (const csr_matrix_class<T, C> &A_cpu, bool use_precond)
    : n_rows ((unsigned) A_cpu.n_rows), n_elements (A_cpu.nnz), precond (use_precond)
  {
    if (A_cpu.n_rows != A_cpu.n_cols)
      throw std::runtime_error ("gpu_bicgstab: the matrix must be square");
    if (cudaMallocHost ((void **) &h_x, sizeof (T) * (n_rows ? n_rows : 1)) != cudaSuccess)
      throw std::runtime_error ("gpu_bicgstab: cannot allocate the pinned solution buffer");
    if (cudaMalloc ((void **) &d_b, sizeof (T) * (n_rows ? n_rows : 1)) != cudaSuccess
        || cudaMalloc ((void **) &d_x, sizeof (T) * (n_rows ? n_rows : 1)) != cudaSuccess)
      {
        release ();
        throw std::runtime_error ("Error! There is not enough memory on gpu");
      }
  }

  ~gpu_bicgstab () { release (); }

  gpu_bicgstab (const gpu_bicgstab &) = delete;
  gpu_bicgstab &operator= (const gpu_bicgstab &) = delete;

  T *solve (const csr_matrix_class<T, C> &A, const T *b, T epsilon, unsigned int max_iterations)
  {
    upload (A);
    bmfp_solver_options o;
    bmfp_solver_options_init (&o);
    o.precision = std::is_same<T, double>::value ? BMFP_SOLVE_FP64 : BMFP_SOLVE_FP32;
    o.preconditioner = precond ? BMFP_PRECOND_JACOBI : BMFP_PRECOND_NONE;
    o.tolerance = (double) epsilon;
    o.max_iterations = (int) max_iterations;
    o.check_true_residual = 0;
    bmfp_solver_t solver = nullptr;
    check (bmfp_solver_create (&solver, matrix, &o, nullptr), "bmfp_solver_create");
    if (cudaMemcpy (d_b, b, sizeof (T) * n_rows, cudaMemcpyHostToDevice) != cudaSuccess)
      {
        bmfp_solver_destroy (solver);
        throw std::runtime_error ("gpu_bicgstab: cannot upload b");
      }
    const int st = bmfp_solver_solve (solver, d_b, d_x, &info, nullptr);
    bmfp_solver_destroy (solver);
    if (st != BMFP_SUCCESS && st != BMFP_ERROR_NOT_CONVERGED && st != BMFP_ERROR_BREAKDOWN)
      throw std::runtime_error (std::string ("gpu_bicgstab: ") + bmfp_last_error ());
    if (cudaMemcpy (h_x, d_x, sizeof (T) * n_rows, cudaMemcpyDeviceToHost) != cudaSuccess)
      throw std::runtime_error ("gpu_bicgstab: cannot download x");
    return h_x;
  }

  // Iterations, residuals and status of the last solve().
  const bmfp_solve_info &last_info () const { return info; }

private:
  void upload (const csr_matrix_class<T, C> &A)
  {
    if (matrix)
      bmfp_matrix_destroy (matrix);
    matrix = nullptr;
    const size_t nnz = (size_t) A.nnz;
    const int *rp = nullptr, *cols = nullptr;
    std::vector<int> rp32, cols32;
    if (sizeof (C) == sizeof (int))
      {
        rp = reinterpret_cast<const int *> (A.row_ptr.get ());
        cols = reinterpret_cast<const int *> (A.columns.get ());
      }
    else
      {
        rp32.assign (A.row_ptr.get (), A.row_ptr.get () + n_rows + 1);
        cols32.assign (A.columns.get (), A.columns.get () + nnz);
        rp = rp32.data ();
        cols = cols32.data ();
      }
    check (bmfp_matrix_create_csr (&matrix, std::is_same<T, double>::value ? BMFP_R64F : BMFP_R32F, (int) n_rows,
                                   (int) A.n_cols, (int64_t) nnz, rp, cols, A.values.get (), nullptr),
           "bmfp_matrix_create_csr");
  }

  static void check (int st, const char *what)
  {
    if (st != BMFP_SUCCESS)
      throw std::runtime_error (std::string (what) + ": " + bmfp_last_error ());
  }

  void release ()
  {
    if (matrix)
      bmfp_matrix_destroy (matrix);
    matrix = nullptr;
    cudaFree (d_b);
    cudaFree (d_x);
    if (h_x)
      cudaFreeHost (h_x);
    d_b = d_x = h_x = nullptr;
  }

  unsigned int n_rows = 0;
  const C n_elements = 0;
  bool precond = false;
  T *h_x = nullptr; // pinned, owned by the solver
  T *d_b = nullptr;
  T *d_x = nullptr;
  bmfp_matrix_t matrix = nullptr;
  bmfp_solve_info info{};
};

#endif // BMFP_BICGSTAB_H
