// The reference's main.cpp measurement flow (perform_measurements,
// main.cpp:131-316, without the fmt printer and the JIT submodule) and its
// solver call (measure_golden_bridge, main.cpp:369-375), compiled against the
// drop-in headers and linked with libbmfp.so. Prints one line per measured
// format ("<bs> <dtype> <format>\t<seconds>\t<GB/s>") and one line per solve.
#include "bicgstab.h"
#include "gpu_matrix_multiplier.h"
#include "matrix_converters.h"
#include "measurement_class.h"

#include <cmath>
#include <cstdio>
#include <memory>
#include <vector>

template <typename T, typename I>
static std::vector<T> cpu_reference (const csr_matrix_class<T, I> &m)
{
  std::vector<T> y ((size_t) m.n_rows);
  for (I r = 0; r < m.n_rows; r++)
    {
      T dot = 0;
      for (I e = m.row_ptr[r]; e < m.row_ptr[r + 1]; e++)
        dot += m.values[e] * (T) 1; // x := 1, as main.cpp:27
      y[r] = dot;
    }
  return y;
}

template <typename T> static void measure (int bs, int n_rows, int bpr, const char *tag)
{
  auto block = gen_n_diag_bcsr<T, int> (n_rows, bpr, bs);
  csr_matrix_class<T, int> csr (*block);
  const std::vector<T> ref = cpu_reference (csr);
  std::vector<measurement_class> all;
  all.push_back (gpu_csr_spmv<T, int> (csr, ref.data ()));
  all.push_back (gpu_csr_vector_spmv<T, int> (csr, ref.data ()));
  std::unique_ptr<T[]> transposed (new T[block->size ()]);
  block->transpose_blocks (transposed.get ());
  auto first = gpu_bcsr_spmv<T, int> (*block, transposed.get (), ref.data ());
  for (int rep = 0; rep < 3; rep++)
    {
      auto next = gpu_bcsr_spmv<T, int> (*block, transposed.get (), ref.data ());
      for (size_t i = 0; i < first.size (); i++)
        first[i] += next[i];
    }
  for (auto &m : first)
    {
      m.finalize ();
      all.push_back (m);
    }
  for (auto &m : all)
    std::printf ("%d %s %s\t%.9g\t%.3f\n", bs, tag, m.get_format ().c_str (), m.get_elapsed (),
                 m.get_effective_bandwidth ());
}

template <typename T, typename C> static void solve (int nx, int ny, bool precond, const char *tag)
{
  bmfp_solver_options unused;
  (void) unused;
  std::vector<int> rp (nx * ny + 1);
  int64_t nnzb = 0;
  bmfp_gen_q4_elasticity (BMFP_R64F, nx, ny, 1.0, 0.3, rp.data (), &nnzb, nullptr, nullptr, nullptr);
  bcsr_matrix_class<T, C> block (nx * ny, nx * ny, 2, (C) nnzb);
  std::vector<int> cols (nnzb);
  std::vector<T> b (2 * nx * ny);
  bmfp_gen_q4_elasticity (sizeof (T) == 8 ? BMFP_R64F : BMFP_R32F, nx, ny, 1.0, 0.3, rp.data (), &nnzb,
                          cols.data (), block.values.get (), b.data ());
  for (size_t i = 0; i < rp.size (); i++)
    block.row_ptr[i] = (C) rp[i];
  for (int64_t i = 0; i < nnzb; i++)
    block.columns[i] = (C) cols[i];
  csr_matrix_class<T, C> A (block);
  const T eps = sizeof (T) == 8 ? (T) 1e-8 : (T) 1e-4;
  gpu_bicgstab<T, C> solver (A, precond);
  const T *x = solver.solve (A, b.data (), eps, 20000);
  double rr = 0, bb = 0;
  for (C r = 0; r < A.n_rows; r++)
    {
      double acc = 0;
      for (C e = A.row_ptr[r]; e < A.row_ptr[r + 1]; e++)
        acc += (double) A.values[e] * (double) x[A.columns[e]];
      rr += (b[r] - acc) * (b[r] - acc);
      bb += (double) b[r] * b[r];
    }
  std::printf ("solve %s precond=%d iterations=%d recursive=%.3e true=%.3e\n", tag, (int) precond,
               solver.last_info ().iterations, solver.last_info ().recursive_rel_residual, std::sqrt (rr / bb));
}

int main ()
{
  for (int bs : { 2, 3, 8 })
    {
      measure<float> (bs, 5000, 6, "f32");
      measure<double> (bs, 5000, 6, "f64");
    }
  solve<double, int> (40, 10, false, "f64/int");
  solve<double, unsigned> (40, 10, true, "f64/unsigned");
  solve<float, int> (20, 5, false, "f32/int");
  return 0;
}
