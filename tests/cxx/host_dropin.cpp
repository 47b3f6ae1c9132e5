// Host-only use of the drop-in headers (no GPU): generator, conversions,
// transpose, MatrixMarket writer and measurement_class, as the reference's
// main.cpp uses them. Writes raw arrays that the pytest compares with the
// golden vectors made from the reference's own headers.
//   host_dropin <out_dir> <f32|f64> <n_rows> <blocks_per_row> <bs>
//   host_dropin <out_dir> mm
//   host_dropin <out_dir> measure
//   host_dropin <out_dir> bridge
#include "golden_gate_bridge.h"
#include "matrix_converters.h"
#include "measurement_class.h"

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

template <typename T> static void dump (const std::string &path, const T *p, size_t n)
{
  std::FILE *f = std::fopen (path.c_str (), "wb");
  if (!f)
    std::exit (2);
  std::fwrite (p, sizeof (T), n, f);
  std::fclose (f);
}

template <typename T> static int run (const std::string &dir, int n, int bpr, int bs)
{
  auto m = gen_n_diag_bcsr<T, int> (n, bpr, bs);
  dump (dir + "/bcsr_row_ptr", m->row_ptr.get (), (size_t) n + 1);
  dump (dir + "/bcsr_cols", m->columns.get (), (size_t) m->nnzb);
  dump (dir + "/bcsr_vals", m->values.get (), (size_t) m->size ());
  std::vector<T> t ((size_t) m->size ());
  m->transpose_blocks (t.data ());
  dump (dir + "/bcsr_vals_colmajor", t.data (), t.size ());
  csr_matrix_class<T, int> csr (*m);
  dump (dir + "/csr_row_ptr", csr.row_ptr.get (), (size_t) csr.n_rows + 1);
  dump (dir + "/csr_cols", csr.columns.get (), (size_t) csr.nnz);
  dump (dir + "/csr_vals", csr.values.get (), (size_t) csr.nnz);
  // get_block_data_by_column finds the diagonal-adjacent block of row 1
  const T *blk = m->get_block_data_by_column (1, m->columns[m->row_ptr[1]]);
  std::printf ("first block of row 1 starts with %.17g\n", (double) blk[0]);
  return 0;
}

int main (int argc, char **argv)
{
  if (argc < 3)
    return 1;
  const std::string dir = argv[1], mode = argv[2];
  if (mode == "mm")
    {
      auto m = gen_n_diag_bcsr<double, int> (6, 3, 2);
      csr_matrix_class<double, int> csr (*m);
      csr.write_mm (dir + "/out.mtx");
      return 0;
    }
  if (mode == "measure")
    {
      const double runs[][3] = { { 0.5, 1e9, 2e9 }, { 0.25, 1e9, 1e9 } };
      measurement_class total;
      for (auto &r : runs)
        total += measurement_class ("m", r[0], r[1], r[2]);
      total.finalize ();
      std::printf ("%.17g %.17g %.17g %s\n", total.get_elapsed (), total.get_effective_bandwidth (),
                   total.get_computational_throughput (), total.get_format ().c_str ());
      return 0;
    }
  if (mode == "bridge")
    {
      // the fixture's bridge: a 1280 m main span, 345 m sides, 230 m towers,
      // the load of main.cpp:356-363
      const double side = 345.0, main_len = 1280.0;
      auto load = [=] (double x) -> std::pair<double, double> {
        const double mid = (main_len + side * 2) / 2;
        if (x > mid - 450 && x < mid + 450)
          return { 0, -2000000.0 };
        return { 0, 0 };
      };
      golden_gate_bridge_2d<double, int, false> bridge (load, main_len, side, 230.0, 7.62);
      const auto &m = *bridge.matrix;
      dump (dir + "/bcsr_row_ptr", m.row_ptr.get (), (size_t) m.n_rows + 1);
      dump (dir + "/bcsr_cols", m.columns.get (), (size_t) m.nnzb);
      dump (dir + "/bcsr_vals", m.values.get (), (size_t) m.size ());
      dump (dir + "/rhs", bridge.forces_rhs.get (), (size_t) m.n_rows * 2);
      bridge.write_vtk (dir + "/bridge.vtk");
      std::vector<double> disp ((size_t) m.n_rows * 2);
      for (size_t i = 0; i < disp.size (); i++)
        disp[i] = ((int) (i % 7) - 3) * 0.001;
      bridge.write_vtk (dir + "/bridge_disp.vtk", disp.data ());
      return 0;
    }
  if (argc != 6)
    return 1;
  const int n = std::atoi (argv[3]), bpr = std::atoi (argv[4]), bs = std::atoi (argv[5]);
  return mode == "f32" ? run<float> (dir, n, bpr, bs) : run<double> (dir, n, bpr, bs);
}
