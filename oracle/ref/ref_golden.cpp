// Golden-vector driver over the reference's OWN headers — TEST INFRASTRUCTURE.
//
// Compiled in place against the reference sources (common/matrix_converters.h,
// common/measurement_class.{h,cpp}, common/mmio.c, fem_2d/golden_gate_bridge.h)
// by oracle/Makefile into oracle/_ref/ref_golden. Nothing here reimplements
// the reference: every number it writes comes from the reference's code.
// tests/golden/make_golden.py runs it and packs the outputs into fixtures.
//
// Modes (all outputs are raw little-endian arrays named <prefix>.<field>):
//   ndiag  f32|f64 n_rows blocks_per_row bs prefix
//          gen_n_diag_bcsr (matrix_converters.h:157-196), transpose_blocks
//          (:32-49) and the BCSR->CSR constructor (:88-117).
//   bridge prefix
//          golden_gate_bridge_2d<double,int,false> on a short span: its BCSR
//          stiffness matrix (golden_gate_bridge.h:767-878), forces_rhs, CSR
//          and write_vtk output (:239-282), plain and displaced.
//   compare f32|f64 n file_a file_b
//          compare_results (measurement_class.h:58-87); prints FLAGGED or OK.
//   measure elapsed bytes ops [elapsed bytes ops ...]
//          measurement_class (measurement_class.cpp:7-16, .h:27-47) summed
//          with += and finalize(); prints elapsed, GB/s, GFLOP/s.
//   mm prefix
//          csr_matrix_class::write_mm (matrix_converters.h:119-144) of a small
//          gen_n_diag_bcsr matrix, to <prefix>.mtx.
#include <string>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <vector>

#include "matrix_converters.h"
#include "measurement_class.h"
#include "fem_2d/golden_gate_bridge.h"

template <typename T>
static void dump (const std::string &name, const T *data, size_t n)
{
  FILE *f = std::fopen (name.c_str (), "wb");
  if (!f)
    {
      std::perror (name.c_str ());
      std::exit (2);
    }
  if (n)
    std::fwrite (data, sizeof (T), n, f);
  std::fclose (f);
}

template <typename T>
static std::vector<T> load (const std::string &name, size_t n)
{
  std::vector<T> v (n);
  FILE *f = std::fopen (name.c_str (), "rb");
  if (!f || std::fread (v.data (), sizeof (T), n, f) != n)
    {
      std::fprintf (stderr, "cannot read %s\n", name.c_str ());
      std::exit (2);
    }
  std::fclose (f);
  return v;
}

template <typename T>
static void dump_bcsr (const std::string &prefix, bcsr_matrix_class<T, int> &m)
{
  const size_t nnzb = m.nnzb, bs = m.bs;
  dump (prefix + ".bcsr_row_ptr", m.row_ptr.get (), (size_t) m.n_rows + 1);
  dump (prefix + ".bcsr_cols", m.columns.get (), nnzb);
  dump (prefix + ".bcsr_vals", m.values.get (), nnzb * bs * bs);

  std::unique_ptr<T[]> tr (new T[nnzb * bs * bs]);
  m.transpose_blocks (tr.get ());
  dump (prefix + ".bcsr_vals_colmajor", tr.get (), nnzb * bs * bs);

  csr_matrix_class<T, int> csr (m);
  dump (prefix + ".csr_row_ptr", csr.row_ptr.get (), (size_t) csr.n_rows + 1);
  dump (prefix + ".csr_cols", csr.columns.get (), (size_t) csr.nnz);
  dump (prefix + ".csr_vals", csr.values.get (), (size_t) csr.nnz);

  std::ofstream meta (prefix + ".meta");
  meta << m.n_rows << " " << m.n_cols << " " << m.bs << " " << m.nnzb << " " << csr.nnz << "\n";
}

template <typename T>
static int run_ndiag (int n_rows, int bpr, int bs, const std::string &prefix)
{
  auto m = gen_n_diag_bcsr<T, int> (n_rows, bpr, bs);
  dump_bcsr (prefix, *m);
  return 0;
}

static int run_bridge (const std::string &prefix)
{
  // A short span (one 1280 m main part, 345 m sides, 230 m towers, 7.62 m
  // segments) keeps the fixture small; the load mimics main.cpp:357-364.
  const double side = 345.0, main_len = 1280.0;
  auto load = [=] (double x) -> std::pair<double, double> {
    const double mid = (main_len + side * 2) / 2;
    if (x > mid - 450 && x < mid + 450)
      return {0, -2000000.0};
    return {0, 0};
  };
  golden_gate_bridge_2d<double, int, false> bridge (load, main_len, side, 230.0, 7.62);
  dump_bcsr (prefix, *bridge.matrix);
  dump (prefix + ".rhs", bridge.forces_rhs.get (), (size_t) bridge.matrix->n_rows * 2);
  // write_vtk (golden_gate_bridge.h:239-282), plain and with a fixed
  // displacement pattern d_i = ((i mod 7) - 3) / 1000
  bridge.write_vtk (prefix + ".vtk");
  std::vector<double> disp ((size_t) bridge.matrix->n_rows * 2);
  for (size_t i = 0; i < disp.size (); i++)
    disp[i] = ((int) (i % 7) - 3) * 0.001;
  bridge.write_vtk (prefix + "_disp.vtk", disp.data ());
  return 0;
}

template <typename T>
static int run_compare (unsigned n, const std::string &fa, const std::string &fb)
{
  auto a = load<T> (fa, n);
  auto b = load<T> (fb, n);
  std::stringstream captured;
  auto *old = std::cerr.rdbuf (captured.rdbuf ());
  compare_results (n, a.data (), b.data ());
  std::cerr.rdbuf (old);
  const std::string out = captured.str ();
  std::printf ("%s\n", out.find ("ERROR") != std::string::npos ? "FLAGGED" : "OK");
  return 0;
}

static int run_measure (int argc, char **argv)
{
  measurement_class total;
  for (int i = 0; i + 2 < argc; i += 3)
    total += measurement_class ("m", std::atof (argv[i]), std::atof (argv[i + 1]), std::atof (argv[i + 2]));
  total.finalize ();
  std::printf ("%.17g %.17g %.17g\n", total.get_elapsed (), total.get_effective_bandwidth (),
               total.get_computational_throughput ());
  return 0;
}

static int run_mm (const std::string &prefix)
{
  auto m = gen_n_diag_bcsr<double, int> (6, 3, 2);
  csr_matrix_class<double, int> csr (*m);
  csr.write_mm (prefix + ".mtx");
  return 0;
}

int main (int argc, char **argv)
{
  if (argc < 2)
    return 1;
  const std::string mode = argv[1];
  if (mode == "ndiag" && argc == 7)
    {
      const std::string dt = argv[2];
      int n = std::atoi (argv[3]), bpr = std::atoi (argv[4]), bs = std::atoi (argv[5]);
      return dt == "f32" ? run_ndiag<float> (n, bpr, bs, argv[6]) : run_ndiag<double> (n, bpr, bs, argv[6]);
    }
  if (mode == "bridge" && argc == 3)
    return run_bridge (argv[2]);
  if (mode == "compare" && argc == 6)
    {
      const std::string dt = argv[2];
      unsigned n = (unsigned) std::atoi (argv[3]);
      return dt == "f32" ? run_compare<float> (n, argv[4], argv[5]) : run_compare<double> (n, argv[4], argv[5]);
    }
  if (mode == "measure")
    return run_measure (argc - 2, argv + 2);
  if (mode == "mm" && argc == 3)
    return run_mm (argv[2]);
  std::fprintf (stderr, "bad arguments\n");
  return 1;
}
