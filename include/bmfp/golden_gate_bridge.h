// Drop-in replacement for the reference's fem_2d/golden_gate_bridge.h.
//
// The same class template golden_gate_bridge_2d<data_type, index_type,
// use_frames> with the constructor, public members (matrix, forces_rhs) and
// write_vtk of fem_2d/golden_gate_bridge.h:101-282, for the truss model
// (use_frames = false) that main.cpp:349-381 builds. The stiffness matrix
// comes from libbmfp.so (bmfp_gen_golden_gate_bridge), bit-exact with the
// reference's; the load function is applied to the deck's top-chord nodes as
// the reference applies it (:170-178). Unlike the reference, the constructor
// writes no "nodes", "forces" and "elements" files into the working
// directory.
#ifndef BMFP_GOLDEN_GATE_BRIDGE_H
#define BMFP_GOLDEN_GATE_BRIDGE_H

#include "matrix_converters.h"

#include <cmath>
#include <fstream>
#include <memory>
#include <string>
#include <tuple>

template <typename data_type, typename index_type, bool use_frames> class golden_gate_bridge_2d
{
  static_assert (!use_frames, "libbmfp builds the truss model (use_frames = false), the one main.cpp uses");

public:
  template <typename function_type>
  explicit golden_gate_bridge_2d (const function_type &load, data_type main_part_length_arg,
                                  data_type side_length_arg, data_type tower_height_arg = 230.0,
                                  data_type segment_length_arg = 7.62)
  {
    bmfp_detail::check_index<index_type> ();
    const int dt = bmfp_detail::dtype_of<data_type> ();
    const double span = main_part_length_arg, side = side_length_arg, tower = tower_height_arg,
                 seg = segment_length_arg;
    int n = 0;
    int64_t nnzb = 0;
    bmfp_detail::throw_on (
      bmfp_gen_golden_gate_bridge (dt, span, side, tower, seg, 0.0, 0.0, &n, &nnzb, nullptr, nullptr, nullptr, nullptr),
      "golden_gate_bridge_2d");
    matrix = std::make_unique<bcsr_matrix_class<data_type, index_type>> (n, n, 2, (index_type) nnzb);
    forces_rhs.reset (new data_type[2 * (size_t) n]);
    bmfp_detail::throw_on (bmfp_gen_golden_gate_bridge (dt, span, side, tower, seg, 0.0, 0.0, &n, &nnzb,
                                                        reinterpret_cast<int *> (matrix->row_ptr.get ()),
                                                        reinterpret_cast<int *> (matrix->columns.get ()),
                                                        matrix->values.get (), forces_rhs.get ()),
                           "golden_gate_bridge_2d");

    int segments = 0, n_elements = 0;
    bmfp_detail::throw_on (bmfp_golden_gate_bridge_geometry (dt, span, side, tower, seg, &segments, &nodes_count,
                                                             &n_elements, nullptr, nullptr, nullptr, nullptr),
                           "golden_gate_bridge_2d");
    elements_count = n_elements;
    nodes_xs.reset (new data_type[(size_t) nodes_count]);
    nodes_ys.reset (new data_type[(size_t) nodes_count]);
    elements_starts.reset (new int[(size_t) n_elements]);
    elements_ends.reset (new int[(size_t) n_elements]);
    bmfp_detail::throw_on (bmfp_golden_gate_bridge_geometry (dt, span, side, tower, seg, &segments, &nodes_count,
                                                             &n_elements, nodes_xs.get (), nodes_ys.get (),
                                                             elements_starts.get (), elements_ends.get ()),
                           "golden_gate_bridge_2d");

    for (int s = 0; s < segments; s++)
      for (const int node : { s * 4, s * 4 + 1 })
        std::tie (forces_rhs[node * 2 + 0], forces_rhs[node * 2 + 1]) = load (nodes_xs[node]);
  }

  // Legacy VTK unstructured grid of the truss, optionally displaced, with the
  // mean absolute displacement per node (golden_gate_bridge.h:239-282).
  void write_vtk (const std::string &filename, const data_type *displacement = nullptr)
  {
    std::ofstream vtk (filename);
    vtk << "# vtk DataFile Version 3.0\n";
    vtk << "vtk output\n";
    vtk << "ASCII\n";
    vtk << "DATASET UNSTRUCTURED_GRID\n";
    vtk << "POINTS " << nodes_count << " double\n";
    for (int node = 0; node < nodes_count; node++)
      {
        if (displacement)
          vtk << nodes_xs[node] + displacement[node * 2 + 0] << " " << nodes_ys[node] + displacement[node * 2 + 1]
              << " 0\n";
        else
          vtk << nodes_xs[node] << " " << nodes_ys[node] << " 0\n";
      }
    vtk << "CELLS " << elements_count << " " << 3 * elements_count << "\n";
    for (int e = 0; e < elements_count; e++)
      vtk << "2 " << elements_starts[e] << " " << elements_ends[e] << "\n";
    vtk << "CELL_TYPES " << elements_count << "\n";
    for (int e = 0; e < elements_count; e++)
      vtk << "3\n"; // VTK_LINE
    vtk << "POINT_DATA " << nodes_count << "\n";
    vtk << "SCALARS AvgDisplacement double 1\n";
    vtk << "LOOKUP_TABLE default\n";
    for (int node = 0; node < nodes_count; node++)
      vtk << (displacement ? (std::abs (displacement[node * 2 + 0]) + std::abs (displacement[node * 2 + 1])) / 2 : 0.0)
          << "\n";
    vtk << "\n";
  }

private:
  int nodes_count = 0;
  int elements_count = 0;
  std::unique_ptr<data_type[]> nodes_xs;
  std::unique_ptr<data_type[]> nodes_ys;
  std::unique_ptr<int[]> elements_starts;
  std::unique_ptr<int[]> elements_ends;

public:
  std::unique_ptr<bcsr_matrix_class<data_type, index_type>> matrix;
  std::unique_ptr<data_type[]> forces_rhs;
};

#endif // BMFP_GOLDEN_GATE_BRIDGE_H
