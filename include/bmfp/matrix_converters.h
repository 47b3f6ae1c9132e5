// Drop-in replacement for the reference's common/matrix_converters.h.
//
// Same class templates, members and functions (bcsr_matrix_class,
// csr_matrix_class, gen_n_diag_bcsr; common/matrix_converters.h:13-196), so
// code written against the reference compiles unchanged. The conversions and
// the generator run in libbmfp.so (bmfp_bcsr_to_csr, bmfp_transpose_blocks,
// bmfp_gen_n_diag_bcsr), bit-exact with the reference's output. Supported
// instantiations are the reference's: float or double values with 32-bit
// indices (int or unsigned).
#ifndef BMFP_MATRIX_CONVERTERS_H
#define BMFP_MATRIX_CONVERTERS_H

#include "bmfp.h"

#include <algorithm>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace bmfp_detail
{
template <typename T> constexpr int dtype_of ()
{
  static_assert (std::is_same<T, float>::value || std::is_same<T, double>::value,
                 "libbmfp handles float and double values");
  return std::is_same<T, double>::value ? BMFP_R64F : BMFP_R32F;
}

template <typename I> constexpr void check_index ()
{
  static_assert (std::is_integral<I>::value && sizeof (I) == 4, "libbmfp uses 32-bit indices (int or unsigned)");
}

inline void throw_on (int status, const char *what)
{
  if (status != BMFP_SUCCESS)
    throw std::runtime_error (std::string (what) + ": " + bmfp_last_error ());
}
} // namespace bmfp_detail

template <typename data_type, typename index_type>
class bcsr_matrix_class
{
public:
  bcsr_matrix_class (index_type n_rows_arg, index_type n_cols_arg, index_type bs_arg, index_type nnzb_arg)
    : n_rows (n_rows_arg), n_cols (n_cols_arg), bs (bs_arg), nnzb (nnzb_arg),
      values (new data_type[(size_t) nnzb_arg * bs_arg * bs_arg]),
      columns (new index_type[(size_t) nnzb_arg]),
      row_ptr (new index_type[(size_t) n_rows_arg + 1])
  {
    bmfp_detail::check_index<index_type> ();
  }

  // Row-major blocks -> column-major blocks into new_values (nnzb*bs*bs).
  void transpose_blocks (data_type *new_values)
  {
    bmfp_detail::throw_on (bmfp_transpose_blocks (bmfp_detail::dtype_of<data_type> (), (int) n_rows, (int) bs,
                                                  reinterpret_cast<const int *> (row_ptr.get ()), values.get (),
                                                  new_values),
                           "transpose_blocks");
  }

  index_type size () const { return nnzb * bs * bs; }

  data_type *get_block_data (index_type row, index_type block_in_row)
  {
    return values.get () + (size_t) (row_ptr[row] + block_in_row) * bs * bs;
  }

  // Block of block row `row` stored at block column `column` (columns sorted).
  data_type *get_block_data_by_column (index_type row, index_type column)
  {
    const index_type *first = columns.get () + row_ptr[row];
    const index_type *last = columns.get () + row_ptr[row + 1];
    return get_block_data (row, (index_type) (std::lower_bound (first, last, column) - first));
  }

public:
  const index_type n_rows{};
  const index_type n_cols{};
  const index_type bs{};
  const index_type nnzb{};
  const std::unique_ptr<data_type[]> values;
  const std::unique_ptr<index_type[]> columns;
  const std::unique_ptr<index_type[]> row_ptr;
};

template <typename data_type, typename index_type>
class csr_matrix_class
{
public:
  explicit csr_matrix_class (const bcsr_matrix_class<data_type, index_type> &m)
    : n_rows (m.n_rows * m.bs), n_cols (m.n_cols * m.bs), nnz (m.nnzb * m.bs * m.bs),
      values (new data_type[(size_t) m.nnzb * m.bs * m.bs]),
      columns (new index_type[(size_t) m.nnzb * m.bs * m.bs]),
      row_ptr (new index_type[(size_t) m.n_rows * m.bs + 1])
  {
    bmfp_detail::check_index<index_type> ();
    bmfp_detail::throw_on (bmfp_bcsr_to_csr (bmfp_detail::dtype_of<data_type> (), (int) m.n_rows, (int) m.bs,
                                             reinterpret_cast<const int *> (m.row_ptr.get ()),
                                             reinterpret_cast<const int *> (m.columns.get ()), m.values.get (),
                                             reinterpret_cast<int *> (row_ptr.get ()),
                                             reinterpret_cast<int *> (columns.get ()), values.get ()),
                           "csr_matrix_class");
  }

  // MatrixMarket coordinate file, 1-based indices, one "%d %d %10.20g" line
  // per stored entry (the text common/matrix_converters.h:119-144 writes).
  void write_mm (const std::string &filename)
  {
    std::FILE *fp = std::fopen (filename.c_str (), "w");
    if (!fp)
      throw std::runtime_error ("write_mm: cannot open " + filename);
    std::fprintf (fp, "%%%%MatrixMarket matrix coordinate real general\n");
    std::fprintf (fp, "%d %d %d\n", (int) n_rows, (int) n_cols, (int) nnz);
    for (index_type r = 0; r < n_rows; r++)
      for (index_type e = row_ptr[r]; e < row_ptr[r + 1]; e++)
        std::fprintf (fp, "%d %d %10.20g\n", (int) r + 1, (int) columns[e] + 1, (double) values[e]);
    std::fclose (fp);
  }

public:
  const index_type n_rows{};
  const index_type n_cols{};
  const index_type nnz{};
  const std::unique_ptr<data_type[]> values;
  const std::unique_ptr<index_type[]> columns;
  const std::unique_ptr<index_type[]> row_ptr;
};

// The reference's contiguous-band generator: blocks_per_row consecutive
// block columns around the diagonal, value (column + i) / n_rows.
template <typename data_type, typename index_type>
std::unique_ptr<bcsr_matrix_class<data_type, index_type>>
gen_n_diag_bcsr (index_type n_rows_arg, index_type blocks_per_row, index_type bs_arg)
{
  std::unique_ptr<bcsr_matrix_class<data_type, index_type>> m (
    new bcsr_matrix_class<data_type, index_type> (n_rows_arg, n_rows_arg, bs_arg, blocks_per_row * n_rows_arg));
  bmfp_detail::throw_on (bmfp_gen_n_diag_bcsr (bmfp_detail::dtype_of<data_type> (), (int) n_rows_arg,
                                               (int) blocks_per_row, (int) bs_arg,
                                               reinterpret_cast<int *> (m->row_ptr.get ()),
                                               reinterpret_cast<int *> (m->columns.get ()), m->values.get ()),
                         "gen_n_diag_bcsr");
  return m;
}

#endif // BMFP_MATRIX_CONVERTERS_H
