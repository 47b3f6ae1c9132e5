// Host-side format conversions and workload generators (no GPU needed).
//
//  bmfp_bcsr_to_csr       common/matrix_converters.h:88-117
//  bmfp_csr_to_bcsr       new: the inverse, bit-exact on the converter's output
//  bmfp_transpose_blocks  common/matrix_converters.h:32-49
//  bmfp_gen_n_diag_bcsr   common/matrix_converters.h:157-196
//  bmfp_gen_band_bcsr     new: seeded +-h random band (the block-size sweep)
//  bmfp_gen_q4_elasticity new: Q4 plane-stress grid (the FEM workloads)
//
// Compiled with -ffp-contract=off so generated values are the same bits on
// x86 and Arm hosts.
#include "internal.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace bmfp
{
namespace
{
template <typename T>
void bcsr_to_csr_t (int nbr, int bs, const int *brp, const int *bc, const T *bv, int *rp, int *c,
                    T *v)
{
  int64_t off = 0;
  for (int br = 0; br < nbr; br++)
    for (int r = 0; r < bs; r++)
      {
        rp[(int64_t) br * bs + r] = (int) off;
        for (int b = brp[br]; b < brp[br + 1]; b++)
          {
            const T *src = bv + (int64_t) b * bs * bs + (int64_t) r * bs;
            const int base = bc[b] * bs;
            for (int k = 0; k < bs; k++)
              {
                c[off] = base + k;
                v[off] = src[k];
                off++;
              }
          }
      }
  rp[(int64_t) nbr * bs] = (int) off;
}

// Distinct block columns of block row br, sorted, into cols_out; returns count.
int block_columns (int br, int bs, const int *rp, const int *c, std::vector<int> &scratch)
{
  scratch.clear ();
  for (int r = 0; r < bs; r++)
    {
      const int row = br * bs + r;
      for (int e = rp[row]; e < rp[row + 1]; e++)
        scratch.push_back (c[e] / bs);
    }
  std::sort (scratch.begin (), scratch.end ());
  scratch.erase (std::unique (scratch.begin (), scratch.end ()), scratch.end ());
  return (int) scratch.size ();
}

template <typename T>
void csr_to_bcsr_fill (int n_rows, int bs, const int *rp, const int *c, const T *v,
                       const int *brp, int *bc, T *bv)
{
  const int nbr = n_rows / bs;
  std::vector<int> cols;
  std::memset (bv, 0, sizeof (T) * (size_t) brp[nbr] * bs * bs);
  for (int br = 0; br < nbr; br++)
    {
      block_columns (br, bs, rp, c, cols);
      std::copy (cols.begin (), cols.end (), bc + brp[br]);
      for (int r = 0; r < bs; r++)
        {
          const int row = br * bs + r;
          for (int e = rp[row]; e < rp[row + 1]; e++)
            {
              const int bcol = c[e] / bs, k = c[e] % bs;
              const int pos = (int) (std::lower_bound (cols.begin (), cols.end (), bcol) - cols.begin ());
              bv[((int64_t) brp[br] + pos) * bs * bs + (int64_t) r * bs + k] = v[e];
            }
        }
    }
}

template <typename T>
void transpose_t (int nbr, int bs, const int *rp, const T *v, T *out)
{
  for (int br = 0; br < nbr; br++)
    for (int b = rp[br]; b < rp[br + 1]; b++)
      {
        const T *o = v + (int64_t) b * bs * bs;
        T *n = out + (int64_t) b * bs * bs;
        for (int i = 0; i < bs; i++)
          for (int j = 0; j < bs; j++)
            n[j * bs + i] = o[i * bs + j];
      }
}

// (data_type(column) + i) / n_rows, with the unsigned i converted to
// data_type first (common/matrix_converters.h:189).
template <typename T>
void gen_n_diag_t (int n_rows, int bpr, int bs, int *rp, int *c, T *v)
{
  int64_t block = 0;
  for (int row = 0; row < n_rows; row++)
    {
      rp[row] = row * bpr;
      int first;
      if (row < bpr / 2)
        first = 0;
      else if (row > n_rows - bpr)
        first = n_rows - bpr;
      else
        first = row - bpr / 2;
      for (int el = 0; el < bpr; el++)
        {
          const int col = first + el;
          T *blk = v + block * bs * bs;
          for (unsigned i = 0; i < (unsigned) (bs * bs); i++)
            blk[i] = ((T) col + (T) i) / (T) n_rows;
          c[block++] = col;
        }
    }
  rp[n_rows] = n_rows * bpr;
}

// ---- SplitMix64 streams (Steele, Lea & Flood, OOPSLA 2014).
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

inline uint64_t splitmix_next (uint64_t &s)
{
  s += kGolden;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Independent stream per (seed, stream, index): the generators can be filled
// in any order and the result depends only on the arguments.
inline uint64_t row_state (uint64_t seed, uint64_t stream, uint64_t row)
{
  uint64_t s = row * kGolden + (seed * 0xD1B54A32D192ED03ull + stream * 0x8CB92BA72F3D8DD7ull);
  return splitmix_next (s);
}

inline double uniform_pm1 (uint64_t z)
{
  return (double) (z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

struct Band
{
  int lo, width, k;
};

inline Band band_of (int row, int nbr, int bpr, int h)
{
  const int lo = std::max (0, row - h);
  const int hi = std::min (nbr - 1, row + h);
  Band b{ lo, hi - lo + 1, 0 };
  b.k = std::min (bpr, b.width);
  return b;
}

template <typename T>
void gen_band_fill (int nbr, int bpr, int h, int bs, uint64_t seed, const int *rp, int *c, T *v)
{
  std::vector<int> perm;
  const int E = bs * bs;
  for (int row = 0; row < nbr; row++)
    {
      const Band b = band_of (row, nbr, bpr, h);
      perm.resize ((size_t) b.width);
      for (int i = 0; i < b.width; i++)
        perm[i] = i;
      uint64_t st = row_state (seed, 0, (uint64_t) row);
      for (int j = 0; j < b.k; j++)
        {
          const uint64_t z = splitmix_next (st);
          const int pick = j + (int) (z % (uint64_t) (b.width - j));
          std::swap (perm[j], perm[pick]);
        }
      int *rc = c + rp[row];
      for (int j = 0; j < b.k; j++)
        rc[j] = perm[j] + b.lo;
      std::sort (rc, rc + b.k);
      uint64_t vs = row_state (seed, 1, (uint64_t) row);
      T *rv = v + (int64_t) rp[row] * E;
      for (int j = 0; j < b.k * E; j++)
        rv[j] = (T) uniform_pm1 (splitmix_next (vs));
    }
}

// Bilinear quad, plane stress, unit square, thickness 1: K = sum over the
// 2x2 Gauss points of B^T D B * det(J) with det(J) = 1/4. Node order is
// counter-clockwise from the lower-left corner, DOFs (ux, uy) per node.
void q4_element (double E, double nu, double ke[8][8])
{
  const double f = E / (1.0 - nu * nu);
  const double D[3][3] = { { f, f * nu, 0.0 }, { f * nu, f, 0.0 }, { 0.0, 0.0, f * (1.0 - nu) / 2.0 } };
  const double xn[4] = { -1.0, 1.0, 1.0, -1.0 };
  const double yn[4] = { -1.0, -1.0, 1.0, 1.0 };
  const double g = 1.0 / std::sqrt (3.0);
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 8; j++)
      ke[i][j] = 0.0;
  for (int gx = 0; gx < 2; gx++)
    for (int gy = 0; gy < 2; gy++)
      {
        const double xi = gx ? g : -g, eta = gy ? g : -g;
        double B[3][8] = {};
        for (int a = 0; a < 4; a++)
          {
            // dN/dx = dN/dxi * 2/hx, dN/dy = dN/deta * 2/hy with hx = hy = 1
            const double dx = 0.25 * xn[a] * (1.0 + eta * yn[a]) * 2.0;
            const double dy = 0.25 * yn[a] * (1.0 + xi * xn[a]) * 2.0;
            B[0][2 * a] = dx;
            B[1][2 * a + 1] = dy;
            B[2][2 * a] = dy;
            B[2][2 * a + 1] = dx;
          }
        double DB[3][8];
        for (int r = 0; r < 3; r++)
          for (int j = 0; j < 8; j++)
            DB[r][j] = D[r][0] * B[0][j] + D[r][1] * B[1][j] + D[r][2] * B[2][j];
        for (int i = 0; i < 8; i++)
          for (int j = 0; j < 8; j++)
            ke[i][j] += (B[0][i] * DB[0][j] + B[1][i] * DB[1][j] + B[2][i] * DB[2][j]) * 0.25;
      }
}

inline int q4_row_len (int i, int j, int nx, int ny)
{
  const int cx = (i > 0) + 1 + (i < nx - 1);
  const int cy = (j > 0) + 1 + (j < ny - 1);
  return cx * cy;
}

template <typename T>
void q4_fill (int nx, int ny, double E, double nu, const int *rp, int *cols, T *vals, T *rhs)
{
  const int n_nodes = nx * ny;
  // Pattern: the full 3x3 node stencil, sorted (row-major node order).
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++)
      {
        int *rc = cols + rp[j * nx + i];
        int k = 0;
        for (int dj = -1; dj <= 1; dj++)
          for (int di = -1; di <= 1; di++)
            {
              const int ii = i + di, jj = j + dj;
              if (ii >= 0 && ii < nx && jj >= 0 && jj < ny)
                rc[k++] = jj * nx + ii;
            }
      }
  // Accumulate element contributions in double, element by element.
  std::vector<double> acc ((size_t) rp[n_nodes] * 4, 0.0);
  double ke[8][8];
  q4_element (E, nu, ke);
  auto block_of = [&] (int row_node, int col_node) -> double * {
    const int *rc = cols + rp[row_node];
    const int len = rp[row_node + 1] - rp[row_node];
    const int pos = (int) (std::lower_bound (rc, rc + len, col_node) - rc);
    return acc.data () + ((size_t) rp[row_node] + pos) * 4;
  };
  for (int j = 0; j + 1 < ny; j++)
    for (int i = 0; i + 1 < nx; i++)
      {
        const int nodes[4] = { j * nx + i, j * nx + i + 1, (j + 1) * nx + i + 1, (j + 1) * nx + i };
        for (int a = 0; a < 4; a++)
          for (int b = 0; b < 4; b++)
            {
              double *blk = block_of (nodes[a], nodes[b]);
              for (int p = 0; p < 2; p++)
                for (int q = 0; q < 2; q++)
                  blk[p * 2 + q] += ke[2 * a + p][2 * b + q];
            }
      }
  // Clamp the left column: zero rows and columns of its DOFs, unit diagonal.
  for (int row = 0; row < n_nodes; row++)
    {
      const bool row_clamped = (row % nx) == 0;
      for (int e = rp[row]; e < rp[row + 1]; e++)
        {
          double *blk = acc.data () + (size_t) e * 4;
          const bool col_clamped = (cols[e] % nx) == 0;
          if (row_clamped || col_clamped)
            {
              for (int t = 0; t < 4; t++)
                blk[t] = 0.0;
              if (row_clamped && cols[e] == row)
                blk[0] = blk[3] = 1.0;
            }
        }
    }
  for (size_t t = 0; t < acc.size (); t++)
    vals[t] = (T) acc[t];
  if (rhs)
    for (int row = 0; row < n_nodes; row++)
      {
        rhs[2 * row] = 0;
        rhs[2 * row + 1] = (row % nx == nx - 1) ? (T) -1.0 : (T) 0.0;
      }
}
} // namespace
} // namespace bmfp

using namespace bmfp;

extern "C" {

int bmfp_bcsr_to_csr (int dtype, int nbr, int bs, const int *brp, const int *bc, const void *bv,
                      int *rp, int *c, void *v)
{
  if (!dtype_ok (dtype) || nbr < 0 || bs < 1 || !brp || !rp)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if (brp[nbr] > 0 && (!bc || !bv || !c || !v))
    return fail (BMFP_ERROR_INVALID_VALUE, "null array");
  if ((int64_t) brp[nbr] * bs * bs > INT32_MAX)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "more than 2^31-1 entries");
  if (dtype == BMFP_R64F)
    bcsr_to_csr_t (nbr, bs, brp, bc, (const double *) bv, rp, c, (double *) v);
  else
    bcsr_to_csr_t (nbr, bs, brp, bc, (const float *) bv, rp, c, (float *) v);
  return BMFP_SUCCESS;
}

int bmfp_csr_to_bcsr (int dtype, int n_rows, int n_cols, int bs, const int *rp, const int *c,
                      const void *v, int *brp, int64_t *nnzb, int *bc, void *bv)
{
  if (!dtype_ok (dtype) || n_rows < 0 || n_cols < 0 || bs < 1 || !rp || !brp)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if (n_rows % bs || n_cols % bs)
    return fail (BMFP_ERROR_INVALID_VALUE, "matrix %d x %d is not a whole number of %d x %d blocks",
                 n_rows, n_cols, bs, bs);
  const int nbr = n_rows / bs;
  if (!bc && !bv)
    {
      for (int64_t e = 0; e < rp[n_rows]; e++)
        if (c[e] < 0 || c[e] >= n_cols)
          return fail (BMFP_ERROR_INVALID_VALUE, "column %d out of range at entry %lld", c[e],
                       (long long) e);
      std::vector<int> scratch;
      int64_t total = 0;
      brp[0] = 0;
      for (int br = 0; br < nbr; br++)
        {
          total += block_columns (br, bs, rp, c, scratch);
          if (total > INT32_MAX)
            return fail (BMFP_ERROR_NOT_SUPPORTED, "more than 2^31-1 blocks");
          brp[br + 1] = (int) total;
        }
      if (nnzb)
        *nnzb = total;
      return BMFP_SUCCESS;
    }
  if (!bc || !bv || (rp[n_rows] > 0 && (!c || !v)))
    return fail (BMFP_ERROR_INVALID_VALUE, "null array");
  if (dtype == BMFP_R64F)
    csr_to_bcsr_fill (n_rows, bs, rp, c, (const double *) v, brp, bc, (double *) bv);
  else
    csr_to_bcsr_fill (n_rows, bs, rp, c, (const float *) v, brp, bc, (float *) bv);
  if (nnzb)
    *nnzb = brp[nbr];
  return BMFP_SUCCESS;
}

int bmfp_transpose_blocks (int dtype, int nbr, int bs, const int *rp, const void *v, void *out)
{
  if (!dtype_ok (dtype) || nbr < 0 || bs < 1 || !rp || (rp[nbr] > 0 && (!v || !out)))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if (dtype == BMFP_R64F)
    transpose_t (nbr, bs, rp, (const double *) v, (double *) out);
  else
    transpose_t (nbr, bs, rp, (const float *) v, (float *) out);
  return BMFP_SUCCESS;
}

int bmfp_gen_n_diag_bcsr (int dtype, int n_rows, int bpr, int bs, int *rp, int *c, void *v)
{
  if (!dtype_ok (dtype) || n_rows < 1 || bpr < 1 || bpr > n_rows || bs < 1 || !rp || !c || !v)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if ((int64_t) n_rows * bpr * bs * bs > INT32_MAX)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "more than 2^31-1 values");
  if (dtype == BMFP_R64F)
    gen_n_diag_t (n_rows, bpr, bs, rp, c, (double *) v);
  else
    gen_n_diag_t (n_rows, bpr, bs, rp, c, (float *) v);
  return BMFP_SUCCESS;
}

int bmfp_gen_band_bcsr (int dtype, int nbr, int bpr, int h, int bs, uint64_t seed, int *rp,
                        int64_t *nnzb, int *c, void *v)
{
  if (!dtype_ok (dtype) || nbr < 0 || bpr < 1 || h < 0 || bs < 1 || !rp)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if (!c && !v)
    {
      int64_t total = 0;
      rp[0] = 0;
      for (int row = 0; row < nbr; row++)
        {
          total += band_of (row, nbr, bpr, h).k;
          if (total * bs * bs > INT32_MAX)
            return fail (BMFP_ERROR_NOT_SUPPORTED, "more than 2^31-1 values");
          rp[row + 1] = (int) total;
        }
      if (nnzb)
        *nnzb = total;
      return BMFP_SUCCESS;
    }
  if (!c || !v)
    return fail (BMFP_ERROR_INVALID_VALUE, "null array");
  if (dtype == BMFP_R64F)
    gen_band_fill (nbr, bpr, h, bs, seed, rp, c, (double *) v);
  else
    gen_band_fill (nbr, bpr, h, bs, seed, rp, c, (float *) v);
  if (nnzb)
    *nnzb = rp[nbr];
  return BMFP_SUCCESS;
}

int bmfp_gen_uniform_vector (int dtype, int64_t n, uint64_t seed, uint64_t stream, void *out)
{
  if (!dtype_ok (dtype) || n < 0 || (n > 0 && !out))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  for (int64_t i = 0; i < n; i++)
    {
      const double u = uniform_pm1 (row_state (seed, stream, (uint64_t) i));
      if (dtype == BMFP_R64F)
        ((double *) out)[i] = u;
      else
        ((float *) out)[i] = (float) u;
    }
  return BMFP_SUCCESS;
}

int bmfp_gen_q4_elasticity (int dtype, int nx, int ny, double young, double poisson, int *rp,
                            int64_t *nnzb, int *c, void *v, void *rhs)
{
  if (!dtype_ok (dtype) || nx < 2 || ny < 2 || !rp || !(poisson > -1.0 && poisson < 0.5))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  const int64_t n_nodes = (int64_t) nx * ny;
  if (n_nodes * 9 * 4 > INT32_MAX)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "grid too large for 32-bit indices");
  if (!c && !v)
    {
      int64_t total = 0;
      rp[0] = 0;
      for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
          {
            total += q4_row_len (i, j, nx, ny);
            rp[j * nx + i + 1] = (int) total;
          }
      if (nnzb)
        *nnzb = total;
      return BMFP_SUCCESS;
    }
  if (!c || !v)
    return fail (BMFP_ERROR_INVALID_VALUE, "null array");
  if (dtype == BMFP_R64F)
    q4_fill (nx, ny, young, poisson, rp, c, (double *) v, (double *) rhs);
  else
    q4_fill (nx, ny, young, poisson, rp, c, (float *) v, (float *) rhs);
  if (nnzb)
    *nnzb = rp[n_nodes];
  return BMFP_SUCCESS;
}

} // extern "C"

// ------------------------------------------------------------ MatrixMarket

namespace
{
struct MmEntry
{
  int row, col;
  int64_t order; // position in the file, to sum duplicates in file order
  double value;
};

struct MmFile
{
  int n_rows = 0, n_cols = 0;
  std::vector<MmEntry> entries;
};

std::string lower (std::string t)
{
  for (char &ch : t)
    ch = (char) std::tolower ((unsigned char) ch);
  return t;
}

// Reads the whole file: banner, comments, size line, entries (1-based).
int mm_parse (const char *path, MmFile &out)
{
  FILE *f = std::fopen (path, "r");
  if (!f)
    return fail (BMFP_ERROR_INVALID_VALUE, "cannot open %s", path);
  struct Closer
  {
    FILE *f;
    ~Closer () { std::fclose (f); }
  } closer{ f };
  char line[4096];
  if (!std::fgets (line, sizeof line, f))
    return fail (BMFP_ERROR_INVALID_VALUE, "%s: empty file", path);
  char w[5][64] = {};
  if (std::sscanf (line, "%63s %63s %63s %63s %63s", w[0], w[1], w[2], w[3], w[4]) != 5
      || lower (w[0]) != "%%matrixmarket" || lower (w[1]) != "matrix")
    return fail (BMFP_ERROR_INVALID_VALUE, "%s: not a MatrixMarket matrix banner", path);
  const std::string format = lower (w[2]), field = lower (w[3]), symmetry = lower (w[4]);
  if (format != "coordinate")
    return fail (BMFP_ERROR_NOT_SUPPORTED, "%s: only coordinate (sparse) files are read", path);
  const bool pattern = field == "pattern";
  if (!pattern && field != "real" && field != "double" && field != "integer")
    return fail (BMFP_ERROR_NOT_SUPPORTED, "%s: field '%s' is not read", path, field.c_str ());
  int mirror = 0; // 0 general, 1 symmetric, -1 skew-symmetric
  if (symmetry == "symmetric")
    mirror = 1;
  else if (symmetry == "skew-symmetric")
    mirror = -1;
  else if (symmetry != "general")
    return fail (BMFP_ERROR_NOT_SUPPORTED, "%s: symmetry '%s' is not read", path, symmetry.c_str ());
  long long m = -1, n = -1, nz = -1;
  while (std::fgets (line, sizeof line, f))
    {
      if (line[0] == '%')
        continue;
      if (std::sscanf (line, "%lld %lld %lld", &m, &n, &nz) == 3)
        break;
      bool blank = true;
      for (const char *c = line; *c; c++)
        blank = blank && std::isspace ((unsigned char) *c);
      if (!blank)
        return fail (BMFP_ERROR_INVALID_VALUE, "%s: bad size line", path);
    }
  if (m < 0 || n < 0 || nz < 0 || m > INT32_MAX || n > INT32_MAX)
    return fail (BMFP_ERROR_INVALID_VALUE, "%s: bad or missing size line", path);
  if ((mirror != 0) && m != n)
    return fail (BMFP_ERROR_INVALID_VALUE, "%s: symmetric file of a non-square matrix", path);
  out.n_rows = (int) m;
  out.n_cols = (int) n;
  out.entries.clear ();
  out.entries.reserve ((size_t) nz * (mirror ? 2 : 1));
  int64_t k = 0;
  while (k < nz && std::fgets (line, sizeof line, f))
    {
      if (line[0] == '%')
        continue;
      char *p = line, *end = nullptr;
      const long long i = std::strtoll (p, &end, 10);
      if (end == p)
        {
          bool blank = true;
          for (const char *c = line; *c; c++)
            blank = blank && std::isspace ((unsigned char) *c);
          if (blank)
            continue;
          return fail (BMFP_ERROR_INVALID_VALUE, "%s: bad entry %lld", path, (long long) k + 1);
        }
      p = end;
      const long long j = std::strtoll (p, &end, 10);
      if (end == p)
        return fail (BMFP_ERROR_INVALID_VALUE, "%s: bad entry %lld", path, (long long) k + 1);
      p = end;
      double v = 1.0;
      if (!pattern)
        {
          v = std::strtod (p, &end);
          if (end == p)
            return fail (BMFP_ERROR_INVALID_VALUE, "%s: entry %lld has no value", path, (long long) k + 1);
        }
      if (i < 1 || i > m || j < 1 || j > n)
        return fail (BMFP_ERROR_INVALID_VALUE, "%s: entry %lld (%lld, %lld) outside %lld x %lld", path,
                     (long long) k + 1, i, j, m, n);
      out.entries.push_back ({ (int) (i - 1), (int) (j - 1), 2 * k, v });
      if (mirror && i != j)
        out.entries.push_back ({ (int) (j - 1), (int) (i - 1), 2 * k + 1, mirror * v });
      k++;
    }
  if (k != nz)
    return fail (BMFP_ERROR_INVALID_VALUE, "%s: %lld of %lld entries present", path, (long long) k, nz);
  // Rows ascending, columns ascending, duplicates kept in file order.
  std::sort (out.entries.begin (), out.entries.end (), [] (const MmEntry &a, const MmEntry &b) {
    if (a.row != b.row)
      return a.row < b.row;
    if (a.col != b.col)
      return a.col < b.col;
    return a.order < b.order;
  });
  return BMFP_SUCCESS;
}

template <typename T> void mm_fill (const MmFile &mf, int *rp, int *cols, T *vals)
{
  std::fill (rp, rp + mf.n_rows + 1, 0);
  int64_t e = -1;
  int prev_row = -1, prev_col = -1;
  double acc = 0.0;
  auto flush = [&] () {
    if (e >= 0)
      vals[e] = (T) acc;
  };
  for (const MmEntry &m : mf.entries)
    {
      if (m.row == prev_row && m.col == prev_col)
        {
          acc += m.value;
          continue;
        }
      flush ();
      e++;
      cols[e] = m.col;
      rp[m.row + 1]++;
      acc = m.value;
      prev_row = m.row;
      prev_col = m.col;
    }
  flush ();
  for (int r = 0; r < mf.n_rows; r++)
    rp[r + 1] += rp[r];
}

int64_t mm_distinct (const MmFile &mf)
{
  int64_t nnz = 0;
  for (size_t k = 0; k < mf.entries.size (); k++)
    if (k == 0 || mf.entries[k].row != mf.entries[k - 1].row || mf.entries[k].col != mf.entries[k - 1].col)
      nnz++;
  return nnz;
}
} // namespace

int bmfp_mm_read_csr (const char *path, int dtype, int *n_rows, int *n_cols, int64_t *nnz, int *row_ptr,
                      int *cols, void *values)
{
  if (!path || !dtype_ok (dtype) || !n_rows || !n_cols || !nnz)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  MmFile mf;
  int st = mm_parse (path, mf);
  if (st != BMFP_SUCCESS)
    return st;
  const int64_t distinct = mm_distinct (mf);
  if (distinct > INT32_MAX)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "more than 2^31-1 entries");
  *n_rows = mf.n_rows;
  *n_cols = mf.n_cols;
  *nnz = distinct;
  if (!row_ptr)
    return BMFP_SUCCESS;
  if (distinct > 0 && (!cols || !values))
    return fail (BMFP_ERROR_INVALID_VALUE, "null output array");
  if (dtype == BMFP_R64F)
    mm_fill (mf, row_ptr, cols, (double *) values);
  else
    mm_fill (mf, row_ptr, cols, (float *) values);
  return BMFP_SUCCESS;
}
