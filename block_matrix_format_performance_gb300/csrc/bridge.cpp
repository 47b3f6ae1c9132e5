// Truss model of the Golden Gate bridge, the reference's second FEM source
// (fem_2d/golden_gate_bridge.h: golden_gate_bridge_2d<T, int, false>, the
// instantiation main.cpp:349-381 builds and solves): BCSR bs 2 stiffness of
// a 2-D pin-jointed truss (road deck of braced segments, two towers, side and
// main cables with vertical hangers) and its load vector.
//
// Geometry, element order, local stiffness arithmetic and assembly order
// follow the reference step by step, because the output is pinned bit for
// bit against the reference's own (tests/golden/bridge_f64.npz). Its quirks
// are kept on purpose:
//  - supported degrees of freedom leave zero rows and columns (no unit
//    diagonal), golden_gate_bridge.h:815-855;
//  - off-diagonal blocks are assigned, not accumulated (:829, :849);
//  - loop bounds compare an int counter with a T quotient, and one hanger
//    end is an int / T quotient truncated back to a node id (:489).
// The reference also writes "nodes", "forces" and "elements" files into the
// working directory (:180-236); this generator writes nothing.
//
// Compiled with -ffp-contract=off (separate multiplies and adds, as the
// reference compiles on x86-64), so the values are the same bits on x86 and
// Arm hosts.
#include "internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace bmfp
{
namespace
{
template <typename T> class Truss
{
public:
  Truss (T main_span, T side_span, T tower_height, T segment_length)
    : main_ (main_span), side_ (side_span), tower_h_ (tower_height), seg_ (segment_length)
  {
  }

  // Returns false when the spans give node ids outside the model (the
  // reference would write out of bounds) or non-finite coordinates.
  bool build ()
  {
    // golden_gate_bridge.h:290-295: segments along the whole deck
    const T per = (main_ + T (2) * side_) / seg_ + T (1);
    if (!(per >= T (2) && per < T (2e7)))
      return false;
    segments_ = (int) per;
    road ();
    towers ();
    side_cables ();
    main_cable ();
    const int n = next_node_;
    if ((int) xs_.size () < n)
      return false;
    for (size_t e = 0; e < lo_.size (); e++)
      if (lo_[e] < 0 || hi_[e] >= n)
        return false;
    for (int i = 0; i < n; i++)
      if (!std::isfinite (xs_[i]) || !std::isfinite (ys_[i]))
        return false;
    for (size_t e = 0; e < lo_.size (); e++)
      if (!(xs_[hi_[e]] != xs_[lo_[e]] || ys_[hi_[e]] != ys_[lo_[e]]))
        return false; // a bar of zero length
    return (int64_t) n + 2 * (int64_t) lo_.size () < INT32_MAX / 4;
  }

  int nodes () const { return next_node_; }
  int segments () const { return segments_; }
  int elements () const { return (int) lo_.size (); }

  void geometry (T *xs, T *ys, int *starts, int *ends) const
  {
    if (xs)
      std::copy (xs_.begin (), xs_.begin () + next_node_, xs);
    if (ys)
      std::copy (ys_.begin (), ys_.begin () + next_node_, ys);
    if (starts)
      std::copy (lo_.begin (), lo_.end (), starts);
    if (ends)
      std::copy (hi_.begin (), hi_.end (), ends);
  }
  int64_t blocks () const { return (int64_t) next_node_ + 2 * (int64_t) lo_.size (); }

  // golden_gate_bridge.h:573-581, 663-735, 737-860 and 170-178.
  void assemble (int *row_ptr, int *cols, T *vals, T *rhs, T window, T fy) const
  {
    const int n = next_node_;
    const int ne = (int) lo_.size ();
    // pattern: the diagonal, then both ends of every element, sorted per row
    std::vector<int> cnt (n, 1);
    for (int e = 0; e < ne; e++)
      {
        cnt[lo_[e]]++;
        cnt[hi_[e]]++;
      }
    row_ptr[0] = 0;
    for (int i = 0; i < n; i++)
      row_ptr[i + 1] = row_ptr[i] + cnt[i];
    std::vector<int> fill (n, 1);
    for (int i = 0; i < n; i++)
      cols[row_ptr[i]] = i;
    for (int e = 0; e < ne; e++)
      {
        cols[row_ptr[lo_[e]] + fill[lo_[e]]++] = hi_[e];
        cols[row_ptr[hi_[e]] + fill[hi_[e]]++] = lo_[e];
      }
    for (int i = 0; i < n; i++)
      std::sort (cols + row_ptr[i], cols + row_ptr[i + 1]);
    std::fill_n (vals, (size_t) row_ptr[n] * 4, T (0));

    auto block = [&] (int row, int col) -> T * {
      const int *b = cols + row_ptr[row], *e = cols + row_ptr[row + 1];
      return vals + (size_t) (row_ptr[row] + (std::lower_bound (b, e, col) - b)) * 4;
    };
    for (int e = 0; e < ne; e++)
      {
        T k[16];
        element_stiffness (e, k);
        const int a = lo_[e], b = hi_[e];
        const int fa[2] = { bcx_[a], bcy_[a] }, fb[2] = { bcx_[b], bcy_[b] };
        T *d = block (a, a);
        for (int i = 0; i < 2; i++)
          if (!fa[i])
            for (int j = 0; j < 2; j++)
              if (!fa[j])
                d[i * 2 + j] += k[i * 4 + j];
        T *o = block (a, b);
        for (int i = 0; i < 2; i++)
          if (!fa[i])
            for (int j = 0; j < 2; j++)
              if (!fb[j])
                o[i * 2 + j] = k[i * 4 + j + 2];
        d = block (b, b);
        for (int i = 0; i < 2; i++)
          if (!fb[i])
            for (int j = 0; j < 2; j++)
              if (!fb[j])
                d[i * 2 + j] += k[(2 + i) * 4 + j + 2];
        o = block (b, a);
        for (int i = 0; i < 2; i++)
          if (!fb[i])
            for (int j = 0; j < 2; j++)
              if (!fa[j])
                o[i * 2 + j] = k[(2 + i) * 4 + j];
      }

    if (rhs)
      {
        // a vertical load on the deck's top chord within `window` of mid-span
        // (the load functions of main.cpp:356-363)
        std::fill_n (rhs, (size_t) n * 2, T (0));
        const T mid = (main_ + side_ * T (2)) / T (2);
        for (int s = 0; s < segments_; s++)
          for (const int node : { s * 4, s * 4 + 1 })
            {
              const T x = xs_[node];
              rhs[node * 2 + 0] = T (0);
              rhs[node * 2 + 1] = (x > mid - window && x < mid + window) ? fy : T (0);
            }
      }
  }

private:
  void node (int id, T x, T y)
  {
    if (id >= (int) xs_.size ())
      {
        xs_.resize (id + 1, T (0));
        ys_.resize (id + 1, T (0));
        bcx_.resize (id + 1, 0);
        bcy_.resize (id + 1, 0);
      }
    xs_[id] = x;
    ys_[id] = y;
  }

  void fix (int id)
  {
    if (id >= (int) xs_.size ())
      node (id, T (0), T (0));
    bcx_[id] = 1;
    bcy_[id] = 1;
  }

  // Elements are numbered in the order they are made (set_element, :283-289).
  void element (int a, int b, T area)
  {
    lo_.push_back (std::min (a, b));
    hi_.push_back (std::max (a, b));
    area_.push_back (area);
  }

  T x_of (int id) const { return id < (int) xs_.size () ? xs_[id] : T (0); }

  // Deck: per segment a top pair (4s, 4s+1) and a bottom pair (4s+2, 4s+3)
  // with eight bars to the next segment, then a closing pair, :319-393.
  void road ()
  {
    const T dx = seg_ / T (2);
    fix (0);
    fix (2);
    const T top = deck_h_, bottom = deck_h_ - section_h_;
    for (int s = 0; s < segments_; s++)
      {
        const int n1 = s * 4, n2 = n1 + 1, n3 = n1 + 2, n4 = n1 + 3;
        const int n1_next = (s + 1) * 4;
        const int n3_next = s == segments_ - 1 ? n1_next + 1 : (s + 1) * 4 + 2;
        node (n1, seg_ * T (s), top);
        node (n2, seg_ * T (s) + dx, top);
        node (n3, seg_ * T (s), bottom);
        node (n4, seg_ * T (s) + dx, bottom);
        const int bars[8][2] = { { n1, n3 }, { n2, n4 }, { n1, n2 },      { n3, n4 },
                                 { n3, n2 }, { n2, n3_next }, { n2, n1_next }, { n4, n3_next } };
        for (const auto &bar : bars)
          element (bar[0], bar[1], segment_a_);
      }
    const int n1 = segments_ * 4, n3 = n1 + 1;
    node (n1, seg_ * T (segments_), top);
    node (n3, seg_ * T (segments_), bottom);
    fix (n1);
    fix (n3);
    element (n1, n3, segment_a_);
    last_road_ = n1;
    next_node_ = n3 + 1;
  }

  // Two vertical towers on fixed feet, :395-419.
  void towers ()
  {
    lt_bottom_ = next_node_++;
    lt_top_ = next_node_++;
    rt_bottom_ = next_node_++;
    rt_top_ = next_node_++;
    const T xl = std::round (side_ / seg_) * seg_ + seg_ / T (2);
    const T xr = std::round ((side_ + main_) / seg_) * seg_ + seg_ / T (2);
    node (lt_bottom_, xl, T (0));
    node (lt_top_, xl, tower_h_);
    node (rt_bottom_, xr, T (0));
    node (rt_top_, xr, tower_h_);
    fix (lt_bottom_);
    fix (rt_bottom_);
    element (lt_bottom_, lt_top_, tower_a_);
    element (rt_bottom_, rt_top_, tower_a_);
  }

  // Straight side cables from the deck ends to the tower tops, with hangers
  // to the deck's top chord, :421-500.
  void side_cables ()
  {
    // y on the line through (x1, y1) and (x2, y2): (c - a x) / b
    struct Line
    {
      T a, b, c;
      T at (T x) const { return (c - a * x) / b; }
    };
    auto line = [] (T y1, T y2, T x1, T x2) { return Line{ y1 - y2, x2 - x1, y1 * x2 - x1 * y2 }; };

    const Line left = line (deck_h_, tower_h_, T (0), x_of (lt_top_));
    element (0, next_node_, rope_a_);
    const T left_end = (side_ - seg_) / seg_;
    for (int s = 0; T (s) < left_end; s++)
      {
        const int top = next_node_++;
        node (top, seg_ * T (s) + seg_ / T (2), T (0));
        ys_[top] = left.at (xs_[top]);
        element (s * 4 + 1, top, rope_a_);
        if (s > 0)
          element (top - 1, top, spin_a_);
      }
    element (lt_top_, int (side_ / seg_) * 4 + 1, rope_a_);
    element (next_node_ - 1, lt_top_, spin_a_);

    const Line right = line (tower_h_, deck_h_, x_of (rt_top_), x_of (last_road_));
    element (rt_top_, next_node_, spin_a_);
    const T right_end = (main_ + T (2) * side_ - seg_) / seg_;
    bool first = true;
    for (int s = int ((side_ + main_ + seg_) / seg_); T (s) < right_end; s++)
      {
        const int top = next_node_++;
        node (top, seg_ * T (s) + seg_ / T (2), T (0));
        ys_[top] = right.at (xs_[top]);
        element (s * 4 + 1, top, rope_a_);
        if (!first)
          element (top - 1, top, spin_a_);
        first = false;
      }
    const T hanger = T (int (side_ + main_ + seg_ / T (2))) / seg_ * T (4) + T (1);
    element (rt_top_, int (hanger), rope_a_);
    element (next_node_ - 1, segments_ * 4, spin_a_);
  }

  // Parabolic main cable through both tower tops and 1 m above the deck at
  // mid-span, with hangers, :502-571.
  void main_cable ()
  {
    const T x1 = x_of (lt_top_), y1 = ys_[lt_top_];
    const T x2 = (main_ + T (2) * side_) / T (2), y2 = deck_h_ + T (1);
    const T x3 = x_of (rt_top_), y3 = ys_[rt_top_];
    const T A1 = x2 * x2 - (x1 * x1), B1 = x2 - x1, D1 = y2 - y1;
    const T A2 = x3 * x3 - x2 * x2, B2 = x3 - x2, D2 = y3 - y2;
    const T Bm = -(B2 / B1);
    const T A3 = Bm * A1 + A2, D3 = Bm * D1 + D2;
    const T a = D3 / A3;
    const T b = (D1 - A1 * a) / B1;
    const T c = y1 - a * x1 * x1 - b * x1;

    element (lt_top_, next_node_, spin_a_);
    const T end = (side_ + main_ - seg_) / seg_;
    bool first = true;
    for (int s = int ((side_ + seg_) / seg_); T (s) < end; s++)
      {
        const int top = next_node_++;
        node (top, seg_ * T (s) + seg_ / T (2), T (0));
        const T x = xs_[top];
        ys_[top] = a * x * x + b * x + c;
        element (s * 4 + 1, top, rope_a_);
        if (!first)
          element (top - 1, top, spin_a_);
        first = false;
      }
    element (rt_top_, next_node_ - 1, spin_a_);
  }

  // Bar stiffness in global axes, K = B^T (k' B) with k' the axial bar
  // matrix and B the rotation (:663-735), each product summed over k in order
  // from zero as the reference's matrix_mult_matrix and
  // matrix_transponse_and_mult do (:16-46).
  void element_stiffness (int e, T *K) const
  {
    const T dx = xs_[hi_[e]] - xs_[lo_[e]];
    const T dy = ys_[hi_[e]] - ys_[lo_[e]];
    const T len = std::sqrt (dx * dx + dy * dy);
    const T cs = dx / len, sn = dy / len;
    const T ae_l = area_[e] * steel_e_ / len;
    T kp[16] = {}, rot[16] = {}, tmp[16];
    kp[0] = ae_l;
    kp[2] = -ae_l;
    kp[8] = -ae_l;
    kp[10] = ae_l;
    rot[0] = cs;
    rot[1] = sn;
    rot[4] = -sn;
    rot[5] = cs;
    rot[10] = cs;
    rot[11] = sn;
    rot[14] = -sn;
    rot[15] = cs;
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++)
        {
          T sum = T (0);
          for (int k = 0; k < 4; k++)
            sum += kp[i * 4 + k] * rot[k * 4 + j];
          tmp[i * 4 + j] = sum;
        }
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++)
        {
          T sum = T (0);
          for (int k = 0; k < 4; k++)
            sum += rot[k * 4 + i] * tmp[k * 4 + j];
          K[i * 4 + j] = sum;
        }
  }

  // golden_gate_bridge.h:63-98 (every member is steel, E = 2e11 Pa)
  const T main_, side_, tower_h_, seg_;
  const T deck_h_ = T (78.0), section_h_ = T (7.62);
  const T steel_e_ = T (2e+11);
  const T spin_a_ = T (0.36), rope_a_ = T (0.06), tower_a_ = T (0.62), segment_a_ = T (0.45);

  int segments_ = 0, next_node_ = 0;
  int lt_bottom_ = 0, lt_top_ = 0, rt_bottom_ = 0, rt_top_ = 0, last_road_ = 0;
  std::vector<T> xs_, ys_;
  std::vector<int> bcx_, bcy_;
  std::vector<int> lo_, hi_;
  std::vector<T> area_;
};

template <typename T>
int gen_bridge (double main_span, double side_span, double tower_height, double segment_length, double window,
                double fy, int *n_block_rows, int64_t *nnzb, int *row_ptr, int *cols, void *vals, void *rhs)
{
  Truss<T> t ((T) main_span, (T) side_span, (T) tower_height, (T) segment_length);
  if (!t.build ())
    return fail (BMFP_ERROR_INVALID_VALUE, "bridge spans give a model outside its node range");
  if (n_block_rows)
    *n_block_rows = t.nodes ();
  if (nnzb)
    *nnzb = t.blocks ();
  if (!row_ptr)
    return BMFP_SUCCESS;
  if (!cols || !vals)
    return fail (BMFP_ERROR_INVALID_VALUE, "null array");
  t.assemble (row_ptr, cols, static_cast<T *> (vals), static_cast<T *> (rhs), (T) window, (T) fy);
  return BMFP_SUCCESS;
}
template <typename T>
int bridge_geometry (double main_span, double side_span, double tower_height, double segment_length,
                     int *n_segments, int *n_nodes, int *n_elements, void *xs, void *ys, int *starts, int *ends)
{
  Truss<T> t ((T) main_span, (T) side_span, (T) tower_height, (T) segment_length);
  if (!t.build ())
    return fail (BMFP_ERROR_INVALID_VALUE, "bridge spans give a model outside its node range");
  if (n_segments)
    *n_segments = t.segments ();
  if (n_nodes)
    *n_nodes = t.nodes ();
  if (n_elements)
    *n_elements = t.elements ();
  t.geometry (static_cast<T *> (xs), static_cast<T *> (ys), starts, ends);
  return BMFP_SUCCESS;
}

bool bridge_args_ok (int dtype, double main_span, double side_span, double tower_height, double segment_length)
{
  return dtype_ok (dtype) && segment_length > 0 && main_span > 0 && side_span > 0 && tower_height > 0
         && std::isfinite (main_span) && std::isfinite (side_span) && std::isfinite (tower_height)
         && std::isfinite (segment_length);
}
} // namespace
} // namespace bmfp

extern "C" int bmfp_golden_gate_bridge_geometry (int dtype, double main_span, double side_span,
                                                 double tower_height, double segment_length, int *n_segments,
                                                 int *n_nodes, int *n_elements, void *xs, void *ys, int *starts,
                                                 int *ends)
{
  using namespace bmfp;
  if (!bridge_args_ok (dtype, main_span, side_span, tower_height, segment_length))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid bridge arguments");
  return dtype == BMFP_R64F ? bridge_geometry<double> (main_span, side_span, tower_height, segment_length,
                                                       n_segments, n_nodes, n_elements, xs, ys, starts, ends)
                            : bridge_geometry<float> (main_span, side_span, tower_height, segment_length,
                                                      n_segments, n_nodes, n_elements, xs, ys, starts, ends);
}

extern "C" int bmfp_gen_golden_gate_bridge (int dtype, double main_span, double side_span, double tower_height,
                                            double segment_length, double load_window, double load_fy,
                                            int *n_block_rows, int64_t *nnzb, int *row_ptr, int *cols,
                                            void *values, void *rhs)
{
  using namespace bmfp;
  if (!bridge_args_ok (dtype, main_span, side_span, tower_height, segment_length) || !std::isfinite (load_window)
      || !std::isfinite (load_fy))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid bridge arguments");
  return dtype == BMFP_R64F ? gen_bridge<double> (main_span, side_span, tower_height, segment_length, load_window,
                                                  load_fy, n_block_rows, nnzb, row_ptr, cols, values, rhs)
                            : gen_bridge<float> (main_span, side_span, tower_height, segment_length, load_window,
                                                 load_fy, n_block_rows, nnzb, row_ptr, cols, values, rhs);
}
