// BiCGStab engines shared by the solver, batch and serving entry points.
#pragma once

#include "internal.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace bmfp
{
// Device-resident scalars of one BiCGStab solve. Each kernel that completes
// a set of dot products (start, phase 2, phase 4, phase 5) has its last CTA
// to finish sum every CTA's partials, in a fixed order, and derive the
// scalars the next phases read (alpha, omega, or beta and the tests that
// open an iteration); the other kernels only read them. So each scalar is
// computed once per kernel, by one thread, and no kernel reads a field it
// writes itself.
//
// Residual replacement (H. A. van der Vorst and Q. Ye, "Residual replacement
// strategies for Krylov subspace iterative methods for the convergence of
// true residuals", SIAM J. Sci. Comput. 22, 2000; the variant with group
// update): dev bounds the deviation between the recursive residual r and the
// true b - A x that rounding has accumulated since the last replacement,
//   dev_i = dev_{i-1} + eps (cA ||x'_i|| + ||r_i||),
// with x' the updates accumulated since then and cA = (entries per row) *
// ||A||_inf. When dev crosses kReplaceThreshold * ||r|| (from below, and
// dev > 1.1 dev0), the accumulated updates are folded into the group base g
// and r is replaced by the true residual c - A g. This keeps the recursive
// residual honest near convergence, so a solve stopped on it meets the
// tolerance in b - A x as well.
struct DevState
{
  double rho;      // (rh, r) of the current iteration
  double rho_prev; // previous iteration's rho
  double alpha;    // set by phase 2's last CTA
  double omega;    // set by phase 4's last CTA
  double beta;     // of the next p update
  double norm_b;   // ||r0|| (set by the first decision)
  double rr;       // last (r, r)
  double tol;      // stop when sqrt(rr) / norm_b < tol
  double eps;      // unit roundoff of the working precision; 0 = no replacement
  double cA;       // max entries per scalar row * max absolute row sum
  double dev;      // deviation bound since the last replacement
  double dev0;     // its value at the last replacement
  double nr_prev;  // ||r|| at the previous decision
  const void *c;   // right-hand side of the run (b, or a restart's residual)
  // done and rep_now side by side (8-byte aligned): every phase reads both
  // with one load at its start.
  int done;        // set by a decision; every kernel returns early once set
  int rep_now;     // this iteration replaces r by the true residual
  int iter;        // iterations completed
  int max_iter;
  int status;      // 0 running, 1 converged, 2 iteration limit, 3 breakdown
  int replacements;
  unsigned arrive; // CTAs of the running kernel that have written their partials
  unsigned gen;    // grid barriers passed by the persistent iteration kernel
  int fault;       // a grid barrier of that kernel gave up waiting
  int pad;
};

// Replacement threshold on dev / ||r|| (van der Vorst and Ye use sqrt(eps),
// which replaces tens of times per solve here). With cA's generous bound, a
// larger threshold places the replacements deeper in the convergence: 1e-2
// measured best on the Q4 elasticity family (every grid of the uneven batch
// ends below 1e-10 in b - A x with one or two replacements; 1000x250 takes
// 4021 iterations, against 4605 with 1e-3 and six replacements).
constexpr double kReplaceThreshold = 1e-2;

static_assert (offsetof (DevState, done) % 8 == 0 && offsetof (DevState, rep_now) == offsetof (DevState, done) + 4,
               "done and rep_now must form one aligned 8-byte word");

enum
{
  kStateRunning = 0,
  kStateConverged = 1,
  kStateMaxIter = 2,
  kStateBreakdown = 3
};

// Whole-GPU BiCGStab on one matrix: five fused phases per iteration over all
// rows on a fixed grid, either as phase kernels captured in a CUDA graph of
// `chunk` iterations or as one persistent cooperative kernel per `chunk`
// iterations with grid barriers between the phases (the same bits on the same
// grid). Dot products are per-CTA partials summed in a fixed order by the
// CTA that finishes the phase last, so a solve is deterministic for a given
// grid.
//
// Every run solves A e = c from e = 0 (c = b for a fresh solve, c = the true
// residual for a restart): the updates accumulate in xp, are folded into the
// group base g at each residual replacement, and the run's result g + xp
// goes into x when the run ends (x = e for a fresh solve, x += e for a
// restart). Between runs x holds the solution.
class WideEngine
{
public:
  WideEngine () = default;
  ~WideEngine ();
  WideEngine (const WideEngine &) = delete;
  WideEngine &operator= (const WideEngine &) = delete;

  // precond: BMFP_PRECOND_NONE, _JACOBI (point) or _BLOCK_JACOBI (bs <= 8).
  // launch_mode: enum bmfp_launch_mode.
  int init (const bmfp_matrix_s *A, int precond, int chunk, cudaStream_t stream, int ctas_per_sm = 4,
            int launch_mode = 0);
  // Residual replacement on (default for FP64 engines) or off (the
  // reference's plain recurrences; FP32 engines always run without it).
  void set_replacement (bool on) { replace_ = on && dtype_ == BMFP_R64F; }
  // Start a solve of A x = b from x0 = 0 (b on the device, engine dtype; it
  // must stay valid until the run ends: replacements read it).
  int start_zero (const void *d_b, double tol, int max_iter, cudaStream_t stream);
  // Restart from the current x with the residual given in d_r (true residual;
  // kept until the run ends, as d_b above).
  // norm_b > 0 sets the reference norm of the convergence test (an engine that
  // never ran start_zero has none); norm_b <= 0 keeps the previous one.
  // iter0 >= 0 restarts the iteration count there (a new solve on an engine
  // whose last run belonged to an earlier one); -1 keeps counting.
  // new_shadow: the shadow residual is r0 perturbed elementwise
  // (shadow_factor) instead of r0 itself, for a restart after a breakdown.
  int start_residual (const void *d_r, double tol, int max_iter_total, double norm_b,
                      cudaStream_t stream, int iter0 = -1, bool new_shadow = false);
  // Runs graphs (or persistent launches) until the device sets done, then
  // writes the run's result
  // into x; returns the final state. With d_snapshot, the run's iterate is
  // copied there each time the recursive residual has fallen 4x below the
  // last copy (and below snapshot_rr on entry), and *snapshot_rr receives
  // the (r, r) of the copy; a run that ends above that point (breakdown,
  // iteration limit on an erratic stretch) returns the copy instead, with
  // out->rr set to its (r, r). A residual that grows 1e16-fold over the best
  // seen, or turns non-finite, stops the run as a breakdown, and so does
  // (stall > 0) a best residual that has not halved within `stall`
  // iterations of the start or of its last halving.
  int run (cudaStream_t stream, DevState *out, void *d_snapshot = nullptr, double *snapshot_rr = nullptr,
           int stall = 0);
  // r = b - A x, returns ||r||^2 and ||b||^2 (synchronises the stream).
  int true_residual (const void *d_b, void *d_r, double *rr, double *bb, cudaStream_t stream);

  int dtype () const { return dtype_; }
  int64_t n () const { return n_; }
  void *x () const { return x_; }
  void *scratch () const { return t_; }
  const bmfp_matrix_s *matrix () const { return A_; }

private:
  int capture (cudaStream_t stream);
  int launch_phase (int phase, cudaStream_t stream);
  int launch_iterations (cudaStream_t stream);
  int barrier_fault (cudaStream_t stream);
  int start (bool zero, const void *c, double tol, int max_iter, double norm_b, int iter0, bool new_shadow,
             cudaStream_t s);

  const bmfp_matrix_s *A_ = nullptr;
  int dtype_ = BMFP_R64F;
  bool jacobi_ = false; // any preconditioner (q, z and P allocated)
  int pre_kind_ = 0;     // PreKind of the vector phases
  bool replace_ = true;
  bool from_zero_ = true; // the current run started from x = 0
  int64_t n_ = 0;
  int grid_ = 0;
  int chunk_ = 16;
  int spmv_kind_ = 0;
  double cA_ = 0.0; // entries per row * ||A||_inf (replacement bound)
  const void *c_ = nullptr; // right-hand side of the current run
  void *x_ = nullptr, *r_ = nullptr, *rh_ = nullptr, *p_ = nullptr, *v_ = nullptr;
  void *q_ = nullptr, *s_ = nullptr, *z_ = nullptr, *t_ = nullptr, *P_ = nullptr;
  void *g_ = nullptr, *xp_ = nullptr;
  double *part_ = nullptr;
  size_t part_bytes_ = 0;
  DevState *state_ = nullptr;
  DevState *h_state_ = nullptr; // pinned, two slots
  cudaGraphExec_t graph_ = nullptr;
  const void *iterate_ = nullptr; // persistent iteration kernel, or null: graphs
  cudaStream_t capture_stream_ = nullptr;
  cudaEvent_t ev_[2] = { nullptr, nullptr };
};

// Caller-provided buffers for one solve (used by the entry point that
// allocates nothing): a non-owning view of the matrix arrays plus every
// Krylov vector, the partial sums and the scalar state.
struct RawSolve
{
  bmfp_matrix_s A;     // view of the caller's device arrays (owns nothing)
  int64_t n = 0;       // scalar rows
  int grid = 0;        // CTAs of every phase kernel
  bool jacobi = false;
  bool aligned = true; // values 16-byte aligned: the vectorised SpMV may run
  void *x = nullptr, *r = nullptr, *rh = nullptr, *p = nullptr, *v = nullptr;
  void *q = nullptr, *s = nullptr, *z = nullptr, *t = nullptr, *P = nullptr;
  void *g = nullptr, *xp = nullptr; // group base and accumulated updates of the run
  double *part = nullptr; // kRawParts * grid doubles
  DevState *st = nullptr;
};
constexpr int kRawParts = 9;

// Grid of the phase kernels for n rows (the same rule as WideEngine).
int raw_solve_grid (int64_t n, int *grid);
// The persistent kernel's grid barrier made to time out on purpose (a wait
// for one CTA more than the grid holds) after limit_s: reports the fault flag
// the timed-out CTAs set and how long the launch took.
int barrier_selftest (double limit_s, int *fault, double *elapsed_s, cudaStream_t s);
int raw_jacobi (const RawSolve &b, cudaStream_t stream);
int raw_start (const RawSolve &b, const void *d_rhs, double tol, int max_iter, cudaStream_t stream);
int raw_phase (const RawSolve &b, int phase, cudaStream_t stream);
// x = g + xp: the run's result into the caller's x (after the last phase).
int raw_finish (const RawSolve &b, cudaStream_t stream);

// Factor in [0.5, 1.5) of element i of a shadow residual after a breakdown:
// rh_i = r_i * shadow_factor (i). BiCGStab breaks down when (rh, r) or
// (rh, v) vanishes; a restart from the true residual with rh = r can meet the
// same breakdown again, so it perturbs rh by a fixed hash of the index
// (SplitMix64 finaliser), staying correlated with r ((rh, r) > 0) but no
// longer parallel to it. Deterministic: the same solve gives the same bits.
__host__ __device__ inline double shadow_factor (int64_t i)
{
  uint64_t z = (uint64_t) i * 0x9E3779B97F4A7C15ull + 0x5DEECE66Dull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return 0.5 + (double) (z >> 11) * (1.0 / 9007199254740992.0);
}

// Elementwise helpers used by the refinement loop (vector_ops.cu).
int axpy_scaled_convert (int dst_dtype, int src_dtype, int64_t n, double a, const void *src,
                         void *dst, cudaStream_t stream); // dst += a * src
int scale_convert (int dst_dtype, int src_dtype, int64_t n, double a, const void *src, void *dst,
                   cudaStream_t stream);                  // dst = a * src
} // namespace bmfp
