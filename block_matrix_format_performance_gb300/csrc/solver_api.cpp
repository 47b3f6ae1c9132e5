// C ABI of the BiCGStab solver: plain FP64 / FP32 solves and the mixed
// FP32-inner / FP64-refinement driver, on top of WideEngine (bicgstab.cu).
#include "batch.h"
#include "solver.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <new>
#include <vector>

using namespace bmfp;

struct bmfp_solver_s
{
  bmfp_solver_options opts{};
  const bmfp_matrix_s *A = nullptr;     // the caller's matrix
  bmfp_matrix_t A_owned = nullptr;      // converted copy (FP32), if any
  std::unique_ptr<WideEngine> main;     // matrix-precision engine (FP64 for MIXED)
  std::unique_ptr<WideEngine> inner;    // FP32 engine (MIXED, or FP32 on an FP64 matrix)
  void *work_a = nullptr;               // residual / converted right-hand side
  void *work_b = nullptr;
  void *work_c = nullptr;               // best iterate kept across restarts
  void *work_d = nullptr;               // best iterate within one run (WideEngine::run snapshot)
  bool fp64_only = false;               // MIXED: the creation probe found FP32 steps unable to progress

  ~bmfp_solver_s ()
  {
    main.reset ();
    inner.reset ();
    if (A_owned)
      bmfp_matrix_destroy (A_owned);
    cudaFree (work_a);
    cudaFree (work_b);
    cudaFree (work_c);
    cudaFree (work_d);
  }
};

namespace
{
int status_of (const DevState &st)
{
  if (st.status == kStateConverged)
    return BMFP_SUCCESS;
  if (st.status == kStateBreakdown)
    return BMFP_ERROR_BREAKDOWN;
  return BMFP_ERROR_NOT_CONVERGED;
}

// Runs the engine with its best-point snapshot: a run that ends above the
// best point it passed (a breakdown, a blow-up stopped by the engine, or the
// iteration limit reached on an erratic stretch of the residual history)
// returns that point. Counts the run's residual replacements into *reps.
int run_keep_best (WideEngine &e, void *d_snap, DevState *st, cudaStream_t s, int *reps)
{
  double snap_rr = INFINITY;
  const int rc = e.run (s, st, d_snap, &snap_rr);
  if (rc == BMFP_SUCCESS && reps)
    *reps += st->replacements;
  return rc;
}

// Restart loop shared by the plain and the mixed solves: verify b - A x,
// restart from the true residual while each restart at least halves it (or,
// after a breakdown, lowers it at all; at most 8 times), and keep the best
// iterate: near the attainable accuracy of the
// working precision a restart can leave x worse (the more so the lower it
// aims: a tenth of its starting residual measured worse than half), and then
// x is restored.
int finish_with_restarts (WideEngine &e, const void *d_b, void *d_r, void *d_xbest, void *d_snap,
                          const bmfp_solver_options &o, DevState &st, int iter_budget, double norm_b,
                          int *restarts_out, double *rel_out, int *reps, cudaStream_t s)
{
  const size_t xbytes = dtype_size (e.dtype ()) * (size_t) e.n ();
  double best = INFINITY;
  int restarts = 0;
  DevState best_st = st;
  for (;;)
    {
      double rr = 0, bb = 0;
      int rc = e.true_residual (d_b, d_r, &rr, &bb, s);
      if (rc != BMFP_SUCCESS)
        return rc;
      const double rel = bb > 0 ? std::sqrt (rr / bb) : 0.0;
      if (!(rel < best))
        {
          if (restarts > 0)
            {
              BMFP_CUDA (cudaMemcpyAsync (e.x (), d_xbest, xbytes, cudaMemcpyDeviceToDevice, s));
              BMFP_CUDA (cudaStreamSynchronize (s));
              st = best_st;
            }
          else
            best = rel;
          break;
        }
      // A restart that met its recursive tolerance but did not at least
      // halve the true residual met the working precision's floor
      // (u ||A| |x|| / ||b||): keep its x, stop. Runs that broke down keep
      // restarting while they improve at all.
      const bool halved = rel <= 0.5 * best || st.status != kStateConverged;
      best = rel;
      best_st = st;
      // A breakdown also restarts (a fresh shadow residual is the usual
      // cure); only the iteration limit ends the loop here.
      if (rel < o.tolerance || st.status == kStateMaxIter || st.iter >= iter_budget || restarts >= 8
          || (restarts > 0 && !halved))
        break;
      BMFP_CUDA (cudaMemcpyAsync (d_xbest, e.x (), xbytes, cudaMemcpyDeviceToDevice, s));
      restarts++;
      // Aim at half the true residual the restart starts from: asked only
      // for the tolerance again, from just above it, a restart moves x by a
      // hair and the true residual with it.
      // After a breakdown the restart takes a perturbed shadow residual
      // (the same one would likely break down again).
      rc = e.start_residual (d_r, std::min (o.tolerance, 0.5 * rel), iter_budget,
                             norm_b > 0 ? norm_b : std::sqrt (bb), s, -1, st.status == kStateBreakdown);
      if (rc == BMFP_SUCCESS)
        rc = run_keep_best (e, d_snap, &st, s, reps);
      if (rc != BMFP_SUCCESS)
        return rc;
    }
  *restarts_out = restarts;
  *rel_out = best;
  return BMFP_SUCCESS;
}

// Solve with one engine from x0 = 0, then (optionally) verify the true
// residual and restart from it (finish_with_restarts).
int solve_plain (WideEngine &e, const void *d_b, void *d_r, void *d_xbest, void *d_snap,
                 const bmfp_solver_options &o, bmfp_solve_info *info, cudaStream_t s)
{
  DevState st{};
  int reps = 0;
  int rc = e.start_zero (d_b, o.tolerance, o.max_iterations, s);
  if (rc == BMFP_SUCCESS)
    rc = run_keep_best (e, d_snap, &st, s, &reps);
  if (rc != BMFP_SUCCESS)
    return rc;
  int status = status_of (st);
  double rel_true = NAN;
  int restarts = 0;
  if (o.check_true_residual)
    {
      rc = finish_with_restarts (e, d_b, d_r, d_xbest, d_snap, o, st, o.max_iterations, -1.0, &restarts, &rel_true,
                                 &reps, s);
      if (rc != BMFP_SUCCESS)
        return rc;
      status = rel_true < o.tolerance ? BMFP_SUCCESS
                                      : (st.status == kStateBreakdown ? BMFP_ERROR_BREAKDOWN : BMFP_ERROR_NOT_CONVERGED);
    }
  info->status = status;
  info->iterations += st.iter;
  info->restarts += restarts;
  info->replacements += reps;
  info->true_rel_residual = rel_true;
  info->recursive_rel_residual = st.norm_b > 0 ? std::sqrt (st.rr) / st.norm_b : 0.0;
  return BMFP_SUCCESS;
}

// Mixed solves whose FP32 steps left the true residual above this (relative
// to ||b||) when they fall back finish in FP64 from x = 0.
constexpr double kFreshFp64Above = 1e-2;

// probe: the creation probe's run (probe_fp32): the FP32 refinement phase
// only, returning with used_fp64_fallback = 1 where a solve would fall back.
int solve_mixed (bmfp_solver_s *sv, const void *d_b, bmfp_solve_info *info, cudaStream_t s, bool probe = false)
{
  const bmfp_solver_options &o = sv->opts;
  WideEngine &e64 = *sv->main;
  WideEngine &e32 = *sv->inner;
  const int64_t n = e64.n ();
  void *r64 = sv->work_a; // FP64 residual
  void *r32 = sv->work_b; // scaled FP32 right-hand side of the inner solve
  BMFP_CUDA (cudaMemsetAsync (e64.x (), 0, sizeof (double) * (size_t) n, s));
  if (sv->fp64_only && o.fallback_fp64)
    {
      // The creation probe found FP32 steps unable to make progress on this
      // matrix (its conditioning is beyond FP32's reach, and it does not
      // change between right-hand sides): go straight to FP64.
      int rc = solve_plain (e64, d_b, r64, sv->work_c, sv->work_d, o, info, s);
      info->used_fp64_fallback = 1;
      info->iterations_fp32 = 0;
      return rc;
    }
  double prev_rel = INFINITY;
  int iters64 = 0, iters32 = 0;
  for (int k = 0;; k++)
    {
      double rr = 0, bb = 0;
      int rc = e64.true_residual (d_b, r64, &rr, &bb, s);
      if (rc != BMFP_SUCCESS)
        return rc;
      const double rel = bb > 0 ? std::sqrt (rr / bb) : 0.0;
      info->true_rel_residual = rel;
      info->recursive_rel_residual = rel;
      if (rel < o.tolerance)
        {
          info->status = BMFP_SUCCESS;
          break;
        }
      const bool budget_left = iters64 + iters32 < o.max_iterations && k < o.max_refinements;
      const bool stalled = k > 0 && rel > prev_rel / 4;
      if (probe && (!budget_left || stalled))
        {
          info->used_fp64_fallback = 1;
          info->status = BMFP_ERROR_NOT_CONVERGED;
          break;
        }
      if (!budget_left || (stalled && o.fallback_fp64))
        {
          if (!o.fallback_fp64 || iters64 + iters32 >= o.max_iterations)
            {
              info->status = BMFP_ERROR_NOT_CONVERGED;
              break;
            }
          info->used_fp64_fallback = 1;
          if (rel > kFreshFp64Above)
            {
              // The FP32 steps gained less than 100x: finish with FP64 from
              // x = 0 (from such an iterate FP64 BiCGStab measured 1.1-1.8x
              // the iterations it needs from zero on the elasticity family).
              bmfp_solver_options o2 = o;
              o2.max_iterations = o.max_iterations - iters32;
              bmfp_solve_info i2{};
              rc = solve_plain (e64, d_b, r64, sv->work_c, sv->work_d, o2, &i2, s);
              if (rc != BMFP_SUCCESS)
                return rc;
              iters64 = i2.iterations;
              info->restarts += i2.restarts;
              info->replacements += i2.replacements;
              info->true_rel_residual = i2.true_rel_residual;
              info->recursive_rel_residual = i2.recursive_rel_residual;
              info->status = i2.status;
              break;
            }
          // Finish in FP64 from the current x (restart from its true residual).
          DevState st{};
          // A fresh count: this engine's device counter still holds the
          // last run of an earlier solve on the same solver.
          int reps = 0;
          rc = e64.start_residual (r64, o.tolerance, o.max_iterations - iters32, std::sqrt (bb), s, 0);
          if (rc == BMFP_SUCCESS)
            rc = run_keep_best (e64, sv->work_d, &st, s, &reps);
          if (rc != BMFP_SUCCESS)
            return rc;
          int restarts = 0;
          double rel_fin = NAN;
          rc = finish_with_restarts (e64, d_b, r64, sv->work_c, sv->work_d, o, st, o.max_iterations - iters32,
                                     std::sqrt (bb), &restarts, &rel_fin, &reps, s);
          if (rc != BMFP_SUCCESS)
            return rc;
          iters64 = st.iter;
          info->true_rel_residual = rel_fin;
          info->recursive_rel_residual = st.norm_b > 0 ? std::sqrt (st.rr) / st.norm_b : 0.0;
          info->status = rel_fin < o.tolerance ? BMFP_SUCCESS
                                               : (st.status == kStateBreakdown ? BMFP_ERROR_BREAKDOWN
                                                                               : BMFP_ERROR_NOT_CONVERGED);
          info->restarts += restarts;
          info->replacements += reps;
          if (info->status == BMFP_ERROR_BREAKDOWN && iters32 + iters64 < o.max_iterations)
            {
              // BiCGStab from the refined iterate can break down again and
              // again (its residual makes a poor shadow vector there, measured
              // on an elasticity system that plain FP64 solves from x = 0).
              // Solve from x = 0 with the budget left and keep the better x.
              const size_t xb = sizeof (double) * (size_t) n;
              BMFP_CUDA (cudaMemcpyAsync (sv->work_b, e64.x (), xb, cudaMemcpyDeviceToDevice, s));
              bmfp_solver_options o2 = o;
              o2.max_iterations = o.max_iterations - iters32 - iters64;
              bmfp_solve_info i2{};
              rc = solve_plain (e64, d_b, r64, sv->work_c, sv->work_d, o2, &i2, s);
              if (rc != BMFP_SUCCESS)
                return rc;
              iters64 += i2.iterations;
              info->restarts += i2.restarts;
              info->replacements += i2.replacements;
              if (i2.true_rel_residual < rel_fin)
                {
                  info->true_rel_residual = i2.true_rel_residual;
                  info->recursive_rel_residual = i2.recursive_rel_residual;
                  info->status = i2.status;
                }
              else
                BMFP_CUDA (cudaMemcpyAsync (e64.x (), sv->work_b, xb, cudaMemcpyDeviceToDevice, s));
            }
          break;
        }
      prev_rel = rel;
      // Inner FP32 solve of A d = r / ||r||, then x += ||r|| d in FP64.
      const double scale = std::sqrt (rr);
      rc = scale_convert (BMFP_R32F, BMFP_R64F, n, 1.0 / scale, r64, r32, s);
      if (rc != BMFP_SUCCESS)
        return rc;
      DevState st{};
      const int cap = std::min (o.inner_max_iterations, o.max_iterations - iters64 - iters32);
      rc = e32.start_zero (r32, o.inner_tolerance, cap, s);
      if (rc == BMFP_SUCCESS)
        rc = e32.run (s, &st, nullptr, nullptr, o.inner_stall_iterations);
      if (rc != BMFP_SUCCESS)
        return rc;
      iters32 += st.iter;
      info->refinements = k + 1;
      if (!(st.norm_b > 0 && std::sqrt (st.rr) < 0.5 * st.norm_b))
        {
          // The FP32 inner solve did not halve its residual (stagnation,
          // breakdown or blow-up): do not apply it; fall back to FP64 next.
          prev_rel = 0.0;
          continue;
        }
      rc = axpy_scaled_convert (BMFP_R64F, BMFP_R32F, n, scale, e32.x (), e64.x (), s);
      if (rc != BMFP_SUCCESS)
        return rc;
    }
  info->iterations = iters64 + iters32;
  info->iterations_fp32 = iters32;
  return BMFP_SUCCESS;
}
// MIXED creation probe: solve_mixed's FP32 refinement phase on a seeded
// right-hand side uniform in [-1, 1). FP32 steps are judged unable to finish
// this matrix when that phase stops where a solve would fall back to FP64
// (an inner solve that does not halve its residual, an outer step that cuts
// the FP64 residual by less than 4x, or the budget spent).
int probe_fp32 (bmfp_solver_s *sv, cudaStream_t s, bool *fp64_only)
{
  const int64_t n = sv->main->n ();
  *fp64_only = false;
  if (n == 0)
    return BMFP_SUCCESS;
  std::vector<double> h ((size_t) n);
  int rc = bmfp_gen_uniform_vector (BMFP_R64F, n, 0x70726f6265ull, 0, h.data ());
  if (rc != BMFP_SUCCESS)
    return rc;
  void *b = sv->work_c; // solve_mixed's refinement phase leaves work_c alone
  BMFP_CUDA (cudaMemcpyAsync (b, h.data (), sizeof (double) * (size_t) n, cudaMemcpyHostToDevice, s));
  bmfp_solve_info pi{};
  rc = solve_mixed (sv, b, &pi, s, true);
  if (rc != BMFP_SUCCESS)
    return rc;
  *fp64_only = pi.used_fp64_fallback != 0 || pi.status != BMFP_SUCCESS;
  return BMFP_SUCCESS;
}
} // namespace

extern "C" {

void bmfp_solver_options_init (bmfp_solver_options *o)
{
  if (!o)
    return;
  o->precision = BMFP_SOLVE_FP64;
  o->preconditioner = BMFP_PRECOND_NONE;
  o->tolerance = 1e-10;
  o->max_iterations = 100000;
  o->check_true_residual = 1;
  o->inner_tolerance = 1e-4;
  o->inner_max_iterations = 1000;
  o->max_refinements = 30;
  o->fallback_fp64 = 1;
  o->iterations_per_graph = 16;
  o->ctas_per_sm = 4;
  o->inner_stall_iterations = 64;
  o->residual_replacement = 1;
  o->launch_mode = BMFP_LAUNCH_AUTO;
}

int bmfp_solver_create (bmfp_solver_t *out, bmfp_matrix_t A, const bmfp_solver_options *opts,
                        void *stream)
{
  if (!out || !A)
    return fail (BMFP_ERROR_INVALID_VALUE, "null argument");
  *out = nullptr;
  bmfp_solver_options o;
  bmfp_solver_options_init (&o);
  if (opts)
    o = *opts;
  if (o.precision < BMFP_SOLVE_FP64 || o.precision > BMFP_SOLVE_MIXED)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid precision %d", o.precision);
  if (o.preconditioner != BMFP_PRECOND_NONE && o.preconditioner != BMFP_PRECOND_JACOBI
      && o.preconditioner != BMFP_PRECOND_BLOCK_JACOBI)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid preconditioner %d", o.preconditioner);
  if (!(o.tolerance > 0) || o.max_iterations < 0 || o.iterations_per_graph < 1 || o.ctas_per_sm < 1
      || o.ctas_per_sm > 8 || o.inner_stall_iterations < 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid tolerance or iteration limits");
  if (o.launch_mode < BMFP_LAUNCH_AUTO || o.launch_mode > BMFP_LAUNCH_PERSISTENT)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid launch mode %d", o.launch_mode);
  if (o.precision == BMFP_SOLVE_MIXED && A->dtype != BMFP_R64F)
    return fail (BMFP_ERROR_INVALID_VALUE, "mixed precision needs an FP64 matrix");
  if (o.precision == BMFP_SOLVE_FP64 && A->dtype != BMFP_R64F)
    return fail (BMFP_ERROR_INVALID_VALUE, "FP64 solves need an FP64 matrix");
  const int n_rows = A->n_rows * (A->bs ? A->bs : 1);
  const int n_cols = A->n_cols * (A->bs ? A->bs : 1);
  if (n_rows != n_cols)
    return fail (BMFP_ERROR_INVALID_VALUE, "BiCGStab needs a square matrix (%d x %d)", n_rows, n_cols);
  cudaStream_t s = as_stream (stream);
  std::unique_ptr<bmfp_solver_s> sv (new (std::nothrow) bmfp_solver_s);
  if (!sv)
    return fail (BMFP_ERROR_OUT_OF_MEMORY, "host allocation failed");
  sv->opts = o;
  sv->A = A;
  const int jac = o.preconditioner;
  int rc = BMFP_SUCCESS;
  const bmfp_matrix_s *A32 = A;
  if (o.precision != BMFP_SOLVE_FP64 && A->dtype == BMFP_R64F)
    {
      rc = bmfp_matrix_convert (&sv->A_owned, A, BMFP_R32F, stream);
      if (rc != BMFP_SUCCESS)
        return rc;
      A32 = sv->A_owned;
    }
  if (o.precision == BMFP_SOLVE_FP32)
    {
      sv->main.reset (new (std::nothrow) WideEngine);
      rc = sv->main->init (A32, jac, o.iterations_per_graph, s, o.ctas_per_sm, o.launch_mode);
    }
  else
    {
      sv->main.reset (new (std::nothrow) WideEngine);
      rc = sv->main->init (A, jac, o.iterations_per_graph, s, o.ctas_per_sm, o.launch_mode);
      if (rc == BMFP_SUCCESS && o.precision == BMFP_SOLVE_MIXED)
        {
          sv->inner.reset (new (std::nothrow) WideEngine);
          rc = sv->inner->init (A32, jac, o.iterations_per_graph, s, o.ctas_per_sm, o.launch_mode);
        }
    }
  if (rc != BMFP_SUCCESS)
    return rc;
  sv->main->set_replacement (o.residual_replacement != 0 && o.check_true_residual != 0);
  const size_t nb = (size_t) std::max (n_rows, 1);
  BMFP_CUDA (cudaMalloc (&sv->work_a, nb * 8));
  BMFP_CUDA (cudaMalloc (&sv->work_b, nb * 8));
  BMFP_CUDA (cudaMalloc (&sv->work_c, nb * 8));
  BMFP_CUDA (cudaMalloc (&sv->work_d, nb * 8));
  if (o.precision == BMFP_SOLVE_MIXED && o.fallback_fp64)
    {
      rc = probe_fp32 (sv.get (), s, &sv->fp64_only);
      if (rc == BMFP_SUCCESS && cudaStreamSynchronize (s) != cudaSuccess)
        rc = fail (BMFP_ERROR_CUDA, "mixed-precision probe failed");
      if (rc != BMFP_SUCCESS)
        return rc;
    }
  *out = sv.release ();
  return BMFP_SUCCESS;
}

int bmfp_solver_solve (bmfp_solver_t sv, const void *d_b, void *d_x, bmfp_solve_info *info_out,
                       void *stream)
{
  if (!sv || !d_b || !d_x)
    return fail (BMFP_ERROR_INVALID_VALUE, "null argument");
  cudaStream_t s = as_stream (stream);
  bmfp_solve_info info{};
  const auto t0 = std::chrono::steady_clock::now ();
  int rc = BMFP_SUCCESS;
  const int64_t n = sv->main->n ();
  const int user_dtype = sv->A->dtype;
  if (sv->opts.precision == BMFP_SOLVE_MIXED)
    {
      rc = solve_mixed (sv, d_b, &info, s);
      if (rc == BMFP_SUCCESS)
        rc = convert_values (BMFP_R64F, user_dtype, n, sv->main->x (), d_x, s);
    }
  else
    {
      WideEngine &e = *sv->main;
      const void *b = d_b;
      if (e.dtype () != user_dtype)
        {
          rc = convert_values (user_dtype, e.dtype (), n, d_b, sv->work_b, s);
          b = sv->work_b;
        }
      if (rc == BMFP_SUCCESS)
        rc = solve_plain (e, b, sv->work_a, sv->work_c, sv->work_d, sv->opts, &info, s);
      if (e.dtype () == BMFP_R32F)
        info.iterations_fp32 = info.iterations;
      if (rc == BMFP_SUCCESS)
        rc = convert_values (e.dtype (), user_dtype, n, e.x (), d_x, s);
    }
  if (rc == BMFP_SUCCESS)
    {
      cudaError_t e = cudaStreamSynchronize (s);
      if (e != cudaSuccess)
        rc = cuda_fail (e, "solve", __FILE__, __LINE__);
    }
  info.seconds = std::chrono::duration<double> (std::chrono::steady_clock::now () - t0).count ();
  if (info_out)
    *info_out = info;
  if (rc != BMFP_SUCCESS)
    return rc;
  if (info.status != BMFP_SUCCESS)
    fail (info.status, "BiCGStab stopped with status %d after %d iterations (true residual %.3e)",
          info.status, info.iterations, info.true_rel_residual);
  return info.status;
}

int bmfp_solver_destroy (bmfp_solver_t sv)
{
  delete sv;
  return BMFP_SUCCESS;
}

int bmfp_selftest_barrier_timeout (double limit_seconds, int *fault, double *elapsed_seconds, void *stream)
{
  return bmfp::barrier_selftest (limit_seconds, fault, elapsed_seconds, as_stream (stream));
}

} // extern "C"

struct bmfp_batch_s
{
  bmfp::BatchEngine engine;
  int n = 0;
};

extern "C" {

int bmfp_batch_create (bmfp_batch_t *out, int n, const bmfp_matrix_t *mats, const bmfp_solver_options *opts,
                       void *stream)
{
  if (!out || n < 0 || (n > 0 && !mats))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  *out = nullptr;
  bmfp_solver_options o;
  bmfp_solver_options_init (&o);
  if (opts)
    o = *opts;
  if (o.precision < BMFP_SOLVE_FP64 || o.precision > BMFP_SOLVE_MIXED || !(o.tolerance > 0)
      || o.inner_stall_iterations < 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid precision, tolerance or stall limit");
  if (o.preconditioner != BMFP_PRECOND_NONE)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "batched solves take no preconditioner");
  std::unique_ptr<bmfp_batch_s> b (new (std::nothrow) bmfp_batch_s);
  if (!b)
    return fail (BMFP_ERROR_OUT_OF_MEMORY, "host allocation failed");
  b->n = n;
  const int rc = b->engine.init (n, reinterpret_cast<const bmfp_matrix_s *const *> (mats), o, as_stream (stream));
  if (rc != BMFP_SUCCESS)
    return rc;
  *out = b.release ();
  return BMFP_SUCCESS;
}

int bmfp_batch_configure (bmfp_batch_t b, int cluster_size, int threads_per_cta)
{
  if (!b)
    return fail (BMFP_ERROR_INVALID_VALUE, "null batch");
  return b->engine.configure (cluster_size, threads_per_cta);
}

int bmfp_batch_autotune (bmfp_batch_t b, const void *const *d_b, void *const *d_x, int probe_iterations,
                         int *cluster_size, int *threads_per_cta, void *stream)
{
  if (!b || (b->n > 0 && (!d_b || !d_x)) || probe_iterations < 1)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  const int rc = b->engine.autotune (d_b, d_x, as_stream (stream), probe_iterations);
  if (cluster_size)
    *cluster_size = b->engine.cluster ();
  if (threads_per_cta)
    *threads_per_cta = b->engine.threads ();
  return rc;
}

int bmfp_batch_solve (bmfp_batch_t b, const void *const *d_b, void *const *d_x, bmfp_solve_info *infos,
                      void *stream)
{
  if (!b || (b->n > 0 && (!d_b || !d_x || !infos)))
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid arguments");
  if (b->n == 0)
    return BMFP_SUCCESS;
  const int rc = b->engine.solve (d_b, d_x, infos, as_stream (stream));
  if (rc != BMFP_SUCCESS && rc != BMFP_ERROR_NOT_CONVERGED && rc != BMFP_ERROR_BREAKDOWN)
    return rc;
  if (rc != BMFP_SUCCESS)
    fail (rc, "at least one batched system did not converge");
  return rc;
}

int bmfp_batch_destroy (bmfp_batch_t b)
{
  delete b;
  return BMFP_SUCCESS;
}

} // extern "C"
