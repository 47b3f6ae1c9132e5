// Batched BiCGStab engine (batch.cu): many systems in one persistent launch.
#pragma once

#include "solver.h"

#include <vector>

namespace bmfp
{
// FP64 work vectors per system (BatchDesc::w64).
constexpr int kBatchW64 = 10;

// One system as the persistent kernel sees it.
struct BatchDesc
{
  int nbr = 0, bs = 1, op = 0;
  int64_t n = 0;
  const int *rp = nullptr, *cols = nullptr;
  const double *vals64 = nullptr;
  const float *vals32 = nullptr;
  const double *b = nullptr;
  double *x = nullptr;
  double *w64 = nullptr; // kBatchW64 n: r, rh, p, v, s, t, residual, best x, in-run snapshot, x'
  float *w32 = nullptr;  // 8 n: r, rh, p, v, s, t, x32, rhs32
  double *x_out = nullptr; // optional copy of x as each system finishes (mapped host memory)
};

// Result of one system. With `out` in mapped host memory (the serving loop),
// `done` is written last, after a system-scope fence, so the host can take a
// finished system while the rest of its launch still runs.
struct BatchOut
{
  int status = 0; // 1 converged, 2 limit, 3 breakdown
  int iterations = 0, iterations_fp32 = 0, refinements = 0, restarts = 0, fallback = 0;
  double true_rel = 0.0, rec_rel = 0.0;
  int done = 0;
  int replacements = 0;
};

struct BatchParams
{
  int n_systems;
  const BatchDesc *desc;
  BatchOut *out;
  int *counter;
  const int *order;
  int precision;
  double tol;
  int max_it;
  double inner_tol;
  int inner_max;
  int inner_stall;
  int max_ref;
  int fallback;
};

// Row routine of a matrix in the batched kernel, and raw launches of the
// batched kernel over caller-built descriptors (the serving loop's
// micro-batches).
int batch_op_for (const bmfp_matrix_s *A);
int batch_launch (int precision, int op, const BatchParams &P, int cluster, int threads, int grid, cudaStream_t s);
int batch_max_clusters (int precision, int op, int cluster, int threads, int *clusters);

class BatchEngine
{
public:
  BatchEngine () = default;
  ~BatchEngine ();
  BatchEngine (const BatchEngine &) = delete;
  BatchEngine &operator= (const BatchEngine &) = delete;

  int init (int n, const bmfp_matrix_s *const *mats, const bmfp_solver_options &o, cudaStream_t s);
  // Choose cluster size and CTA width (captures a new graph).
  int configure (int cluster, int threads);
  int autotune (const void *const *d_b, void *const *d_x, cudaStream_t s, int probe_iterations);
  int solve (const void *const *d_b, void *const *d_x, bmfp_solve_info *infos, cudaStream_t s);
  int cluster () const { return cluster_; }
  int threads () const { return threads_; }
  int grid () const { return grid_; }

private:
  int set_vectors (const void *const *d_b, void *const *d_x, cudaStream_t s);
  int launch (cudaStream_t s, int max_it_override);

  int n_ = 0;
  bmfp_solver_options opts_{};
  int cluster_ = 8, threads_ = 512, grid_ = 0; // the fastest on uneven elasticity batches
  int op_ = 0;
  void *kernel_ = nullptr;
  BatchDesc *h_desc_ = nullptr, *d_desc_ = nullptr;
  BatchOut *h_out_ = nullptr, *d_out_ = nullptr;
  int *d_counter_ = nullptr, *d_order_ = nullptr;
  void *w64_ = nullptr, *w32_ = nullptr;
  std::vector<void *> vals32_;
  cudaGraphExec_t graph_ = nullptr;
  cudaStream_t capture_stream_ = nullptr;
};
} // namespace bmfp
