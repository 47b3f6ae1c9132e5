// Serving loop: continuous batching of solve requests on one GPU.
//
// Callers submit (matrix handle, right-hand side) requests from any thread;
// a dispatcher thread admits them in arrival order while the device memory
// they need fits the HBM budget and the in-flight limit, and launches what it
// admitted right away as a micro-batch: one persistent cluster-per-system
// launch of the batched BiCGStab kernel (batch.cu) on one of several streams.
// Requests that arrive while earlier micro-batches are still running join the
// GPU in their own launches, which overlap on the device with the running
// ones; memory returns to the budget as each micro-batch completes. Matrices
// stay resident (handles owned by the caller; FP32 copies for mixed
// precision are made once per matrix and kept), and each request's Krylov
// state lives on the device from admission to completion. Requests above
// wide_threshold_rows go to whole-GPU lanes (the single-system engine), each
// on its own thread and stream, several at once.
//
// A request's numbers do not depend on what else is in flight: the batched
// kernel solves every system alone within its cluster, in a fixed reduction
// order, and the micro-batch configuration (cluster size, CTA width) is fixed
// per server.
#include "batch.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace bmfp;
using Clock = std::chrono::steady_clock;

namespace
{
struct Request
{
  uint64_t ticket = 0;
  const bmfp_matrix_s *A = nullptr;
  std::vector<double> b;
  double *h_x = nullptr;
  int64_t n = 0;
  size_t bytes = 0;
  Clock::time_point t_submit;
  bmfp_solve_info info{};
  bool done = false;
  bool wide = false;
  // device slices (inside the micro-batch's allocation)
  double *d_b = nullptr, *d_x = nullptr, *w64 = nullptr;
  float *w32 = nullptr;
};

struct MicroBatch
{
  std::vector<Request *> reqs;
  int stream = 0;
  void *d_mem = nullptr;
  size_t bytes = 0;
  char *h_slab = nullptr; // pinned staging from the server's pool
  size_t h_cap = 0;
  BatchDesc *h_desc = nullptr;
  BatchOut *h_out = nullptr;
  std::vector<double *> h_x; // pinned copies of each request's x
  std::vector<char> taken;   // request already handed back
  size_t req_bytes = 0;      // budget bytes of all its requests, released at the end
  cudaEvent_t done = nullptr;
};

size_t align256 (size_t b) { return (b + 255) & ~(size_t) 255; }

// Page-locked staging buffers, recycled. Allocating or freeing page-locked
// memory (like device memory) on the host serialises the streams of the
// device, which would undo the overlap of micro-batches, so buffers are kept
// and handed out again; new ones are only made while the pool grows.
class PinnedPool
{
public:
  // Caller holds the server lock.
  char *take (size_t bytes, size_t *cap)
  {
    auto it = free_.lower_bound (bytes);
    if (it != free_.end ())
      {
        char *p = it->second;
        *cap = it->first;
        free_.erase (it);
        return p;
      }
    size_t c = 64 << 10;
    while (c < bytes)
      c <<= 1;
    void *p = nullptr;
    if (cudaHostAlloc (&p, c, cudaHostAllocMapped) != cudaSuccess)
      return nullptr;
    all_.push_back (p);
    *cap = c;
    return (char *) p;
  }
  // Device address of page-locked memory the kernels write to directly.
  static char *device_alias (char *h)
  {
    void *d = nullptr;
    return cudaHostGetDevicePointer (&d, h, 0) == cudaSuccess ? (char *) d : nullptr;
  }
  void give (char *p, size_t cap)
  {
    if (p)
      free_.emplace (cap, p);
  }
  ~PinnedPool ()
  {
    for (void *p : all_)
      cudaFreeHost (p);
  }

private:
  std::multimap<size_t, char *> free_;
  std::vector<void *> all_;
};
} // namespace

struct bmfp_server_s
{
  bmfp_server_options opts{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> pending;
  std::deque<Request *> wide_queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> requests;
  std::vector<std::unique_ptr<MicroBatch>> running;
  std::map<const bmfp_matrix_s *, void *> vals32; // FP32 copies for mixed / FP32 serving
  std::map<std::pair<int, const bmfp_matrix_s *>, bmfp_solver_t> wide_solvers; // per (lane, matrix)
  std::vector<cudaStream_t> streams;
  std::vector<char> stream_busy;       // a micro-batch runs on the stream
  cudaStream_t convert_stream = nullptr; // FP32 copies of matrices (waited on alone, not behind a batch)
  std::vector<cudaStream_t> wide_streams;
  PinnedPool pinned;                   // staging for micro-batches (lock held)
  cudaMemPool_t pool = nullptr;        // device memory of requests, stream-ordered
  size_t bytes_in_use = 0, peak_bytes = 0;
  int in_flight = 0;
  uint64_t next_ticket = 1, submitted = 0, completed = 0, micro_batches = 0, wide_solves = 0;
  int op = -1;
  int cluster_cap = 1;
  bool stop = false;
  int error = BMFP_SUCCESS;
  std::thread dispatcher;
  std::vector<std::thread> wide_workers;
};

namespace
{
size_t request_bytes (const bmfp_server_s *sv, int64_t n, bool wide)
{
  if (wide)
    return (size_t) n * 8 * 15; // solver vectors (work and Krylov) + b, x
  size_t b = align256 (n * 8) * 2 + align256 (n * 8 * kBatchW64); // b, x, FP64 work vectors
  if (sv->opts.solver.precision != BMFP_SOLVE_FP64)
    b += align256 (n * 4 * 8); // 8 FP32 work vectors
  return b;
}

int ensure_vals32 (bmfp_server_s *sv, const bmfp_matrix_s *A, cudaStream_t s)
{
  if (sv->opts.solver.precision == BMFP_SOLVE_FP64 || sv->vals32.count (A))
    return BMFP_SUCCESS;
  const int64_t nv = A->bs ? A->nnz * A->bs * A->bs : A->nnz;
  void *p = nullptr;
  BMFP_CUDA (cudaMallocFromPoolAsync (&p, sizeof (float) * (size_t) std::max<int64_t> (nv, 1), sv->pool, s));
  int rc = convert_values (BMFP_R64F, BMFP_R32F, nv, A->d_vals, p, s);
  if (rc == BMFP_SUCCESS && cudaStreamSynchronize (s) != cudaSuccess)
    rc = BMFP_ERROR_CUDA; // other streams read the copy next
  if (rc != BMFP_SUCCESS)
    {
      cudaFreeAsync (p, s);
      return rc;
    }
  sv->vals32[A] = p;
  sv->bytes_in_use += sizeof (float) * (size_t) nv;
  return BMFP_SUCCESS;
}

void finish (bmfp_server_s *sv, Request *r)
{
  r->info.seconds = std::chrono::duration<double> (Clock::now () - r->t_submit).count ();
  r->done = true;
  sv->completed++;
}

// Launch one micro-batch (called with the lock held; the device work is
// asynchronous on the chosen stream).
int launch_micro_batch (bmfp_server_s *sv, std::vector<Request *> &reqs, int stream)
{
  std::unique_ptr<MicroBatch> mb (new MicroBatch);
  mb->reqs = reqs;
  mb->stream = stream;
  cudaStream_t s = sv->streams[mb->stream];
  const int n = (int) reqs.size ();
  size_t total = align256 (sizeof (BatchDesc) * n) + 256 + align256 (sizeof (int) * n);
  for (Request *r : reqs)
    {
      total += r->bytes;
      mb->req_bytes += r->bytes;
    }
  mb->taken.assign (n, 0);
  BMFP_CUDA (cudaMallocFromPoolAsync (&mb->d_mem, total, sv->pool, s));
  mb->bytes = total;
  // Pinned, mapped staging: descriptors, results, launch order, then b and x
  // of every request. The kernel writes each system's result and x here as
  // soon as it finishes, so a request leaves without waiting for the slowest
  // system of its launch.
  size_t hbytes = align256 (sizeof (BatchDesc) * n) + align256 (sizeof (BatchOut) * n) + align256 (sizeof (int) * n);
  for (Request *r : reqs)
    hbytes += 2 * align256 (sizeof (double) * r->n);
  mb->h_slab = sv->pinned.take (hbytes, &mb->h_cap);
  if (!mb->h_slab)
    {
      cudaFreeAsync (mb->d_mem, s);
      return fail (BMFP_ERROR_OUT_OF_MEMORY, "page-locked staging of %zu bytes failed", hbytes);
    }
  char *dev_slab = PinnedPool::device_alias (mb->h_slab);
  if (!dev_slab)
    {
      sv->pinned.give (mb->h_slab, mb->h_cap);
      cudaFreeAsync (mb->d_mem, s);
      return fail (BMFP_ERROR_CUDA, "page-locked staging is not mapped into the device");
    }
  auto dev_of = [&] (const void *h) { return dev_slab + ((const char *) h - mb->h_slab); };
  char *hp = mb->h_slab;
  mb->h_desc = (BatchDesc *) hp;
  hp += align256 (sizeof (BatchDesc) * n);
  mb->h_out = (BatchOut *) hp;
  hp += align256 (sizeof (BatchOut) * n);
  int *h_order = (int *) hp;
  hp += align256 (sizeof (int) * n);
  mb->h_x.resize (n);
  char *p = (char *) mb->d_mem;
  BatchDesc *d_desc = (BatchDesc *) p;
  p += align256 (sizeof (BatchDesc) * n);
  std::memset ((void *) mb->h_out, 0, sizeof (BatchOut) * n);
  BatchOut *d_out = (BatchOut *) dev_of (mb->h_out);
  int *d_counter = (int *) p;
  p += 256;
  int *d_order = (int *) p;
  p += align256 (sizeof (int) * n);
  std::vector<int> order (n);
  for (int i = 0; i < n; i++)
    {
      double *h_b = (double *) hp;
      hp += align256 (sizeof (double) * reqs[i]->n);
      mb->h_x[i] = (double *) hp;
      hp += align256 (sizeof (double) * reqs[i]->n);
      std::memcpy (h_b, reqs[i]->b.data (), sizeof (double) * reqs[i]->n);
      Request *r = reqs[i];
      r->d_b = (double *) p;
      p += align256 (r->n * 8);
      r->d_x = (double *) p;
      p += align256 (r->n * 8);
      r->w64 = (double *) p;
      p += align256 (r->n * 8 * kBatchW64);
      if (sv->opts.solver.precision != BMFP_SOLVE_FP64)
        {
          r->w32 = (float *) p;
          p += align256 (r->n * 4 * 8);
        }
      BMFP_CUDA (cudaMemcpyAsync (r->d_b, h_b, sizeof (double) * r->n, cudaMemcpyHostToDevice, s));
      BatchDesc &D = mb->h_desc[i];
      D = BatchDesc{}; // recycled page-locked memory: start from the defaults
      const bmfp_matrix_s *A = r->A;
      D.nbr = A->n_rows;
      D.bs = A->bs ? A->bs : 1;
      D.op = sv->op;
      D.n = r->n;
      D.rp = A->d_row_ptr;
      D.cols = A->d_cols;
      D.vals64 = (const double *) A->d_vals;
      D.vals32 = sv->opts.solver.precision != BMFP_SOLVE_FP64 ? (const float *) sv->vals32[A] : nullptr;
      D.b = r->d_b;
      D.x = r->d_x;
      D.w64 = r->w64;
      D.w32 = r->w32;
      D.x_out = r->h_x ? (double *) dev_of (mb->h_x[i]) : nullptr;
      order[i] = i;
    }
  std::stable_sort (order.begin (), order.end (), [&] (int a, int b) { return reqs[a]->n > reqs[b]->n; });
  std::memcpy (h_order, order.data (), sizeof (int) * n);
  BMFP_CUDA (cudaMemcpyAsync (d_desc, mb->h_desc, sizeof (BatchDesc) * n, cudaMemcpyHostToDevice, s));
  BMFP_CUDA (cudaMemcpyAsync (d_order, h_order, sizeof (int) * n, cudaMemcpyHostToDevice, s));
  BMFP_CUDA (cudaMemsetAsync (d_counter, 0, sizeof (int), s));
  BatchParams P;
  P.n_systems = n;
  P.desc = d_desc;
  P.out = d_out;
  P.counter = d_counter;
  P.order = d_order;
  const bmfp_solver_options &o = sv->opts.solver;
  P.precision = o.precision;
  P.tol = o.tolerance;
  P.max_it = o.max_iterations;
  P.inner_tol = o.inner_tolerance;
  P.inner_max = o.inner_max_iterations;
  P.inner_stall = o.inner_stall_iterations;
  P.max_ref = o.max_refinements;
  P.fallback = o.fallback_fp64;
  const int clusters = std::max (1, std::min (n, sv->cluster_cap));
  int rc = batch_launch (o.precision, sv->op, P, sv->opts.cluster_size, sv->opts.threads_per_cta,
                         clusters * sv->opts.cluster_size, s);
  if (rc != BMFP_SUCCESS)
    return rc;
  BMFP_CUDA (cudaEventCreateWithFlags (&mb->done, cudaEventDisableTiming));
  BMFP_CUDA (cudaEventRecord (mb->done, s));
  for (Request *r : reqs)
    r->info.status = BMFP_PENDING;
  sv->micro_batches++;
  sv->stream_busy[stream] = 1;
  sv->running.push_back (std::move (mb));
  return BMFP_SUCCESS;
}

// Hand back one request of a micro-batch (lock held). After finish() the
// waiter may free the Request at any moment, so the slot is cleared.
void take_request (bmfp_server_s *sv, MicroBatch *mb, size_t i, bool ok)
{
  Request *r = mb->reqs[i];
  const BatchOut &o = mb->h_out[i];
  if (ok && r->h_x)
    std::memcpy (r->h_x, mb->h_x[i], sizeof (double) * r->n);
  bmfp_solve_info &f = r->info;
  f.status = !ok ? BMFP_ERROR_CUDA
                 : (o.status == 1 ? BMFP_SUCCESS : (o.status == 3 ? BMFP_ERROR_BREAKDOWN : BMFP_ERROR_NOT_CONVERGED));
  f.iterations = o.iterations;
  f.iterations_fp32 = o.iterations_fp32;
  f.refinements = o.refinements;
  f.restarts = o.restarts;
  f.replacements = o.replacements;
  f.used_fp64_fallback = o.fallback;
  f.true_rel_residual = o.true_rel;
  f.recursive_rel_residual = o.rec_rel;
  mb->taken[i] = 1;
  mb->reqs[i] = nullptr;
  finish (sv, r);
}

// Hand back the requests whose systems have finished, and retire completed
// micro-batches (lock held). Returns true if any request finished.
bool retire (bmfp_server_s *sv)
{
  bool any = false;
  for (size_t k = 0; k < sv->running.size ();)
    {
      MicroBatch *mb = sv->running[k].get ();
      for (size_t i = 0; i < mb->reqs.size (); i++)
        if (!mb->taken[i] && *reinterpret_cast<volatile int *> (&mb->h_out[i].done))
          {
            take_request (sv, mb, i, true);
            any = true;
          }
      const cudaError_t q = cudaEventQuery (mb->done);
      if (q == cudaErrorNotReady)
        {
          k++;
          continue;
        }
      if (q != cudaSuccess && sv->error == BMFP_SUCCESS)
        sv->error = cuda_fail (q, "micro-batch", __FILE__, __LINE__);
      for (size_t i = 0; i < mb->reqs.size (); i++)
        if (!mb->taken[i])
          {
            take_request (sv, mb, i, q == cudaSuccess && mb->h_out[i].done);
            any = true;
          }
      sv->bytes_in_use -= mb->req_bytes;
      sv->in_flight -= (int) mb->reqs.size ();
      cudaFreeAsync (mb->d_mem, sv->streams[mb->stream]);
      sv->stream_busy[mb->stream] = 0;
      cudaEventDestroy (mb->done);
      sv->pinned.give (mb->h_slab, mb->h_cap);
      sv->running.erase (sv->running.begin () + k);
      any = true;
    }
  return any;
}

// Launch a micro-batch; if that fails, its requests end with the error (so
// their waiters return and the server can still shut down) and the server
// refuses further work.
void launch_or_fail (bmfp_server_s *sv, std::vector<Request *> &reqs, int slot)
{
  const int rc = launch_micro_batch (sv, reqs, slot);
  if (rc == BMFP_SUCCESS)
    return;
  if (sv->error == BMFP_SUCCESS)
    sv->error = rc;
  for (Request *r : reqs)
    {
      r->info.status = rc;
      sv->bytes_in_use -= r->bytes;
      sv->in_flight--;
      finish (sv, r);
    }
  sv->cv_done.notify_all ();
}

void dispatcher_main (bmfp_server_s *sv)
{
  cudaSetDevice (sv->device);
  std::unique_lock<std::mutex> lk (sv->mu);
  for (;;)
    {
      if (retire (sv))
        sv->cv_done.notify_all ();
      // Admit in arrival order while budget and slots allow. A micro-batch
      // starts only on an idle stream; while every stream is busy, arrivals
      // wait and the next launch takes up to max_batch of them at once (one
      // largest-first work queue for its teams). Light load thus gets a launch
      // per request; heavy load gets large batches, which keep the teams
      // busy from one system to the next. Whole-GPU requests do not wait for
      // micro-batch streams.
      std::vector<Request *> admitted;
      auto free_stream = [&] () {
        for (size_t k = 0; k < sv->stream_busy.size (); k++)
          if (!sv->stream_busy[k])
            return (int) k;
        return -1;
      };
      int slot = free_stream ();
      bool blocked = false; // budget or in-flight limit reached: keep arrival order
      for (auto it = sv->pending.begin (); it != sv->pending.end () && !blocked;)
        {
          Request *r = *it;
          if (!r->wide && slot < 0)
            {
              ++it;
              continue;
            }
          if (sv->bytes_in_use + r->bytes > sv->opts.hbm_budget_bytes || sv->in_flight >= sv->opts.max_in_flight)
            {
              blocked = true;
              break;
            }
          if (!r->wide && ensure_vals32 (sv, r->A, sv->convert_stream) != BMFP_SUCCESS)
            {
              blocked = true;
              break;
            }
          it = sv->pending.erase (it);
          sv->bytes_in_use += r->bytes;
          sv->peak_bytes = std::max (sv->peak_bytes, sv->bytes_in_use);
          sv->in_flight++;
          if (r->wide)
            {
              sv->wide_queue.push_back (r);
              sv->cv_work.notify_all ();
              continue;
            }
          admitted.push_back (r);
          if ((int) admitted.size () >= sv->opts.max_batch)
            {
              launch_or_fail (sv, admitted, slot);
              admitted.clear ();
              slot = free_stream ();
            }
        }
      if (!admitted.empty ())
        launch_or_fail (sv, admitted, slot);
      if (sv->stop && sv->pending.empty () && sv->running.empty () && sv->in_flight == 0)
        break;
      // Sleep until new work arrives or a short poll interval passes while
      // micro-batches run (completion is polled through their events).
      if (sv->running.empty () && sv->pending.empty () && !sv->stop)
        sv->cv_work.wait (lk);
      else
        sv->cv_work.wait_for (lk, std::chrono::microseconds (50));
    }
}

void wide_main (bmfp_server_s *sv, int lane)
{
  cudaSetDevice (sv->device);
  cudaStream_t stream = sv->wide_streams[lane];
  // This lane's page-locked staging for b and x, grown when a larger request
  // comes (allocating page-locked memory serialises the device's streams).
  double *h_stage = nullptr;
  int64_t stage_n = 0;
  std::unique_lock<std::mutex> lk (sv->mu);
  for (;;)
    {
      sv->cv_work.wait (lk, [&] { return !sv->wide_queue.empty () || (sv->stop && sv->pending.empty () && sv->in_flight == 0); });
      if (sv->wide_queue.empty ())
        break;
      Request *r = sv->wide_queue.front ();
      sv->wide_queue.pop_front ();
      bmfp_solver_t solver = nullptr;
      const auto key = std::make_pair (lane, r->A);
      auto it = sv->wide_solvers.find (key);
      int rc = BMFP_SUCCESS;
      if (it == sv->wide_solvers.end ())
        {
          bmfp_solver_options o = sv->opts.solver;
          // Lanes share the GPU with the batched solver and each other: a
          // persistent kernel would hold every SM while it runs.
          o.launch_mode = BMFP_LAUNCH_GRAPH;
          rc = bmfp_solver_create (&solver, const_cast<bmfp_matrix_s *> (r->A), &o, stream);
          if (rc == BMFP_SUCCESS)
            sv->wide_solvers[key] = solver;
        }
      else
        solver = it->second;
      lk.unlock ();
      if (rc == BMFP_SUCCESS && stage_n < r->n)
        {
          if (h_stage)
            cudaFreeHost (h_stage);
          h_stage = nullptr;
          stage_n = 0;
          if (cudaMallocHost (&h_stage, sizeof (double) * (size_t) r->n) == cudaSuccess)
            stage_n = r->n;
          else
            rc = BMFP_ERROR_OUT_OF_MEMORY;
        }
      double *d_bx = nullptr; // b then x, from the server's stream-ordered pool
      if (rc == BMFP_SUCCESS
          && cudaMallocFromPoolAsync ((void **) &d_bx, 2 * sizeof (double) * (size_t) r->n, sv->pool, stream)
               != cudaSuccess)
        rc = BMFP_ERROR_OUT_OF_MEMORY;
      if (rc == BMFP_SUCCESS)
        {
          double *d_b = d_bx, *d_x = d_bx + r->n;
          std::memcpy (h_stage, r->b.data (), sizeof (double) * r->n);
          cudaMemcpyAsync (d_b, h_stage, sizeof (double) * r->n, cudaMemcpyHostToDevice, stream);
          rc = bmfp_solver_solve (solver, d_b, d_x, &r->info, stream);
          if (r->h_x)
            {
              cudaMemcpyAsync (h_stage, d_x, sizeof (double) * r->n, cudaMemcpyDeviceToHost, stream);
              cudaStreamSynchronize (stream);
              std::memcpy (r->h_x, h_stage, sizeof (double) * r->n);
            }
        }
      else
        r->info.status = rc;
      if (d_bx)
        cudaFreeAsync (d_bx, stream);
      lk.lock ();
      sv->bytes_in_use -= r->bytes;
      sv->in_flight--;
      sv->wide_solves++;
      finish (sv, r);
      sv->cv_done.notify_all ();
      sv->cv_work.notify_all ();
    }
  lk.unlock ();
  cudaStreamSynchronize (stream);
  if (h_stage)
    cudaFreeHost (h_stage);
}
} // namespace

extern "C" {

void bmfp_server_options_init (bmfp_server_options *o)
{
  if (!o)
    return;
  o->hbm_budget_bytes = (size_t) 120 << 30;
  o->max_in_flight = 4096;
  o->max_batch = 64;
  // Eight concurrent micro-batches: under load each later launch gathers up
  // to max_batch waiting requests. Teams of 4 CTAs x 512 threads: on the
  // served stream (1000 requests at 2000 req/s) 4 x 512, 8 x 512 and 8 x 256
  // measured within 5 % of each other (38.0, 39.3 and 39.8 solves/s), 4 x 512
  // with the lowest median latency (1.07 s against 1.39 and 1.24 s).
  o->streams = 8;
  o->cluster_size = 4;
  o->threads_per_cta = 512;
  // Above 200 000 rows a 4-CTA team takes tens of milliseconds per iteration
  // and can wander to the iteration cap (measured on 500 000-row elasticity
  // requests); the whole-GPU engine finishes them in about 0.35 s.
  o->wide_threshold_rows = 200000;
  // Eight whole-GPU solves side by side, each over one CTA per SM: they then
  // share the SMs instead of taking turns on all of them (61 requests of
  // 500 000 rows: 22.1 s, against 28 s for four lanes of four CTAs per SM).
  o->wide_lanes = 8;
  bmfp_solver_options_init (&o->solver);
  o->solver.ctas_per_sm = 1;
}

int bmfp_server_create (bmfp_server_t *out, const bmfp_server_options *opts)
{
  if (!out)
    return fail (BMFP_ERROR_INVALID_VALUE, "null output");
  *out = nullptr;
  bmfp_server_options o;
  bmfp_server_options_init (&o);
  if (opts)
    o = *opts;
  if (o.max_in_flight < 1 || o.max_batch < 1 || o.streams < 1 || o.streams > 64 || o.hbm_budget_bytes == 0
      || o.wide_lanes < 1 || o.wide_lanes > 16 || o.solver.inner_stall_iterations < 0)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid server options");
  if (o.solver.preconditioner != BMFP_PRECOND_NONE)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "the server takes no preconditioner");
  std::unique_ptr<bmfp_server_s> sv (new (std::nothrow) bmfp_server_s);
  if (!sv)
    return fail (BMFP_ERROR_OUT_OF_MEMORY, "host allocation failed");
  sv->opts = o;
  BMFP_CUDA (cudaGetDevice (&sv->device));
  {
    // Requests' device memory comes from a pool of the server's own, kept
    // (up to the HBM budget) between requests: no cudaMalloc / cudaFree, which
    // would serialise the device's streams, on the serving path.
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = sv->device;
    BMFP_CUDA (cudaMemPoolCreate (&sv->pool, &props));
    uint64_t keep = (uint64_t) o.hbm_budget_bytes;
    BMFP_CUDA (cudaMemPoolSetAttribute (sv->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  }
  BMFP_CUDA (cudaStreamCreateWithFlags (&sv->convert_stream, cudaStreamNonBlocking));
  sv->streams.resize (o.streams);
  sv->stream_busy.assign (o.streams, 0);
  for (auto &s : sv->streams)
    BMFP_CUDA (cudaStreamCreateWithFlags (&s, cudaStreamNonBlocking));
  sv->wide_streams.resize (o.wide_lanes);
  for (auto &s : sv->wide_streams)
    BMFP_CUDA (cudaStreamCreateWithFlags (&s, cudaStreamNonBlocking));
  // Several micro-batches should run side by side: give each at most a
  // quarter of the co-resident clusters.
  int clusters = 0;
  for (int op = 0; op < 3; op++)
    {
      int c = 0;
      const int rc = batch_max_clusters (o.solver.precision, op, o.cluster_size, o.threads_per_cta, &c);
      if (rc != BMFP_SUCCESS)
        return rc;
      clusters = op == 0 ? c : std::min (clusters, c);
    }
  if (clusters < 1)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "cluster %d x %d threads does not fit", o.cluster_size, o.threads_per_cta);
  sv->cluster_cap = std::max (1, clusters / 4);
  bmfp_server_s *raw = sv.get ();
  raw->dispatcher = std::thread (dispatcher_main, raw);
  for (int lane = 0; lane < o.wide_lanes; lane++)
    raw->wide_workers.emplace_back (wide_main, raw, lane);
  *out = sv.release ();
  return BMFP_SUCCESS;
}

int bmfp_server_submit (bmfp_server_t sv, bmfp_matrix_t A, const double *h_b, double *h_x, uint64_t *ticket)
{
  if (!sv || !A || !h_b || !ticket)
    return fail (BMFP_ERROR_INVALID_VALUE, "null argument");
  if (A->dtype != BMFP_R64F || A->n_rows != A->n_cols || (A->bs ? A->bs : 1) > 32)
    return fail (BMFP_ERROR_INVALID_VALUE, "requests need a square FP64 matrix with bs <= 32");
  std::unique_ptr<Request> r (new (std::nothrow) Request);
  if (!r)
    return fail (BMFP_ERROR_OUT_OF_MEMORY, "host allocation failed");
  r->A = A;
  r->n = (int64_t) A->n_rows * (A->bs ? A->bs : 1);
  r->b.assign (h_b, h_b + r->n);
  r->h_x = h_x;
  r->wide = r->n > sv->opts.wide_threshold_rows;
  r->bytes = request_bytes (sv, r->n, r->wide);
  r->t_submit = Clock::now ();
  r->info.status = BMFP_PENDING;
  if (r->bytes > sv->opts.hbm_budget_bytes)
    return fail (BMFP_ERROR_BUDGET, "request needs %zu bytes, above the %zu-byte HBM budget", r->bytes,
                 sv->opts.hbm_budget_bytes);
  std::lock_guard<std::mutex> lk (sv->mu);
  if (sv->error != BMFP_SUCCESS)
    return fail (sv->error, "server stopped after an error");
  const int op = batch_op_for (A);
  if (!r->wide)
    {
      if (sv->op < 0)
        sv->op = op;
      else if (sv->op != op)
        sv->op = 2; // mixed block sizes: the generic row routine serves all
    }
  r->ticket = sv->next_ticket++;
  *ticket = r->ticket;
  sv->pending.push_back (r.get ());
  sv->requests[r->ticket] = std::move (r);
  sv->submitted++;
  sv->cv_work.notify_all ();
  return BMFP_SUCCESS;
}

static int take_result (bmfp_server_t sv, uint64_t ticket, bmfp_solve_info *info, bool block)
{
  std::unique_lock<std::mutex> lk (sv->mu);
  auto it = sv->requests.find (ticket);
  if (it == sv->requests.end ())
    return fail (BMFP_ERROR_INVALID_VALUE, "unknown ticket %llu", (unsigned long long) ticket);
  if (block)
    sv->cv_done.wait (lk, [&] { return it->second->done || sv->error != BMFP_SUCCESS; });
  if (!it->second->done)
    return sv->error != BMFP_SUCCESS ? sv->error : BMFP_PENDING;
  if (info)
    *info = it->second->info;
  const int st = it->second->info.status;
  sv->requests.erase (it);
  return st;
}

int bmfp_server_poll (bmfp_server_t sv, uint64_t ticket, bmfp_solve_info *info)
{
  if (!sv)
    return fail (BMFP_ERROR_INVALID_VALUE, "null server");
  return take_result (sv, ticket, info, false);
}

int bmfp_server_wait (bmfp_server_t sv, uint64_t ticket, bmfp_solve_info *info)
{
  if (!sv)
    return fail (BMFP_ERROR_INVALID_VALUE, "null server");
  return take_result (sv, ticket, info, true);
}

int bmfp_server_get_stats (bmfp_server_t sv, bmfp_server_stats *st)
{
  if (!sv || !st)
    return fail (BMFP_ERROR_INVALID_VALUE, "null argument");
  std::lock_guard<std::mutex> lk (sv->mu);
  st->submitted = sv->submitted;
  st->completed = sv->completed;
  st->micro_batches = sv->micro_batches;
  st->wide_solves = sv->wide_solves;
  st->bytes_in_use = sv->bytes_in_use;
  st->peak_bytes = sv->peak_bytes;
  st->in_flight = sv->in_flight;
  st->pending = (int) sv->pending.size ();
  return BMFP_SUCCESS;
}

int bmfp_server_destroy (bmfp_server_t sv)
{
  if (!sv)
    return BMFP_SUCCESS;
  {
    std::lock_guard<std::mutex> lk (sv->mu);
    sv->stop = true;
    sv->cv_work.notify_all ();
  }
  if (sv->dispatcher.joinable ())
    sv->dispatcher.join ();
  {
    std::lock_guard<std::mutex> lk (sv->mu);
    sv->cv_work.notify_all ();
  }
  for (auto &t : sv->wide_workers)
    if (t.joinable ())
      t.join ();
  for (auto &kv : sv->wide_solvers)
    bmfp_solver_destroy (kv.second);
  for (auto &kv : sv->vals32)
    cudaFreeAsync (kv.second, sv->convert_stream);
  if (sv->convert_stream)
    {
      cudaStreamSynchronize (sv->convert_stream);
      cudaStreamDestroy (sv->convert_stream);
    }
  for (auto s : sv->streams)
    {
      cudaStreamSynchronize (s);
      cudaStreamDestroy (s);
    }
  for (auto s : sv->wide_streams)
    {
      cudaStreamSynchronize (s);
      cudaStreamDestroy (s);
    }
  if (sv->pool)
    cudaMemPoolDestroy (sv->pool);
  delete sv;
  return BMFP_SUCCESS;
}

} // extern "C"
