// BiCGStab on the GPU: the recurrences of the reference solver
// (gpu/bicgstab.cu:387-513, optional point-Jacobi right preconditioning as in
// :201-238), restructured for GB300.
//
// One iteration is five phases over all rows on a fixed grid; the scalars
// rho, alpha, omega, beta live in device memory (DevState), so no host round
// trip separates the phases (the reference did four blocking copies and a
// print per iteration, gpu/bicgstab.cu:447-510):
//
//   phase 1  p = r + beta (p - omega v);   q = P p
//   phase 2  v = A q, partial (rh, v)       fused into the SpMV epilogue
//            -> alpha = rho / (rh, v)
//   phase 3  s = r - alpha v;  z = P s
//   phase 4  t = A z, partials (t, s), (t, t)
//            -> omega = (t, s) / (t, t)
//   phase 5  x' += alpha q + omega z;  r = s - omega t
//            partials (rh, r), (r, r), (x', x')
//            -> convergence, limit and breakdown tests, the replacement
//               decision, beta = (rho / rho_prev)(alpha / omega)
//
// Algorithmic traffic per iteration: 2 SpMV + 17 n vector elements (no
// preconditioner). Each CTA reduces its threads' terms to one partial per dot
// product; the CTA that finishes a phase last (an acq_rel arrival counter)
// sums the grid's partials in index order and derives the scalars (the
// arrows above), so a solve is deterministic for a given grid.
//
// The phases run in one of two ways, with the same bits on the same grid:
// a CUDA graph of five kernels per iteration (`chunk` iterations per graph),
// or one persistent cooperative kernel per `chunk` iterations whose phases
// are separated by grid barriers, the last CTA to reach a barrier doing the
// phase's scalar work (the auto choice from kPersistentRows rows). The host
// only polls the done flag between launches; phases after convergence return
// at once.
//
// Residual replacement with group update (van der Vorst and Ye 2000, see
// DevState): the decision at the end of phase 5 tracks the deviation bound
// and, when it is time, the next iteration's phase 1 does the fold
// g += x', x' = 0 instead of the p update; phase 2 then computes r = c - A g
// instead of v = A q (and (rh, r), (r, r)), phases 3 and 4 return at once and
// phase 5 only takes the decision on those sums. No kernel is added to the
// graph for it.
//
// Differences from the reference, on purpose: the solution returned is the
// last iterate (the reference copied buffer half 0, bicgstab.cu:515), the
// recursive residual is replaced by the true one near convergence (above),
// and a solve finishes with a true-residual check b - A x (restarting from
// the true residual when the recursive one has drifted below the tolerance
// first).
#include "solver.h"
#include "spmv_core.cuh"

#include <cuda/atomic>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace bmfp
{
namespace
{
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

enum PartKind
{
  kRhR = 0,
  kRR = 1,
  kRhV = 2,
  kTS = 3,
  kTT = 4,
  kResRR = 5,
  kResBB = 6,
  kXX = 7, // (x', x') of phase 5
  kGG = 8, // (g, g) after a fold (phase 1) or 0 at a run's start
  kParts = 9
};
// The allocation-free entry point sizes its partial-sum slot by kRawParts.
static_assert (kParts == kRawParts, "solver.h kRawParts must equal the number of partial kinds");

template <typename T> struct Args
{
  int nbr, bs;
  const int *rp, *cols;
  const T *vals;
  int64_t n;
  T *x, *r, *rh, *p, *v, *q, *s, *z, *t;
  const T *P;
  T *g, *xp; // group base and updates accumulated since the last replacement
  double *part;
  int grid;
  DevState *st;
};

__device__ __forceinline__ double warp_sum (double v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    v += __shfl_xor_sync (0xffffffffu, v, off);
  return v;
}

// done and rep_now in one load. Both are written by earlier kernels (done
// also by block 0 of phases 1, 3 and 5, in cases where every block of that
// phase takes the same early return anyway), so a plain load suffices.
__device__ __forceinline__ int2 flags (const DevState *st)
{
  return *reinterpret_cast<const int2 *> (&st->done);
}

__device__ __forceinline__ bool is_done (const DevState *st) { return flags (st).x != 0; }

// Sum the grid partials of NK kinds in a fixed order, broadcast to the CTA.
// Every thread loads its share of the partials at once (the grid is a few
// CTAs per SM, so a handful of loads each), then warps and the warps' totals
// reduce by butterflies: a few memory round trips instead of one per 32
// partials, on the path every phase waits for.
template <int NK>
__device__ __forceinline__ void sum_parts (const double *part, int grid, const int (&ks)[NK],
                                           double (&out)[NK])
{
  __shared__ double sh_w[NK][kWarps];
  __shared__ double sh[NK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double acc[NK];
#pragma unroll
  for (int k = 0; k < NK; k++)
    acc[k] = 0.0;
  // __ldcg: the partials were written by other CTAs of this kernel (L2 is
  // coherent, this SM's L1 need not be)
  for (int i = threadIdx.x; i < grid; i += kThreads)
#pragma unroll
    for (int k = 0; k < NK; k++)
      acc[k] += __ldcg (part + ks[k] * grid + i);
#pragma unroll
  for (int k = 0; k < NK; k++)
    {
      const double s = warp_sum (acc[k]);
      if (lane == 0)
        sh_w[k][w] = s;
    }
  __syncthreads ();
  if (w == 0)
#pragma unroll
    for (int k = 0; k < NK; k++)
      {
        const double a = warp_sum (lane < kWarps ? sh_w[k][lane] : 0.0);
        if (lane == 0)
          sh[k] = a;
      }
  __syncthreads ();
#pragma unroll
  for (int k = 0; k < NK; k++)
    out[k] = sh[k];
}

// True in exactly one CTA of the kernel: the last to finish writing its
// partials (each CTA's thread 0 wrote them, fences, then counts itself in
// st->arrive). That CTA resets the counter for the next kernel. No thread
// waits on another: the last CTA just finds everyone else already done.
__device__ __forceinline__ bool arrive_last (DevState *st, int grid)
{
  __shared__ int sh_last;
  __syncthreads ();
  if (threadIdx.x == 0)
    {
      // acq_rel at device scope: releases this thread's partial writes to
      // the CTA that comes last, and acquires everyone's for that CTA.
      cuda::atomic_ref<unsigned, cuda::thread_scope_device> arrive (st->arrive);
      const unsigned t = arrive.fetch_add (1u, cuda::memory_order_acq_rel);
      sh_last = t == (unsigned) grid - 1;
      if (sh_last)
        arrive.store (0u, cuda::memory_order_relaxed);
    }
  __syncthreads ();
  return sh_last != 0;
}

// Reduce per-thread values over the CTA (fixed order) into part[k][blockIdx]:
// a tree through shared memory (128, 64, 32 threads add pairs) and one warp
// butterfly for the last 32. Each warp-wide FP64 add costs GB300's narrow
// FP64 pipe the same whatever the number of useful lanes: the tree takes
// 12 warp adds per value and CTA, a butterfly in every warp took 45.
template <int NK>
__device__ __forceinline__ void store_parts (double (&v)[NK], double *part, int grid,
                                             const int (&ks)[NK])
{
  __shared__ double sh[NK][kThreads];
  const int t = threadIdx.x;
#pragma unroll
  for (int k = 0; k < NK; k++)
    sh[k][t] = v[k];
  __syncthreads ();
#pragma unroll
  for (int h = kThreads / 2; h >= 32; h >>= 1)
    {
      if (t < h)
#pragma unroll
        for (int k = 0; k < NK; k++)
          sh[k][t] += sh[k][t + h];
      __syncthreads ();
    }
  if (t < 32)
#pragma unroll
    for (int k = 0; k < NK; k++)
      {
        const double a = warp_sum (sh[k][t]);
        if (t == 0)
          part[ks[k] * grid + blockIdx.x] = a;
      }
}

#define GRID_STRIDE(i, n)                                                                          \
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < (n);                       \
       i += (int64_t) gridDim.x * blockDim.x)

// ------------------------------------------------------------ SpMV phases

template <typename T, int BS, int G, class XL = dev::XNc> struct FlatOp
{
  template <class Epi>
  __device__ static void run (const Args<T> &a, const T *x, T *y, Epi &e)
  {
    const int64_t group = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ng = (int64_t) gridDim.x * blockDim.x / G;
    for (int64_t row = group; row < a.nbr; row += ng)
      core::flat_row<T, BS, G, 4, XL> ((int) row, a.rp, a.cols, a.vals, x, y, e);
  }
};

template <typename T, int BSC, class XL = dev::XNc> struct TprOp
{
  template <class Epi>
  __device__ static void run (const Args<T> &a, const T *x, T *y, Epi &e)
  {
    const int64_t warp = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (int64_t) gridDim.x * blockDim.x >> 5;
    for (int64_t row = warp; row < a.nbr; row += nw)
      core::tpr_row<T, BSC, XL> ((int) row, a.bs, a.rp, a.cols, a.vals, x, y, e);
  }
};

template <typename T, int G, class XL = dev::XNc> struct CsrOp
{
  template <class Epi>
  __device__ static void run (const Args<T> &a, const T *x, T *y, Epi &e)
  {
    const int64_t group = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ng = (int64_t) gridDim.x * blockDim.x / G;
    for (int64_t row = group; row < a.nbr; row += ng)
      core::csr_row<T, G, XL> ((int) row, a.rp, a.cols, a.vals, x, y, e);
  }
};

// Dot-product accumulators of the SpMV epilogues and phase 5 run in T: each
// thread sums a handful of terms, then warps, CTAs and the grid combine the
// partials in FP64. For FP64 solves that is FP64 throughout; the FP32 engine
// (inner solves of mixed precision, asked for 1e-4) keeps GB300's narrow
// FP64 pipe out of its per-element work.
template <typename T> struct EpiDot
{
  const T *a;
  T acc = 0;
  __device__ void operator() (int64_t i, T y) { acc = fma (a[i], y, acc); }
};

template <typename T> struct EpiTS
{
  const T *s;
  T ts = 0, tt = 0;
  __device__ void operator() (int64_t i, T t)
  {
    ts = fma (s[i], t, ts);
    tt = fma (t, t, tt);
  }
};

template <typename T> struct EpiResidual
{
  const T *b;
  T *r;
  double rr = 0.0, bb = 0.0;
  __device__ void operator() (int64_t i, T y)
  {
    const T bi = b[i];
    const T ri = bi - y;
    r[i] = ri;
    rr = fma ((double) ri, (double) ri, rr);
    bb = fma ((double) bi, (double) bi, bb);
  }
};

// Residual replacement: r = c - A g, with (rh, r) and (r, r).
template <typename T> struct EpiReplace
{
  const T *c;
  T *r;
  const T *rh;
  T rhr = 0, rr = 0;
  __device__ void operator() (int64_t i, T y)
  {
    const T ri = c[i] - y;
    r[i] = ri;
    rhr = fma (rh[i], ri, rhr);
    rr = fma (ri, ri, rr);
  }
};

// The scalars that open an iteration, from the sums of (rh, r), (r, r) and
// nn: the convergence, limit and breakdown tests, the replacement decision
// (nn = (g, g) after a replacement or at a run's start, which resets the
// deviation bound; else (x', x')) and beta. One thread of the last CTA of
// the kernel that completed the sums runs it. GB300's FP64 pipe is narrow
// (about 1/58 of FP32): the divides and square roots run once per kernel,
// not in every CTA.
__device__ void decide (DevState *st, double rho, double rr, double nn, bool after_rep)
{
  if (st->norm_b < 0.0)
    st->norm_b = sqrt (rr); // ||r0|| of a fresh solve
  const double nb = st->norm_b;
  const double omega = st->omega;
  int status = kStateRunning;
  double beta = 0.0;
  const double nr = sqrt (rr);
  if (nb == 0.0 || nr < st->tol * nb) // gpu/bicgstab.cu:512
    status = kStateConverged;
  else if (st->iter >= st->max_iter)
    status = kStateMaxIter;
  else if (rho == 0.0 || omega == 0.0 || !isfinite (rho))
    status = kStateBreakdown;
  else
    {
      beta = rho / st->rho_prev * st->alpha / omega; // gpu/bicgstab.cu:451
      if (!isfinite (beta))
        status = kStateBreakdown;
    }
  int rep = 0;
  const double eps = st->eps;
  if (status == kStateRunning && eps > 0.0)
    {
      if (after_rep)
        st->dev = st->dev0 = eps * (st->cA * sqrt (nn) + nr);
      else
        {
          const double dev = st->dev + eps * (st->cA * sqrt (nn) + nr);
          rep = st->dev <= kReplaceThreshold * st->nr_prev && dev > kReplaceThreshold * nr && dev > 1.1 * st->dev0;
          st->dev = dev;
        }
      st->nr_prev = nr;
    }
  st->rr = rr;
  if (status != kStateRunning)
    {
      st->status = status;
      *reinterpret_cast<volatile int *> (&st->done) = 1;
    }
  else if (rep)
    {
      st->rep_now = 1;
      st->replacements = st->replacements + 1;
    }
  else
    {
      st->rep_now = 0;
      st->rho = rho;
      st->beta = beta;
    }
}

// Each phase is a body, run by every CTA, and (for phases that end in a dot
// product) a tail that turns the grid's partial sums into the next scalars.
// The phase kernels of the iteration graph run the tail in the last CTA to
// finish (arrive_last) on the device state in global memory; the persistent
// iteration kernel runs it in every CTA, on a copy of the state in shared
// memory, after a grid barrier. Both sum the partials in the same order, so
// both give the same bits.

// phase 2: v = A q, partial (rh, v). In a replacement iteration r = c - A g
// with partials (rh, r), (r, r) instead (A g lands in t, free until phase 4).
template <typename T, class Op> __device__ __forceinline__ void body_v (const Args<T> &a, const DevState *sc, bool rep)
{
  if (rep)
    {
      EpiReplace<T> e{ static_cast<const T *> (sc->c), a.r, a.rh };
      Op::run (a, a.g, a.t, e);
      double vals[2] = { (double) e.rhr, (double) e.rr };
      const int ks[2] = { kRhR, kRR };
      store_parts<2> (vals, a.part, a.grid, ks);
      return;
    }
  EpiDot<T> e{ a.rh };
  Op::run (a, a.q, a.v, e);
  double vals[1] = { (double) e.acc };
  const int ks[1] = { kRhV };
  store_parts<1> (vals, a.part, a.grid, ks);
}

// alpha from (rh, v), or a breakdown.
__device__ __forceinline__ void tail_v (DevState *st, const double *part, int grid)
{
  double sv[1];
  const int ks[1] = { kRhV };
  sum_parts<1> (part, grid, ks, sv);
  if (threadIdx.x == 0)
    {
      const double alpha = st->rho / sv[0]; // gpu/bicgstab.cu:466
      if (sv[0] != 0.0 && isfinite (alpha))
        st->alpha = alpha;
      else
        {
          st->status = kStateBreakdown;
          *reinterpret_cast<volatile int *> (&st->done) = 1;
        }
    }
}

// phase 4: t = A z, partials (t, s), (t, t).
template <typename T, class Op> __device__ __forceinline__ void body_t (const Args<T> &a)
{
  EpiTS<T> e{ a.s };
  Op::run (a, a.z, a.t, e);
  double vals[2] = { (double) e.ts, (double) e.tt };
  const int ks[2] = { kTS, kTT };
  store_parts<2> (vals, a.part, a.grid, ks);
}

// omega from (t, s) and (t, t), or a breakdown.
__device__ __forceinline__ void tail_t (DevState *st, const double *part, int grid)
{
  double sv[2];
  const int ks[2] = { kTS, kTT };
  sum_parts<2> (part, grid, ks, sv);
  if (threadIdx.x == 0)
    {
      const double omega = sv[1] != 0.0 ? sv[0] / sv[1] : 0.0; // :488
      if (isfinite (omega))
        st->omega = omega;
      else
        {
          // Leave x' untouched so the run keeps the last finite iterate.
          st->status = kStateBreakdown;
          *reinterpret_cast<volatile int *> (&st->done) = 1;
        }
    }
}

// End of an iteration: the decision that opens the next one, from (rh, r),
// (r, r) and (x', x') of phase 5, or in a replacement iteration from r,
// (rh, r) and (r, r) of phase 2 and (g, g) of phase 1.
__device__ __forceinline__ void tail_end (DevState *st, const double *part, int grid, bool rep)
{
  double sv[3];
  const int ks[3] = { kRhR, kRR, rep ? kGG : kXX };
  sum_parts<3> (part, grid, ks, sv);
  if (threadIdx.x == 0)
    {
      if (!rep)
        {
          st->rho_prev = st->rho;
          st->iter = st->iter + 1;
        }
      decide (st, sv[0], sv[1], sv[2], rep);
    }
}

template <typename T, class Op>
__global__ void __launch_bounds__ (kThreads) phase_v (Args<T> a)
{
  DevState *st = a.st;
  const int2 f = flags (st);
  if (f.x)
    return;
  body_v<T, Op> (a, st, f.y != 0);
  if (f.y || !arrive_last (st, a.grid))
    return;
  tail_v (st, a.part, a.grid);
}

template <typename T, class Op>
__global__ void __launch_bounds__ (kThreads) phase_t (Args<T> a)
{
  DevState *st = a.st;
  const int2 f = flags (st);
  if (f.x || f.y)
    return;
  body_t<T, Op> (a);
  if (!arrive_last (st, a.grid))
    return;
  tail_t (st, a.part, a.grid);
}

// r = b - A x (x given), partials ||r||^2, ||b||^2 — the true residual.
template <typename T, class Op>
__global__ void __launch_bounds__ (kThreads)
  residual_kernel (Args<T> a, const T *x, const T *b, T *r, T *y)
{
  EpiResidual<T> e{ b, r };
  Op::run (a, x, y, e);
  double vals[2] = { e.rr, e.bb };
  const int ks[2] = { kResRR, kResBB };
  store_parts<2> (vals, a.part, a.grid, ks);
}

// ------------------------------------------------------------ vector phases

// Start of a run solving A e = c from e = 0 (ZERO: a fresh solve; else a
// restart whose c is the true residual of the current x). x itself is not
// touched until the run ends. Its last CTA takes the first decision.
template <typename T, bool ZERO>
__global__ void __launch_bounds__ (kThreads)
  start_kernel (Args<T> a, const T *src, double tol, int max_iter, double norm_b, int iter0, double eps,
                double cA, int new_shadow)
{
  DevState *st = a.st;
  if (blockIdx.x == 0 && threadIdx.x == 0)
    {
      st->rho_prev = 1.0; // gpu/bicgstab.cu:414-420
      st->alpha = 1.0;
      st->omega = 1.0;
      st->rho = 0.0;
      st->beta = 0.0;
      st->tol = tol;
      st->max_iter = max_iter;
      st->done = 0;
      st->status = kStateRunning;
      st->eps = eps;
      st->cA = cA;
      st->c = src;
      st->rep_now = 0;
      st->replacements = 0;
      st->dev = st->dev0 = st->nr_prev = 0.0;
      if (ZERO)
        {
          st->iter = 0;
          st->norm_b = -1.0; // set by the first decision
        }
      else
        {
          if (norm_b > 0.0)
            st->norm_b = norm_b;
          if (iter0 >= 0)
            st->iter = iter0;
        }
    }
  double rr = 0.0, rhr = 0.0;
  GRID_STRIDE (i, a.n)
  {
    const T ri = src[i];
    const T hi = new_shadow ? (T) (ri * shadow_factor (i)) : ri;
    a.r[i] = ri;
    a.rh[i] = hi;
    a.p[i] = 0;
    a.v[i] = 0;
    a.g[i] = 0;
    a.xp[i] = 0;
    rr = fma ((double) ri, (double) ri, rr);
    rhr = fma ((double) hi, (double) ri, rhr);
  }
  double vals[3] = { rhr, rr, 0.0 };
  const int ks[3] = { kRhR, kRR, kGG };
  store_parts<3> (vals, a.part, a.grid, ks);
  if (!arrive_last (st, a.grid))
    return;
  double sv[3];
  sum_parts<3> (a.part, a.grid, ks, sv);
  if (threadIdx.x == 0)
    decide (st, sv[0], sv[1], sv[2], true);
}

// Preconditioner of the vector phases (right preconditioning, q = M^-1 p,
// z = M^-1 s): none, point Jacobi (gpu/bicgstab.cu:201-238), or block
// Jacobi (M^-1 = the inverses of the bs x bs diagonal blocks), the latter
// for bs = 2 with the block in registers and for any bs <= 8 (a block and
// its inverse fit a thread's registers and a small local frame; the FEM
// operators this serves have bs 2 or 3).
enum PreKind
{
  kPreNone = 0,
  kPrePoint = 1,
  kPreBlock2 = 2,
  kPreBlockAny = 3
};

constexpr int kMaxBlockJacobi = 8;

// One block row of a phase with block Jacobi: out = new values of the block
// (computed by f(k) for k < bs, stored to dst), then prec = Minv * out.
template <typename T, int PK, class F>
__device__ __forceinline__ void block_row_apply (const Args<T> &a, int64_t br, T *dst, T *prec, F f)
{
  const int bs = PK == kPreBlock2 ? 2 : a.bs;
  const int64_t base = br * bs;
  const T *M = a.P + (size_t) br * bs * bs;
  T u[PK == kPreBlock2 ? 2 : kMaxBlockJacobi];
  for (int k = 0; k < bs; k++)
    {
      u[k] = f (base + k);
      dst[base + k] = u[k];
    }
  for (int r = 0; r < bs; r++)
    {
      T acc = 0;
      for (int c = 0; c < bs; c++)
        acc = fma (M[r * bs + c], u[c], acc);
      prec[base + r] = acc;
    }
}

// phase 1: p = r + beta (p - omega v) (q = M^-1 p), with beta from the
// decision that closed the previous kernel; in a replacement iteration the
// fold g += x', x' = 0 and the partial (g, g) instead.
template <typename T, int PK> __device__ __forceinline__ void body_p (const Args<T> &a, const DevState *sc, bool rep)
{
  const int64_t stride = (int64_t) gridDim.x * blockDim.x;
  if (rep)
    {
      // Group update: fold the accumulated updates into the base, which
      // phase 2 multiplies by A for the true residual.
      double gg = 0.0;
      GRID_STRIDE (i, a.n)
      {
        const T gi = a.g[i] + a.xp[i];
        a.g[i] = gi;
        a.xp[i] = 0;
        gg = fma ((double) gi, (double) gi, gg);
      }
      double vals[1] = { gg };
      const int kg[1] = { kGG };
      store_parts<1> (vals, a.part, a.grid, kg);
      return;
    }
  const T tb = (T) sc->beta, tw = (T) sc->omega;
  if constexpr (PK >= kPreBlock2)
    {
      // block Jacobi: one block row per thread, q = Minv p of the block
      for (int64_t br = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; br < a.nbr; br += stride)
        block_row_apply<T, PK> (a, br, a.p, a.q,
                                [&] (int64_t i) { return a.r[i] + tb * (a.p[i] - tw * a.v[i]); });
      return;
    }
  const bool PRE = PK == kPrePoint;
  // Four grid-stride elements per pass, loads first (the arrays may alias as
  // far as the compiler knows, so it would not hoist them itself).
  int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < a.n; i += 4 * stride)
    {
      T rv[4], pv[4], vv[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
        {
          rv[u] = a.r[i + u * stride];
          pv[u] = a.p[i + u * stride];
          vv[u] = a.v[i + u * stride];
        }
#pragma unroll
      for (int u = 0; u < 4; u++)
        {
          const T pn = rv[u] + tb * (pv[u] - tw * vv[u]); // :286-304
          a.p[i + u * stride] = pn;
          if (PRE)
            a.q[i + u * stride] = a.P[i + u * stride] * pn; // :227-238
        }
    }
  for (; i < a.n; i += stride)
    {
      const T pn = a.r[i] + tb * (a.p[i] - tw * a.v[i]);
      a.p[i] = pn;
      if (PRE)
        a.q[i] = a.P[i] * pn;
    }
}

// phase 3
template <typename T, int PK> __device__ __forceinline__ void body_s (const Args<T> &a, const DevState *sc)
{
  const T ta = (T) sc->alpha;
  const int64_t stride = (int64_t) gridDim.x * blockDim.x;
  if constexpr (PK >= kPreBlock2)
    {
      for (int64_t br = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; br < a.nbr; br += stride)
        block_row_apply<T, PK> (a, br, a.s, a.z, [&] (int64_t i) { return a.r[i] - ta * a.v[i]; });
      return;
    }
  const bool PRE = PK == kPrePoint;
  int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < a.n; i += 4 * stride)
    {
      T rv[4], vv[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
        {
          rv[u] = a.r[i + u * stride];
          vv[u] = a.v[i + u * stride];
        }
#pragma unroll
      for (int u = 0; u < 4; u++)
        {
          const T si = rv[u] - ta * vv[u]; // :306-327
          a.s[i + u * stride] = si;
          if (PRE)
            a.z[i + u * stride] = a.P[i + u * stride] * si;
        }
    }
  for (; i < a.n; i += stride)
    {
      const T si = a.r[i] - ta * a.v[i];
      a.s[i] = si;
      if (PRE)
        a.z[i] = a.P[i] * si;
    }
}

// phase 5: x' += alpha q + omega z, r = s - omega t, partials (rh, r),
// (r, r), (x', x'); its last CTA takes the decision that opens the next
// iteration.
template <typename T, int PK> __device__ __forceinline__ void body_x (const Args<T> &a, const DevState *sc)
{
  const T ta = (T) sc->alpha, tw = (T) sc->omega;
  // (x', x') feeds the replacement bound only: skipped (0) when it is off.
  const bool track = sc->eps > 0.0;
  T rhr = 0, rr = 0, xx = 0;
  const T *qa = PK != kPreNone ? a.q : a.p;
  const T *za = PK != kPreNone ? a.z : a.s;
  const int64_t stride = (int64_t) gridDim.x * blockDim.x;
  int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < a.n; i += 4 * stride)
    {
      T xv[4], qv[4], zv[4], sv[4], tv[4], hv[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
        {
          const int64_t k = i + u * stride;
          xv[u] = a.xp[k];
          qv[u] = qa[k];
          zv[u] = za[k];
          sv[u] = a.s[k];
          tv[u] = a.t[k];
          hv[u] = a.rh[k];
        }
      // Same per-thread accumulation order as one element at a time.
#pragma unroll
      for (int u = 0; u < 4; u++)
        {
          const int64_t k = i + u * stride;
          const T xn = xv[u] + ta * qv[u] + tw * zv[u]; // h = x + alpha q; x = h + omega z
          a.xp[k] = xn;
          const T ri = sv[u] - tw * tv[u];              // :340-357
          a.r[k] = ri;
          rhr = fma (hv[u], ri, rhr);
          rr = fma (ri, ri, rr);
          if (track)
            xx = fma (xn, xn, xx);
        }
    }
  for (; i < a.n; i += stride)
    {
      const T xn = a.xp[i] + ta * qa[i] + tw * za[i];
      a.xp[i] = xn;
      const T ri = a.s[i] - tw * a.t[i];
      a.r[i] = ri;
      rhr = fma (a.rh[i], ri, rhr);
      rr = fma (ri, ri, rr);
      if (track)
        xx = fma (xn, xn, xx);
    }
  double vals[3] = { (double) rhr, (double) rr, (double) xx };
  const int kk[3] = { kRhR, kRR, kXX };
  store_parts<3> (vals, a.part, a.grid, kk);
}

template <typename T, int PK>
__global__ void __launch_bounds__ (kThreads) phase_p (Args<T> a)
{
  const int2 f = flags (a.st);
  if (f.x)
    return;
  body_p<T, PK> (a, a.st, f.y != 0);
}

template <typename T, int PK>
__global__ void __launch_bounds__ (kThreads) phase_s (Args<T> a)
{
  const int2 f = flags (a.st);
  if (f.x || f.y)
    return;
  body_s<T, PK> (a, a.st);
}

// phase 5 ends the iteration: its last CTA takes the decision that opens the
// next one (in a replacement iteration on phase 1 and 2's partials).
template <typename T, int PK>
__global__ void __launch_bounds__ (kThreads) phase_x (Args<T> a)
{
  DevState *st = a.st;
  const int2 f = flags (st);
  if (f.x)
    return;
  if (!f.y)
    body_x<T, PK> (a, st);
  if (!arrive_last (st, a.grid))
    return;
  tail_end (st, a.part, a.grid, f.y != 0);
}

// ------------------------------------------------------------ persistent iteration

// A grid barrier waits at most this long (the longest phase of the largest
// system this engine runs takes milliseconds); past it the CTA records a
// fault and leaves, and so does every CTA behind a later barrier.
constexpr unsigned long long kBarrierLimitNs = 4000000000ull;

// Scalar rows from which the auto launch mode runs the persistent kernel,
// and its CTAs per SM at most (launch bounds: up to 80 registers a thread).
constexpr int64_t kPersistentRows = 1000000;
constexpr int kIterateCtasPerSm = 3;

__device__ __forceinline__ unsigned long long global_ns ()
{
  unsigned long long t;
  asm volatile ("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Barrier over the whole cooperative grid, after which every CTA sees every
// CTA's writes from before it. Thread 0 of each CTA counts the CTA in with an
// acq_rel add; the last one in runs `tail` (the phase's scalar work, with the
// whole CTA, on the device state) before it resets the count and advances
// the generation with a release; the others wait for that with a bounded
// acquire poll. gen is thread 0's copy of the generation. False when the wait
// gave up (the fault is recorded): the caller must return. (Two-level
// arrival through counters of 4 or 16 CTAs, and polls backing off to 32 or
// 256 ns, measured slower on GB300: 33-34 against 29 us per iteration at
// 20 000 rows.)
template <class Tail>
__device__ __forceinline__ bool grid_sync (DevState *st, int grid, unsigned &gen, Tail tail,
                                          unsigned long long limit_ns = kBarrierLimitNs)
{
  __shared__ int s_last, s_ok;
  __syncthreads ();
  cuda::atomic_ref<unsigned, cuda::thread_scope_device> arrive (st->arrive);
  cuda::atomic_ref<unsigned, cuda::thread_scope_device> g (st->gen);
  if (threadIdx.x == 0)
    {
      int ok = 1;
      const int last = arrive.fetch_add (1u, cuda::memory_order_acq_rel) == (unsigned) grid - 1;
      if (!last)
        {
          const unsigned long long t0 = global_ns ();
          unsigned polls = 0;
          while (g.load (cuda::memory_order_acquire) == gen)
            {
              if ((++polls & 255u) == 0 && global_ns () - t0 > limit_ns)
                {
                  ok = 0;
                  cuda::atomic_ref<int, cuda::thread_scope_device> fault (st->fault);
                  fault.store (1, cuda::memory_order_relaxed);
                  break;
                }
              __nanosleep (20);
            }
        }
      gen++;
      s_last = last;
      s_ok = ok;
    }
  __syncthreads ();
  if (s_last)
    {
      tail ();
      __syncthreads ();
      if (threadIdx.x == 0)
        {
          arrive.store (0u, cuda::memory_order_relaxed);
          g.store (gen, cuda::memory_order_release);
        }
    }
  return s_ok != 0;
}

// Up to `iters` BiCGStab iterations in one cooperative launch: the five phase
// bodies separated by grid barriers instead of kernel boundaries, the scalar
// work of a phase done by the last CTA to reach its barrier, on the device
// state, as the last CTA of the phase kernels does it (the same sums in the
// same order: the same bits). The x vector of each product was written by
// other CTAs of this kernel, so the products load it coherently (XCoh).
template <typename T, class Op, int PK>
__global__ void __launch_bounds__ (kThreads, kIterateCtasPerSm) iterate_kernel (Args<T> a, int iters)
{
  DevState *st = a.st;
  unsigned gen = 0;
  if (threadIdx.x == 0)
    gen = cuda::atomic_ref<unsigned, cuda::thread_scope_device> (st->gen).load (cuda::memory_order_relaxed);
  const double *part = a.part;
  const int grid = a.grid;
  auto none = [] () {};
  for (int it = 0; it < iters; it++)
    {
      const int2 f = flags (st);
      if (f.x)
        break;
      const bool rep = f.y != 0;
      body_p<T, PK> (a, st, rep);
      if (!grid_sync (st, grid, gen, none))
        return;
      body_v<T, Op> (a, st, rep);
      if (rep)
        {
          if (!grid_sync (st, grid, gen, [&] () { tail_end (st, part, grid, true); }))
            return;
          continue;
        }
      if (!grid_sync (st, grid, gen, [&] () { tail_v (st, part, grid); }))
        return;
      if (flags (st).x)
        break;
      body_s<T, PK> (a, st);
      if (!grid_sync (st, grid, gen, none))
        return;
      body_t<T, Op> (a);
      if (!grid_sync (st, grid, gen, [&] () { tail_t (st, part, grid); }))
        return;
      if (flags (st).x)
        break;
      body_x<T, PK> (a, st);
      if (!grid_sync (st, grid, gen, [&] () { tail_end (st, part, grid, false); }))
        return;
    }
}

// The grid barrier's bounded wait, exercised: every CTA waits for one CTA
// more than the grid holds, so no CTA is ever last; each gives up after
// limit_ns, records the fault and returns, and the context stays usable.
__global__ void barrier_selftest_kernel (DevState *st, unsigned long long limit_ns)
{
  unsigned gen = 0;
  if (threadIdx.x == 0)
    gen = cuda::atomic_ref<unsigned, cuda::thread_scope_device> (st->gen).load (cuda::memory_order_relaxed);
  grid_sync (st, (int) gridDim.x + 1, gen, [] () {}, limit_ns);
}

// End of a run: x = e (a fresh solve) or x += e (a restart), with e the run's
// result g + x' or, when a snapshot is restored, the snapshot.
template <typename T>
__global__ void finish_kernel (int64_t n, T *x, const T *g, const T *xp, const T *snap, int add)
{
  GRID_STRIDE (i, n)
  {
    const T e = snap ? snap[i] : g[i] + xp[i];
    x[i] = add ? x[i] + e : e;
  }
}

// The run's current iterate g + x' into snap (the best-point copy).
template <typename T> __global__ void snapshot_kernel (int64_t n, const T *g, const T *xp, T *snap)
{
  GRID_STRIDE (i, n)
  snap[i] = g[i] + xp[i];
}

// cA = (entries per scalar row) * ||A||_inf, maxima over rows by atomics on
// the bit patterns (non-negative doubles order like their bits).
template <typename T>
__global__ void row_norm_kernel (int nbr, int bs, const int *rp, const T *vals, unsigned long long *max_abs,
                                 int *max_count)
{
  const int b = bs > 0 ? bs : 1;
  // Each thread keeps its own maxima, then the warp combines them: one
  // atomic per warp, not one per row on two addresses.
  unsigned long long amax = 0;
  int cmax = 0;
  GRID_STRIDE (i, (int64_t) nbr * b)
  {
    const int br = (int) (i / b), r = (int) (i % b);
    double sum = 0.0;
    int count = 0;
    for (int k = rp[br]; k < rp[br + 1]; k++)
      {
        if (bs > 0)
          for (int c = 0; c < bs; c++)
            sum += fabs ((double) vals[(size_t) k * bs * bs + (size_t) r * bs + c]);
        else
          sum += fabs ((double) vals[k]);
        count += b;
      }
    amax = max (amax, (unsigned long long) __double_as_longlong (sum));
    cmax = max (cmax, count);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    {
      amax = max (amax, __shfl_xor_sync (0xffffffffu, amax, off));
      cmax = max (cmax, __shfl_xor_sync (0xffffffffu, cmax, off));
    }
  if ((threadIdx.x & 31) == 0)
    {
      atomicMax (max_abs, amax);
      atomicMax (max_count, cmax);
    }
}

// Point Jacobi from the diagonal blocks: P = 1/a_rr (1 when |a_rr| < 1e-20
// or when the row stores no diagonal), gpu/bicgstab.cu:201-225.
template <typename T>
__global__ void jacobi_kernel (int nbr, int bs, const int *rp, const int *cols, const T *vals, T *P)
{
  GRID_STRIDE (i, (int64_t) nbr * bs)
  {
    const int br = (int) (i / bs), r = (int) (i % bs);
    T d = 1;
    for (int b = rp[br]; b < rp[br + 1]; b++)
      if (cols[b] == br)
        {
          const T a = vals[(size_t) b * bs * bs + r * bs + r];
          d = fabs ((double) a) < 1e-20 ? (T) 1 : (T) 1 / a;
          break;
        }
    P[i] = d;
  }
}

// Block Jacobi: Minv[br] = inverse of the diagonal block of block row br
// (Gauss-Jordan with partial pivoting in FP64, one thread per block row),
// the identity when the row stores no diagonal block or a pivot falls below
// 1e-20 times the block's largest entry: the block form of the point rule
// above (1 where |a_ii| < 1e-20 or no diagonal is stored).
template <typename T>
__global__ void block_jacobi_kernel (int nbr, int bs, const int *rp, const int *cols, const T *vals, T *Minv)
{
  GRID_STRIDE (br, (int64_t) nbr)
  {
    const int e = bs * bs;
    T *out = Minv + (size_t) br * e;
    const T *blk = nullptr;
    for (int b = rp[br]; b < rp[br + 1]; b++)
      if (cols[b] == (int) br)
        {
          blk = vals + (size_t) b * e;
          break;
        }
    double a[kMaxBlockJacobi * kMaxBlockJacobi], inv[kMaxBlockJacobi * kMaxBlockJacobi];
    double amax = 0.0;
    for (int k = 0; k < e; k++)
      {
        a[k] = blk ? (double) blk[k] : 0.0;
        inv[k] = (k / bs == k % bs) ? 1.0 : 0.0;
        amax = fmax (amax, fabs (a[k]));
      }
    bool ok = blk != nullptr && amax > 0.0;
    for (int c = 0; c < bs && ok; c++)
      {
        int piv = c;
        for (int r = c + 1; r < bs; r++)
          if (fabs (a[r * bs + c]) > fabs (a[piv * bs + c]))
            piv = r;
        if (!(fabs (a[piv * bs + c]) >= 1e-20 * amax))
          {
            ok = false;
            break;
          }
        if (piv != c)
          for (int k = 0; k < bs; k++)
            {
              double t = a[c * bs + k];
              a[c * bs + k] = a[piv * bs + k];
              a[piv * bs + k] = t;
              t = inv[c * bs + k];
              inv[c * bs + k] = inv[piv * bs + k];
              inv[piv * bs + k] = t;
            }
        const double d = 1.0 / a[c * bs + c];
        for (int k = 0; k < bs; k++)
          {
            a[c * bs + k] *= d;
            inv[c * bs + k] *= d;
          }
        for (int r = 0; r < bs; r++)
          if (r != c)
            {
              const double f = a[r * bs + c];
              if (f != 0.0)
                for (int k = 0; k < bs; k++)
                  {
                    a[r * bs + k] -= f * a[c * bs + k];
                    inv[r * bs + k] -= f * inv[c * bs + k];
                  }
            }
      }
    for (int k = 0; k < e; k++)
      out[k] = ok ? (T) inv[k] : (T) ((k / bs == k % bs) ? 1 : 0);
  }
}

// ------------------------------------------------------------ dispatch

enum SpmvKind
{
  kCsr8,
  kFlat2,
  kFlat4,
  kFlat8,
  kFlat16,
  kFlat32,
  kTpr3,
  kTprAny
};

template <typename T, int K, class XL = dev::XNc> struct OpOf;
template <typename T, class XL> struct OpOf<T, kCsr8, XL> { using type = CsrOp<T, 8, XL>; };
// Few lanes per block row: every lane then holds whole block lines, so the
// warp-level FP64 instructions are not spent on predicated-off lanes or on
// shuffle-reduction adds (each FP64 warp instruction costs the same issue
// time on GB300's narrow FP64 pipe however many lanes are active).
template <typename T, class XL> struct OpOf<T, kFlat2, XL> { using type = FlatOp<T, 2, 2, XL>; };
template <typename T, class XL> struct OpOf<T, kFlat4, XL> { using type = FlatOp<T, 4, 4, XL>; };
template <typename T, class XL> struct OpOf<T, kFlat8, XL> { using type = FlatOp<T, 8, 4, XL>; };
template <typename T, class XL> struct OpOf<T, kFlat16, XL> { using type = FlatOp<T, 16, 8, XL>; };
template <typename T, class XL> struct OpOf<T, kFlat32, XL> { using type = FlatOp<T, 32, 16, XL>; };
template <typename T, class XL> struct OpOf<T, kTpr3, XL> { using type = TprOp<T, 3, XL>; };
template <typename T, class XL> struct OpOf<T, kTprAny, XL> { using type = TprOp<T, 0, XL>; };

int spmv_kind_for (const bmfp_matrix_s *A)
{
  switch (A->bs)
    {
    case 0:
    case 1: return kCsr8;
    case 2: return kFlat2;
    case 4: return kFlat4;
    case 8: return kFlat8;
    case 16: return kFlat16;
    case 32: return kFlat32;
    case 3: return kTpr3;
    default: return kTprAny;
    }
}

template <typename T, int K>
void launch_spmv_phase (int phase, const Args<T> &a, cudaStream_t s)
{
  using Op = typename OpOf<T, K>::type;
  if (phase == 2)
    phase_v<T, Op><<<a.grid, kThreads, 0, s>>> (a);
  else
    phase_t<T, Op><<<a.grid, kThreads, 0, s>>> (a);
}

template <typename T>
void launch_spmv_dispatch (int kind, int phase, const Args<T> &a, cudaStream_t s)
{
  switch (kind)
    {
    case kCsr8: launch_spmv_phase<T, kCsr8> (phase, a, s); break;
    case kFlat2: launch_spmv_phase<T, kFlat2> (phase, a, s); break;
    case kFlat4: launch_spmv_phase<T, kFlat4> (phase, a, s); break;
    case kFlat8: launch_spmv_phase<T, kFlat8> (phase, a, s); break;
    case kFlat16: launch_spmv_phase<T, kFlat16> (phase, a, s); break;
    case kFlat32: launch_spmv_phase<T, kFlat32> (phase, a, s); break;
    case kTpr3: launch_spmv_phase<T, kTpr3> (phase, a, s); break;
    default: launch_spmv_phase<T, kTprAny> (phase, a, s); break;
    }
}

template <typename T>
void launch_residual (int kind, const Args<T> &a, const T *x, const T *b, T *r, T *y, cudaStream_t s)
{
  switch (kind)
    {
#define BMFP_RES(K) case K: residual_kernel<T, typename OpOf<T, K>::type><<<a.grid, kThreads, 0, s>>> (a, x, b, r, y); break;
      BMFP_RES (kCsr8) BMFP_RES (kFlat2) BMFP_RES (kFlat4) BMFP_RES (kFlat8) BMFP_RES (kFlat16)
      BMFP_RES (kFlat32) BMFP_RES (kTpr3)
#undef BMFP_RES
    default: residual_kernel<T, typename OpOf<T, kTprAny>::type><<<a.grid, kThreads, 0, s>>> (a, x, b, r, y); break;
    }
}

template <typename T>
Args<T> make_args (const bmfp_matrix_s *A, int64_t n, void *x, void *r, void *rh, void *p, void *v,
                   void *q, void *s, void *z, void *t, void *P, void *g, void *xp, double *part, int grid,
                   DevState *st)
{
  Args<T> a;
  a.nbr = A->n_rows;
  a.bs = A->bs ? A->bs : 1;
  a.rp = A->d_row_ptr;
  a.cols = A->d_cols;
  a.vals = (const T *) A->d_vals;
  a.n = n;
  a.x = (T *) x;
  a.r = (T *) r;
  a.rh = (T *) rh;
  a.p = (T *) p;
  a.v = (T *) v;
  a.q = (T *) q;
  a.s = (T *) s;
  a.z = (T *) z;
  a.t = (T *) t;
  a.P = (const T *) P;
  a.g = (T *) g;
  a.xp = (T *) xp;
  a.part = part;
  a.grid = grid;
  a.st = st;
  return a;
}

template <typename T, int PK>
void launch_vector_phase_k (int phase, const Args<T> &a, cudaStream_t s)
{
  if (phase == 1)
    phase_p<T, PK><<<a.grid, kThreads, 0, s>>> (a);
  else if (phase == 3)
    phase_s<T, PK><<<a.grid, kThreads, 0, s>>> (a);
  else
    phase_x<T, PK><<<a.grid, kThreads, 0, s>>> (a);
}

template <typename T> void launch_vector_phase (int pk, int phase, const Args<T> &a, cudaStream_t s)
{
  switch (pk)
    {
    case kPrePoint: launch_vector_phase_k<T, kPrePoint> (phase, a, s); break;
    case kPreBlock2: launch_vector_phase_k<T, kPreBlock2> (phase, a, s); break;
    case kPreBlockAny: launch_vector_phase_k<T, kPreBlockAny> (phase, a, s); break;
    default: launch_vector_phase_k<T, kPreNone> (phase, a, s); break;
    }
}

template <typename T, int K> const void *iterate_for_pre (int pk)
{
  using Op = typename OpOf<T, K, dev::XCoh>::type;
  if (pk == kPreNone)
    return reinterpret_cast<const void *> (&iterate_kernel<T, Op, kPreNone>);
  if (pk == kPrePoint)
    return reinterpret_cast<const void *> (&iterate_kernel<T, Op, kPrePoint>);
  return nullptr; // block Jacobi runs as graphs
}

// The persistent iteration kernel for a product kind and preconditioner, or
// null. Its grid must fit the device at once (3 CTAs of 256 threads per SM,
// 80 registers a thread): the products of bs 8, 16 and 32 need more
// registers than that, and with their long rows the launch gaps the kernel
// saves matter least; they run as graphs.
template <typename T> const void *iterate_for (int kind, int pk)
{
  switch (kind)
    {
    case kCsr8: return iterate_for_pre<T, kCsr8> (pk);
    case kFlat2: return iterate_for_pre<T, kFlat2> (pk);
    case kFlat4: return iterate_for_pre<T, kFlat4> (pk);
    case kTpr3: return iterate_for_pre<T, kTpr3> (pk);
    case kTprAny: return iterate_for_pre<T, kTprAny> (pk);
    default: return nullptr;
    }
}

// Unit roundoff of the engine's precision (replacement bound).
double unit_roundoff (int dtype) { return dtype == BMFP_R64F ? 0x1p-53 : 0x1p-24; }

// cA = max entries per scalar row * max absolute row sum of A (synchronises).
int matrix_bound (const bmfp_matrix_s *A, int grid, double *cA, cudaStream_t s)
{
  struct Maxima
  {
    unsigned long long abs_bits;
    int count;
  };
  Maxima *d = nullptr;
  BMFP_CUDA (cudaMallocAsync (&d, sizeof (Maxima), s));
  BMFP_CUDA (cudaMemsetAsync (d, 0, sizeof (Maxima), s));
  if (A->dtype == BMFP_R64F)
    row_norm_kernel<double><<<grid, kThreads, 0, s>>> (A->n_rows, A->bs, A->d_row_ptr, (const double *) A->d_vals,
                                                        &d->abs_bits, &d->count);
  else
    row_norm_kernel<float><<<grid, kThreads, 0, s>>> (A->n_rows, A->bs, A->d_row_ptr, (const float *) A->d_vals,
                                                       &d->abs_bits, &d->count);
  cudaError_t e = cudaGetLastError ();
  Maxima h{};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (&h, d, sizeof (Maxima), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync (d, s);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize (s);
  if (e != cudaSuccess)
    return cuda_fail (e, "matrix_bound", __FILE__, __LINE__);
  double amax;
  const long long bits = (long long) h.abs_bits;
  std::memcpy (&amax, &bits, sizeof amax);
  *cA = (double) h.count * amax;
  return BMFP_SUCCESS;
}
} // namespace

// ------------------------------------------------------------ WideEngine

WideEngine::~WideEngine ()
{
  if (graph_)
    cudaGraphExecDestroy (graph_);
  if (capture_stream_)
    cudaStreamDestroy (capture_stream_);
  for (cudaEvent_t e : ev_)
    if (e)
      cudaEventDestroy (e);
  for (void *ptr : { x_, r_, rh_, p_, v_, q_, s_, z_, t_, P_, g_, xp_ })
    cudaFree (ptr);
  cudaFree (part_);
  cudaFree (state_);
  if (h_state_)
    cudaFreeHost (h_state_);
}

int WideEngine::init (const bmfp_matrix_s *A, int precond, int chunk, cudaStream_t stream, int ctas_per_sm,
                      int launch_mode)
{
  if (!A)
    return fail (BMFP_ERROR_INVALID_VALUE, "null matrix");
  const int bs = A->bs ? A->bs : 1;
  if (precond == BMFP_PRECOND_BLOCK_JACOBI && bs > kMaxBlockJacobi)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "block Jacobi takes bs <= %d (bs %d)", kMaxBlockJacobi, bs);
  if (A->bs && A->n_rows != A->n_cols)
    return fail (BMFP_ERROR_INVALID_VALUE, "BiCGStab needs a square matrix");
  if (!A->bs && A->n_rows != A->n_cols)
    return fail (BMFP_ERROR_INVALID_VALUE, "BiCGStab needs a square matrix");
  A_ = A;
  dtype_ = A->dtype;
  jacobi_ = precond != BMFP_PRECOND_NONE;
  const bool block = precond == BMFP_PRECOND_BLOCK_JACOBI;
  pre_kind_ = !jacobi_ ? kPreNone : !block ? kPrePoint : bs == 2 ? kPreBlock2 : kPreBlockAny;
  replace_ = dtype_ == BMFP_R64F;
  chunk_ = std::max (1, std::min (chunk, 256));
  n_ = (int64_t) A->n_rows * bs;
  spmv_kind_ = spmv_kind_for (A);
  // Flat phases need 16-byte aligned values; cudaMalloc'd handles always are.
  int dev = 0, sms = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  BMFP_CUDA (cudaDeviceGetAttribute (&sms, cudaDevAttrMultiProcessorCount, dev));
  // Persistent iterations need a cooperative launch whose CTAs all fit on
  // the device at once: at most kIterateCtasPerSm CTAs per SM (the kernel's
  // launch bounds). Auto takes them from kPersistentRows up (measured on the
  // Q4 elasticity operator, FP64, us per iteration, graph at 4 CTAs per SM /
  // persistent at 3: 500 000 rows 79.3 / 79.9, 1.1 M rows 147.7 / 134.3,
  // 2 M rows 251.3 / 234.0; at 4 CTAs per SM and 64 registers the
  // persistent kernel spilled and took 84.2 / 142.2 / 234.0).
  iterate_ = nullptr;
  int cps = std::max (1, std::min (ctas_per_sm, 8));
  if (launch_mode == BMFP_LAUNCH_PERSISTENT || (launch_mode == BMFP_LAUNCH_AUTO && n_ >= kPersistentRows))
    {
      const void *fn = dtype_ == BMFP_R64F ? iterate_for<double> (spmv_kind_, pre_kind_)
                                           : iterate_for<float> (spmv_kind_, pre_kind_);
      int coop = 0, per_sm = 0;
      BMFP_CUDA (cudaDeviceGetAttribute (&coop, cudaDevAttrCooperativeLaunch, dev));
      if (fn && coop)
        BMFP_CUDA (cudaOccupancyMaxActiveBlocksPerMultiprocessor (&per_sm, fn, kThreads, 0));
      if (fn && coop && per_sm >= 1)
        {
          iterate_ = fn;
          cps = std::min (cps, per_sm);
        }
      else if (launch_mode == BMFP_LAUNCH_PERSISTENT)
        return fail (BMFP_ERROR_NOT_SUPPORTED,
                     "persistent iterations need no preconditioner or point Jacobi, bs other than 8, 16 "
                     "and 32, and a device with cooperative launch");
    }
  // A few CTAs per SM, never more than the rows need.
  const int64_t want = std::max<int64_t> (1, (n_ + kThreads - 1) / kThreads);
  grid_ = (int) std::min<int64_t> ((int64_t) sms * cps, want);
  const size_t S = dtype_size (dtype_);
  const size_t vb = S * (size_t) std::max<int64_t> (n_, 1);
  for (void **ptr : { &x_, &r_, &rh_, &p_, &v_, &s_, &t_, &g_, &xp_ })
    BMFP_CUDA (cudaMalloc (ptr, vb));
  BMFP_CUDA (cudaMemsetAsync (x_, 0, vb, stream));
  if (jacobi_)
    {
      BMFP_CUDA (cudaMalloc (&q_, vb));
      BMFP_CUDA (cudaMalloc (&z_, vb));
      BMFP_CUDA (cudaMalloc (&P_, block ? vb * (size_t) bs : vb)); // block: bs x bs per block row
      if (block && dtype_ == BMFP_R64F)
        block_jacobi_kernel<double><<<grid_, kThreads, 0, stream>>> (A->n_rows, bs, A->d_row_ptr, A->d_cols,
                                                                      (const double *) A->d_vals, (double *) P_);
      else if (block)
        block_jacobi_kernel<float><<<grid_, kThreads, 0, stream>>> (A->n_rows, bs, A->d_row_ptr, A->d_cols,
                                                                     (const float *) A->d_vals, (float *) P_);
      else if (dtype_ == BMFP_R64F)
        jacobi_kernel<double><<<grid_, kThreads, 0, stream>>> (A->n_rows, bs, A->d_row_ptr, A->d_cols,
                                                                (const double *) A->d_vals, (double *) P_);
      else
        jacobi_kernel<float><<<grid_, kThreads, 0, stream>>> (A->n_rows, bs, A->d_row_ptr, A->d_cols,
                                                               (const float *) A->d_vals, (float *) P_);
      BMFP_LAUNCH_CHECK ();
    }
  else
    {
      q_ = nullptr;
      z_ = nullptr;
    }
  part_bytes_ = sizeof (double) * (size_t) kParts * grid_;
  BMFP_CUDA (cudaMalloc (&part_, part_bytes_));
  BMFP_CUDA (cudaMemsetAsync (part_, 0, part_bytes_, stream));
  BMFP_CUDA (cudaMalloc (&state_, sizeof (DevState)));
  BMFP_CUDA (cudaMemsetAsync (state_, 0, sizeof (DevState), stream));
  BMFP_CUDA (cudaMallocHost (&h_state_, 2 * sizeof (DevState)));
  BMFP_CUDA (cudaEventCreateWithFlags (&ev_[0], cudaEventDisableTiming));
  BMFP_CUDA (cudaEventCreateWithFlags (&ev_[1], cudaEventDisableTiming));
  BMFP_CUDA (cudaStreamCreateWithFlags (&capture_stream_, cudaStreamNonBlocking));
  int rc = matrix_bound (A, grid_, &cA_, stream); // synchronises the stream
  if (rc != BMFP_SUCCESS)
    return rc;
  return iterate_ ? BMFP_SUCCESS : capture (capture_stream_);
}

int WideEngine::launch_iterations (cudaStream_t s)
{
  void *q = jacobi_ ? q_ : p_;
  void *z = jacobi_ ? z_ : s_;
  int iters = chunk_;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3 ((unsigned) grid_);
  cfg.blockDim = dim3 (kThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if (dtype_ == BMFP_R64F)
    {
      Args<double> a
        = make_args<double> (A_, n_, x_, r_, rh_, p_, v_, q, s_, z, t_, P_, g_, xp_, part_, grid_, state_);
      void *args[] = { &a, &iters };
      e = cudaLaunchKernelExC (&cfg, iterate_, args);
    }
  else
    {
      Args<float> a
        = make_args<float> (A_, n_, x_, r_, rh_, p_, v_, q, s_, z, t_, P_, g_, xp_, part_, grid_, state_);
      void *args[] = { &a, &iters };
      e = cudaLaunchKernelExC (&cfg, iterate_, args);
    }
  if (e != cudaSuccess)
    return cuda_fail (e, "cooperative launch of the iteration kernel", __FILE__, __LINE__);
  return BMFP_SUCCESS;
}

int WideEngine::launch_phase (int phase, cudaStream_t s)
{
  void *q = jacobi_ ? q_ : p_;
  void *z = jacobi_ ? z_ : s_;
  if (dtype_ == BMFP_R64F)
    {
      Args<double> a
        = make_args<double> (A_, n_, x_, r_, rh_, p_, v_, q, s_, z, t_, P_, g_, xp_, part_, grid_, state_);
      if (phase == 2 || phase == 4)
        launch_spmv_dispatch<double> (spmv_kind_, phase, a, s);
      else
        launch_vector_phase<double> (pre_kind_, phase, a, s);
    }
  else
    {
      Args<float> a
        = make_args<float> (A_, n_, x_, r_, rh_, p_, v_, q, s_, z, t_, P_, g_, xp_, part_, grid_, state_);
      if (phase == 2 || phase == 4)
        launch_spmv_dispatch<float> (spmv_kind_, phase, a, s);
      else
        launch_vector_phase<float> (pre_kind_, phase, a, s);
    }
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int WideEngine::capture (cudaStream_t s)
{
  cudaGraph_t g = nullptr;
  BMFP_CUDA (cudaStreamBeginCapture (s, cudaStreamCaptureModeThreadLocal));
  int st = BMFP_SUCCESS;
  for (int it = 0; it < chunk_ && st == BMFP_SUCCESS; it++)
    for (int ph = 1; ph <= 5 && st == BMFP_SUCCESS; ph++)
      st = launch_phase (ph, s);
  cudaError_t e = cudaStreamEndCapture (s, &g);
  if (st != BMFP_SUCCESS)
    {
      if (g)
        cudaGraphDestroy (g);
      return st;
    }
  if (e != cudaSuccess)
    return cuda_fail (e, "cudaStreamEndCapture", __FILE__, __LINE__);
  e = cudaGraphInstantiate (&graph_, g, 0);
  cudaGraphDestroy (g);
  if (e != cudaSuccess)
    return cuda_fail (e, "cudaGraphInstantiate", __FILE__, __LINE__);
  return BMFP_SUCCESS;
}

int WideEngine::start (bool zero, const void *c, double tol, int max_iter, double norm_b, int iter0, bool new_shadow,
                        cudaStream_t s)
{
  void *q = jacobi_ ? q_ : p_;
  void *z = jacobi_ ? z_ : s_;
  const double eps = replace_ ? unit_roundoff (dtype_) : 0.0;
  c_ = c;
  from_zero_ = zero;
  if (dtype_ == BMFP_R64F)
    {
      const Args<double> a
        = make_args<double> (A_, n_, x_, r_, rh_, p_, v_, q, s_, z, t_, P_, g_, xp_, part_, grid_, state_);
      if (zero)
        start_kernel<double, true><<<grid_, kThreads, 0, s>>> (a, (const double *) c, tol, max_iter, norm_b, iter0,
                                                                eps, cA_, new_shadow ? 1 : 0);
      else
        start_kernel<double, false><<<grid_, kThreads, 0, s>>> (a, (const double *) c, tol, max_iter, norm_b,
                                                                 iter0, eps, cA_, new_shadow ? 1 : 0);
    }
  else
    {
      const Args<float> a
        = make_args<float> (A_, n_, x_, r_, rh_, p_, v_, q, s_, z, t_, P_, g_, xp_, part_, grid_, state_);
      if (zero)
        start_kernel<float, true><<<grid_, kThreads, 0, s>>> (a, (const float *) c, tol, max_iter, norm_b, iter0,
                                                               eps, cA_, new_shadow ? 1 : 0);
      else
        start_kernel<float, false><<<grid_, kThreads, 0, s>>> (a, (const float *) c, tol, max_iter, norm_b, iter0,
                                                                eps, cA_, new_shadow ? 1 : 0);
    }
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int WideEngine::start_zero (const void *d_b, double tol, int max_iter, cudaStream_t s)
{
  return start (true, d_b, tol, max_iter, -1.0, 0, false, s);
}

int WideEngine::start_residual (const void *d_r, double tol, int max_iter_total, double norm_b,
                                cudaStream_t s, int iter0, bool new_shadow)
{
  return start (false, d_r, tol, max_iter_total, norm_b, iter0, new_shadow, s);
}

namespace
{
// Stops a run from the host side: the phase kernels of the graphs still to
// come see done and return at once.
__global__ void stop_kernel (DevState *st)
{
  st->done = 1;
  st->status = kStateBreakdown;
}
} // namespace

// A barrier of the persistent kernel gave up: the barrier words may hold a
// partial count, so the state (and the partials) are cleared (the next solve
// starts a new run) and the solve fails.
int WideEngine::barrier_fault (cudaStream_t s)
{
  BMFP_CUDA (cudaStreamSynchronize (s));
  BMFP_CUDA (cudaMemsetAsync (state_, 0, sizeof (DevState), s));
  BMFP_CUDA (cudaMemsetAsync (part_, 0, part_bytes_, s));
  BMFP_CUDA (cudaStreamSynchronize (s));
  return fail (BMFP_ERROR_TIMEOUT, "a grid barrier of the iteration kernel gave up waiting");
}

int WideEngine::run (cudaStream_t s, DevState *out, void *d_snap, double *snap_rr, int stall)
{
  // Keep one graph in flight while the host inspects the previous one.
  long k = 0;
  const long limit = 1 + (long) 1e9 / chunk_;
  double best = INFINITY;                              // smallest (r, r) polled
  const double snap_in = snap_rr ? *snap_rr : INFINITY;
  double snap_at = snap_in;                            // (r, r) of the last copy
  long snap_k = -1;                                    // graph whose end the copy holds
  double mark = INFINITY;                              // best (r, r) at the last halving
  int mark_it = 0;                                     // iteration of that halving
  bool stopping = false;
  for (;; k++)
    {
      if (iterate_)
        {
          const int rc = launch_iterations (s);
          if (rc != BMFP_SUCCESS)
            return rc;
        }
      else
        BMFP_CUDA (cudaGraphLaunch (graph_, s));
      BMFP_CUDA (cudaMemcpyAsync (&h_state_[k & 1], state_, sizeof (DevState), cudaMemcpyDeviceToHost, s));
      BMFP_CUDA (cudaEventRecord (ev_[k & 1], s));
      if (k > 0)
        {
          BMFP_CUDA (cudaEventSynchronize (ev_[(k - 1) & 1]));
          const DevState &h = h_state_[(k - 1) & 1];
          if (h.fault)
            return barrier_fault (s);
          if (snap_k == k - 1)
            *snap_rr = snap_at = h.rr;
          if (h.done)
            break;
          if (h.rr < best)
            best = h.rr;
          // The iterate after graph k (queued behind it); its (r, r) is read
          // at the next poll.
          if (d_snap && snap_rr && h.rr < 0.25 * snap_at && snap_k != k - 1)
            {
              if (dtype_ == BMFP_R64F)
                snapshot_kernel<double><<<grid_, kThreads, 0, s>>> (n_, (const double *) g_, (const double *) xp_,
                                                                     (double *) d_snap);
              else
                snapshot_kernel<float><<<grid_, kThreads, 0, s>>> (n_, (const float *) g_, (const float *) xp_,
                                                                    (float *) d_snap);
              BMFP_LAUNCH_CHECK ();
              snap_k = k;
              snap_at = h.rr;
            }
          if (mark == INFINITY)
            mark = h.norm_b * h.norm_b;
          if (best <= 0.25 * mark)
            {
              mark = best;
              mark_it = h.iter;
            }
          const bool stalled = stall > 0 && h.iter - mark_it >= stall;
          if (!stopping && (!(h.rr <= 1e16 * best) || stalled))
            {
              stop_kernel<<<1, 1, 0, s>>> (state_);
              BMFP_LAUNCH_CHECK ();
              stopping = true;
            }
        }
      if (k > limit)
        return fail (BMFP_ERROR_TIMEOUT, "solver did not stop");
    }
  BMFP_CUDA (cudaStreamSynchronize (s));
  *out = h_state_[k & 1];
  if (out->fault)
    return barrier_fault (s);
  if (snap_k == k && snap_rr)
    *snap_rr = out->rr;
  // The run's result into x: the snapshot when the run ended above the best
  // point it passed (and that point is a copy of this run), else g + x'.
  const bool restore = d_snap && snap_rr && snap_k >= 0 && out->status != kStateConverged && *snap_rr < snap_in
                       && !(out->rr <= *snap_rr);
  if (restore)
    out->rr = *snap_rr;
  const int add = from_zero_ ? 0 : 1;
  if (dtype_ == BMFP_R64F)
    finish_kernel<double><<<grid_, kThreads, 0, s>>> (n_, (double *) x_, (const double *) g_, (const double *) xp_,
                                                       restore ? (const double *) d_snap : nullptr, add);
  else
    finish_kernel<float><<<grid_, kThreads, 0, s>>> (n_, (float *) x_, (const float *) g_, (const float *) xp_,
                                                      restore ? (const float *) d_snap : nullptr, add);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int WideEngine::true_residual (const void *d_b, void *d_r, double *rr, double *bb, cudaStream_t s)
{
  if (dtype_ == BMFP_R64F)
    {
      Args<double> a
        = make_args<double> (A_, n_, x_, r_, rh_, p_, v_, p_, s_, s_, t_, P_, g_, xp_, part_, grid_, state_);
      launch_residual<double> (spmv_kind_, a, (const double *) x_, (const double *) d_b, (double *) d_r,
                               (double *) t_, s);
    }
  else
    {
      Args<float> a
        = make_args<float> (A_, n_, x_, r_, rh_, p_, v_, p_, s_, s_, t_, P_, g_, xp_, part_, grid_, state_);
      launch_residual<float> (spmv_kind_, a, (const float *) x_, (const float *) d_b, (float *) d_r,
                              (float *) t_, s);
    }
  BMFP_LAUNCH_CHECK ();
  std::vector<double> h (2 * (size_t) grid_);
  BMFP_CUDA (cudaMemcpyAsync (h.data (), part_ + (size_t) kResRR * grid_, sizeof (double) * 2 * grid_,
                              cudaMemcpyDeviceToHost, s));
  BMFP_CUDA (cudaStreamSynchronize (s));
  double a = 0.0, b = 0.0;
  for (int i = 0; i < grid_; i++)
    {
      a += h[i];
      b += h[grid_ + i];
    }
  *rr = a;
  *bb = b;
  return BMFP_SUCCESS;
}
// ------------------------------------------------------------ raw buffers
// Launchers over caller-provided buffers, for the entry point that
// allocates nothing (noalloc.cu). They run the same phase kernels as
// WideEngine, without graphs, and without residual replacement (the
// reference's plain recurrences).

int barrier_selftest (double limit_s, int *fault, double *elapsed_s, cudaStream_t s)
{
  if (!(limit_s > 0.0 && limit_s <= 1.0))
    return fail (BMFP_ERROR_INVALID_VALUE, "the self-test waits between 0 and 1 s (got %g)", limit_s);
  int dev = 0, sms = 0, coop = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  BMFP_CUDA (cudaDeviceGetAttribute (&sms, cudaDevAttrMultiProcessorCount, dev));
  BMFP_CUDA (cudaDeviceGetAttribute (&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "no cooperative launch on this device");
  DevState *st = nullptr;
  BMFP_CUDA (cudaMalloc (&st, sizeof (DevState)));
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaMemsetAsync (st, 0, sizeof (DevState), s);
  if (e == cudaSuccess)
    e = cudaEventCreate (&a);
  if (e == cudaSuccess)
    e = cudaEventCreate (&b);
  if (e == cudaSuccess)
    e = cudaEventRecord (a, s);
  if (e == cudaSuccess)
    {
      unsigned long long limit_ns = (unsigned long long) (limit_s * 1e9);
      void *args[] = { &st, &limit_ns };
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3 ((unsigned) sms);
      cfg.blockDim = dim3 (kThreads);
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      e = cudaLaunchKernelExC (&cfg, (const void *) barrier_selftest_kernel, args);
    }
  DevState h{};
  if (e == cudaSuccess)
    e = cudaEventRecord (b, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (&h, st, sizeof (DevState), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize (s);
  float ms = 0.0f;
  if (e == cudaSuccess)
    e = cudaEventElapsedTime (&ms, a, b);
  if (a)
    cudaEventDestroy (a);
  if (b)
    cudaEventDestroy (b);
  cudaFree (st);
  if (e != cudaSuccess)
    return cuda_fail (e, "barrier self-test", __FILE__, __LINE__);
  if (fault)
    *fault = h.fault;
  if (elapsed_s)
    *elapsed_s = ms * 1e-3;
  return BMFP_SUCCESS;
}

int raw_solve_grid (int64_t n, int *grid)
{
  int dev = 0, sms = 0;
  BMFP_CUDA (cudaGetDevice (&dev));
  BMFP_CUDA (cudaDeviceGetAttribute (&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t want = std::max<int64_t> (1, (n + kThreads - 1) / kThreads);
  *grid = (int) std::min<int64_t> ((int64_t) sms * 4, want);
  return BMFP_SUCCESS;
}

namespace
{
int raw_kind (const RawSolve &b)
{
  const int kind = spmv_kind_for (&b.A);
  if (b.aligned)
    return kind;
  // The vectorised row routine needs 16-byte aligned values; fall back to
  // scalar loads for caller arrays that are not.
  return (kind == kCsr8 || kind == kTpr3) ? kind : kTprAny;
}

template <typename T> Args<T> raw_args (const RawSolve &b)
{
  void *q = b.jacobi ? b.q : b.p;
  void *z = b.jacobi ? b.z : b.s;
  return make_args<T> (&b.A, b.n, b.x, b.r, b.rh, b.p, b.v, q, b.s, z, b.t, b.P, b.g, b.xp, b.part, b.grid, b.st);
}
} // namespace

int raw_jacobi (const RawSolve &b, cudaStream_t s)
{
  const int bs = b.A.bs ? b.A.bs : 1;
  if (b.A.dtype == BMFP_R64F)
    jacobi_kernel<double><<<b.grid, kThreads, 0, s>>> (b.A.n_rows, bs, b.A.d_row_ptr, b.A.d_cols,
                                                       (const double *) b.A.d_vals, (double *) b.P);
  else
    jacobi_kernel<float><<<b.grid, kThreads, 0, s>>> (b.A.n_rows, bs, b.A.d_row_ptr, b.A.d_cols,
                                                      (const float *) b.A.d_vals, (float *) b.P);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int raw_start (const RawSolve &b, const void *d_rhs, double tol, int max_iter, cudaStream_t s)
{
  if (b.A.dtype == BMFP_R64F)
    start_kernel<double, true><<<b.grid, kThreads, 0, s>>> (raw_args<double> (b), (const double *) d_rhs,
                                                            tol, max_iter, -1.0, 0, 0.0, 0.0, 0);
  else
    start_kernel<float, true><<<b.grid, kThreads, 0, s>>> (raw_args<float> (b), (const float *) d_rhs,
                                                           tol, max_iter, -1.0, 0, 0.0, 0.0, 0);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int raw_phase (const RawSolve &b, int phase, cudaStream_t s)
{
  const int kind = raw_kind (b);
  if (b.A.dtype == BMFP_R64F)
    {
      const Args<double> a = raw_args<double> (b);
      if (phase == 2 || phase == 4)
        launch_spmv_dispatch<double> (kind, phase, a, s);
      else
        launch_vector_phase<double> (b.jacobi ? kPrePoint : kPreNone, phase, a, s);
    }
  else
    {
      const Args<float> a = raw_args<float> (b);
      if (phase == 2 || phase == 4)
        launch_spmv_dispatch<float> (kind, phase, a, s);
      else
        launch_vector_phase<float> (b.jacobi ? kPrePoint : kPreNone, phase, a, s);
    }
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}

int raw_finish (const RawSolve &b, cudaStream_t s)
{
  if (b.A.dtype == BMFP_R64F)
    finish_kernel<double><<<b.grid, kThreads, 0, s>>> (b.n, (double *) b.x, (const double *) b.g,
                                                       (const double *) b.xp, nullptr, 0);
  else
    finish_kernel<float><<<b.grid, kThreads, 0, s>>> (b.n, (float *) b.x, (const float *) b.g, (const float *) b.xp,
                                                      nullptr, 0);
  BMFP_LAUNCH_CHECK ();
  return BMFP_SUCCESS;
}
} // namespace bmfp
