// Batched BiCGStab: many independent systems of uneven size in ONE persistent
// launch (captured in a CUDA graph together with the work-queue reset).
//
// A "team" is a thread-block cluster (1, 2, 4 or 8 CTAs; two CTAs of 512
// threads fit an SM, so two teams share each SM's FP64 pipe). Teams
// pull systems from a queue ordered largest first (longest-processing-time
// scheduling) and run the whole solve of a system on their own: BiCGStab
// phases separated by hardware cluster barriers, dot products reduced
// CTA-locally and then across the cluster through distributed shared memory,
// always in rank order. Nothing in a system's arithmetic depends on which
// team, which SMs or which other systems share the launch, so a system's
// result is bitwise the same alone and inside any batch solved with the same
// configuration. There are no spin waits: the only waits are cluster and CTA
// barriers that every thread of the team reaches the same number of times
// (every loop decision is taken from team-wide sums).
//
// Precision modes per system, as for the single-system solver:
//  FP64   BiCGStab in FP64, then b - A x in FP64 and restarts from it while
//         each restart still cuts the true residual by 10 % or more;
//  FP32   BiCGStab in FP32 on an FP32 copy of the values;
//  MIXED  FP32 inner BiCGStab, FP64 true residual / update / outer norm
//         (iterative refinement), finishing in FP64 when a refinement step
//         cuts the residual by less than 4x.
// Scalars (alpha, beta, omega, norms) are computed by one thread per CTA and
// shared through shared memory: GB300's FP64 pipe is too narrow to evaluate
// divides and square roots in every thread.
#include "batch.h"
#include "spmv_core.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <vector>

namespace cg = cooperative_groups;

namespace bmfp
{
namespace
{
constexpr int kMaxThreads = 1024;
constexpr int kLaunchThreads = 512; // the batch kernel's launch bounds

__device__ __forceinline__ double warp_sum_d (double v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    v += __shfl_xor_sync (0xffffffffu, v, off);
  return v;
}

// Team-wide sums of NK values, fixed order: warps, then CTAs by rank.
template <int NK>
__device__ void team_sum (cg::cluster_group &cl, double (&v)[NK], double (&out)[NK])
{
  __shared__ double sh_w[NK][kMaxThreads / 32];
  __shared__ double sh_cta[NK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NK; k++)
    {
      const double s = warp_sum_d (v[k]);
      if (lane == 0)
        sh_w[k][w] = s;
    }
  __syncthreads ();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NK; k++)
      {
        double a = 0.0;
        for (int i = 0; i < nw; i++)
          a += sh_w[k][i];
        sh_cta[k] = a;
      }
  cl.sync ();
  // Thread 0 adds the CTAs' totals in rank order; the second cluster barrier
  // publishes the sum to the CTA and keeps sh_cta alive until every CTA has
  // read it. (Every thread summing the ranks itself issued size warp-wide
  // FP64 adds per warp and value on GB300's narrow FP64 pipe.)
  __shared__ double sh_sum[NK];
  if (threadIdx.x == 0)
    {
      const unsigned size = cl.num_blocks ();
#pragma unroll
      for (int k = 0; k < NK; k++)
        {
          double a = 0.0;
          for (unsigned r = 0; r < size; r++)
            a += *cl.map_shared_rank (&sh_cta[k], r);
          sh_sum[k] = a;
        }
    }
  cl.sync ();
#pragma unroll
  for (int k = 0; k < NK; k++)
    out[k] = sh_sum[k];
}

// Team-wide maxima of NK non-negative values.
template <int NK>
__device__ void team_max (cg::cluster_group &cl, double (&v)[NK], double (&out)[NK])
{
  __shared__ double sh_w[NK][kMaxThreads / 32];
  __shared__ double sh_cta[NK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NK; k++)
    {
      double m = v[k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        m = fmax (m, __shfl_xor_sync (0xffffffffu, m, off));
      if (lane == 0)
        sh_w[k][w] = m;
    }
  __syncthreads ();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NK; k++)
      {
        double a = 0.0;
        for (int i = 0; i < nw; i++)
          a = fmax (a, sh_w[k][i]);
        sh_cta[k] = a;
      }
  cl.sync ();
  __shared__ double sh_max[NK];
  if (threadIdx.x == 0)
    {
      const unsigned size = cl.num_blocks ();
#pragma unroll
      for (int k = 0; k < NK; k++)
        {
          double a = 0.0;
          for (unsigned r = 0; r < size; r++)
            a = fmax (a, *cl.map_shared_rank (&sh_cta[k], r));
          sh_max[k] = a;
        }
    }
  cl.sync ();
#pragma unroll
  for (int k = 0; k < NK; k++)
    out[k] = sh_max[k];
}

template <typename T> struct TeamSys
{
  int nbr, bs;
  int64_t n;
  const int *rp, *cols;
  const T *vals;
  T *r, *rh, *p, *v, *s, *t;
};

struct TeamIdx
{
  int64_t elem0, elem_stride; // elementwise ownership
  int64_t group0, group_stride; // SpMV row-group ownership
};

// Row-group loop of one SpMV over the team: FLAT (bs 2, 16-byte loads),
// CSR (bs 1) or TPR (any bs <= 32, warp per block row).
enum BatchOp
{
  kOpFlat2 = 0,
  kOpCsr = 1,
  kOpTpr = 2
};

template <typename T, int OP> struct TeamOp;
template <typename T> struct TeamOp<T, kOpFlat2>
{
  static constexpr int G = 2;
  template <class Epi>
  __device__ static void run (const TeamSys<T> &S, const TeamIdx &ix, const T *x, T *y, Epi &e)
  {
    for (int64_t row = ix.group0; row < S.nbr; row += ix.group_stride)
      core::flat_row<T, 2, 2, 4> ((int) row, S.rp, S.cols, S.vals, x, y, e);
  }
};
template <typename T> struct TeamOp<T, kOpCsr>
{
  static constexpr int G = 4;
  template <class Epi>
  __device__ static void run (const TeamSys<T> &S, const TeamIdx &ix, const T *x, T *y, Epi &e)
  {
    for (int64_t row = ix.group0; row < S.nbr; row += ix.group_stride)
      core::csr_row<T, 4> ((int) row, S.rp, S.cols, S.vals, x, y, e);
  }
};
template <typename T> struct TeamOp<T, kOpTpr>
{
  static constexpr int G = 32;
  template <class Epi>
  __device__ static void run (const TeamSys<T> &S, const TeamIdx &ix, const T *x, T *y, Epi &e)
  {
    for (int64_t row = ix.group0; row < S.nbr; row += ix.group_stride)
      core::tpr_row<T, 0> ((int) row, S.bs, S.rp, S.cols, S.vals, x, y, e);
  }
};

template <int G> __device__ TeamIdx team_index (const cg::cluster_group &cl)
{
  TeamIdx ix;
  const int64_t rank = cl.block_rank (), size = cl.num_blocks ();
  ix.elem0 = rank * blockDim.x + threadIdx.x;
  ix.elem_stride = size * blockDim.x;
  const int64_t groups_per_cta = blockDim.x / G;
  ix.group0 = rank * groups_per_cta + threadIdx.x / G;
  ix.group_stride = size * groups_per_cta;
  return ix;
}

template <typename T> struct EpiDotT
{
  const T *a;
  double acc = 0.0;
  __device__ void operator() (int64_t i, T y) { acc = fma ((double) a[i], (double) y, acc); }
};
template <typename T> struct EpiTST
{
  const T *s;
  double ts = 0.0, tt = 0.0;
  __device__ void operator() (int64_t i, T t)
  {
    ts = fma ((double) s[i], (double) t, ts);
    tt = fma ((double) t, (double) t, tt);
  }
};
struct EpiResid
{
  const double *b;
  double *r;
  double rr = 0.0, bb = 0.0;
  __device__ void operator() (int64_t i, double y)
  {
    const double ri = b[i] - y;
    r[i] = ri;
    rr = fma (ri, ri, rr);
    bb = fma (b[i], b[i], bb);
  }
};

// Residual replacement: r = b - A x with (rh, r) and (r, r).
struct EpiReplaceT
{
  const double *b;
  double *r;
  const double *rh;
  double rhr = 0.0, rr = 0.0;
  __device__ void operator() (int64_t i, double y)
  {
    const double ri = b[i] - y;
    r[i] = ri;
    rhr = fma (rh[i], ri, rhr);
    rr = fma (ri, ri, rr);
  }
};

// cA = (entries per scalar row) * ||A||_inf of one system, over the team:
// the residual-replacement bound of team_bicgstab.
template <typename T>
__device__ double team_matrix_bound (cg::cluster_group &cl, const TeamSys<T> &S)
{
  const TeamIdx ix = team_index<1> (cl);
  double amax = 0.0, cmax = 0.0;
  for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
    {
      const int br = (int) (i / S.bs), r = (int) (i % S.bs);
      double sum = 0.0;
      int count = 0;
      for (int k = S.rp[br]; k < S.rp[br + 1]; k++)
        {
          for (int c = 0; c < S.bs; c++)
            sum += fabs ((double) S.vals[(size_t) k * S.bs * S.bs + (size_t) r * S.bs + c]);
          count += S.bs;
        }
      amax = fmax (amax, sum);
      cmax = fmax (cmax, (double) count);
    }
  double in[2] = { amax, cmax }, out[2];
  team_max<2> (cl, in, out);
  return out[0] * out[1];
}

struct SolveOut
{
  int iters = 0;
  int status = 0; // kState*
  double rec_rel = 0.0;
};

// Thread 0 of each CTA evaluates the scalars; the rest read them here.
struct Scal
{
  double a, b, c;
  int status;
  int rep; // replace r by the true residual before the next iteration
};

// One BiCGStab solve by the team. r0 = rhs (x updated in place from x0 = 0
// when zero_x, else from the given x with rhs its residual). Stops when
// ||r|| < tol * norm_ref (norm_ref <= 0: ||rhs||).
//
// With snap (FP64 runs), the iterate is copied there whenever the recursive
// residual has fallen 4x below the last copy, and a run that ends above that
// point (breakdown, iteration limit) returns it; a residual that grows
// 1e16-fold over the best seen, or turns non-finite, ends the run as a
// breakdown. Each thread copies and restores the elements it also updates,
// so the copies need no barrier of their own.
//
// stall > 0 (inner solves of mixed precision): a run whose best recursive
// residual has not halved within a window of `stall` iterations (counted
// from the start or from the last halving) ends with status 4. The caller
// keeps such a run only if it halved at least once, so the iterations of a
// plateau would be spent on a result the next refinement step redoes.
//
// RR (FP64 runs): residual replacement with group update (van der Vorst and
// Ye 2000), the rule of the whole-GPU engine (DevState in solver.h): x is the
// group base, the updates accumulate in xp; when the deviation bound
//   dev += eps (cA ||xp|| + ||r||)
// crosses kReplaceThreshold * ||r||, xp is folded into x and r is replaced
// by the true residual bt - A x (bt: the system's b). Applied at once, in the
// iteration where the bound crosses.
template <typename T, int OP, bool RR = false>
__device__ SolveOut team_bicgstab (cg::cluster_group &cl, const TeamSys<T> &S, const T *rhs, T *x, bool zero_x,
                                   double tol, int max_it, double norm_ref, T *snap = nullptr, int stall = 0,
                                   const T *bt = nullptr, T *xp = nullptr, double cA = 0.0, int *reps = nullptr,
                                   bool new_shadow = false)
{
  using Op = TeamOp<T, OP>;
  const TeamIdx ix = team_index<Op::G> (cl);
  __shared__ Scal sc;
  SolveOut o;
  double rr0 = 0.0, rhr0 = 0.0;
  for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
    {
      const T ri = rhs[i];
      if (zero_x)
        x[i] = 0;
      if (RR)
        xp[i] = 0;
      // after a breakdown: a perturbed shadow residual (shadow_factor)
      const T hi = new_shadow ? (T) (ri * shadow_factor (i)) : ri;
      S.r[i] = ri;
      S.rh[i] = hi;
      S.p[i] = 0;
      S.v[i] = 0;
      rr0 = fma ((double) ri, (double) ri, rr0);
      rhr0 = fma ((double) hi, (double) ri, rhr0);
    }
  double in1[3] = { rr0, 0.0, rhr0 }, out1[3];
  if (RR && !zero_x)
    for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
      in1[1] = fma ((double) x[i], (double) x[i], in1[1]);
  team_sum<3> (cl, in1, out1);
  if (threadIdx.x == 0)
    sc.a = norm_ref > 0.0 ? norm_ref : sqrt (out1[0]);
  __syncthreads ();
  const double nb = sc.a;
  double rho = out1[2], rr = out1[0]; // rho = (rh, r0), rh = r0 unless perturbed
  double mark_rr = out1[0];           // best (r, r) at the last halving
  int mark_it = 0;
  double rho_prev = 1.0, alpha = 1.0, omega = 1.0;
  // Team-uniform (every thread holds the same rr), so no broadcast needed.
  double best_rr = rr, snap_rr = INFINITY;
  // Replacement bound: kept by thread 0 only, which takes every scalar
  // decision (nn = (x', x') of the last iteration, or the base's (g, g) at
  // the start and after a replacement, when reset says so).
  constexpr double eps = 0x1p-53;
  double dev = 0.0, dev0 = 0.0, nr_prev = 0.0, nn = out1[1];
  bool reset = true;
  for (;;)
    {
      if (rr < best_rr)
        best_rr = rr;
      if (best_rr <= 0.25 * mark_rr)
        {
          mark_rr = best_rr;
          mark_it = o.iters;
        }
      if (snap && rr < 0.25 * snap_rr)
        {
          for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
            snap[i] = RR ? x[i] + xp[i] : x[i];
          snap_rr = rr;
        }
      // convergence, limits and beta (gpu/bicgstab.cu:451, :512)
      __syncthreads ();
      if (threadIdx.x == 0)
        {
          int st = 0;
          double beta = 0.0;
          if (nb == 0.0 || sqrt (rr) < tol * nb)
            st = 1;
          else if (o.iters >= max_it)
            st = 2;
          else if (stall > 0 && o.iters - mark_it >= stall)
            st = 4;
          else if (rho == 0.0 || omega == 0.0 || !isfinite (rho) || !(rr <= 1e16 * best_rr))
            st = 3;
          else
            {
              beta = rho / rho_prev * alpha / omega;
              if (!isfinite (beta))
                st = 3;
            }
          int rep = 0;
          if (RR && st == 0)
            {
              const double nr = sqrt (rr);
              if (reset)
                dev = dev0 = eps * (cA * sqrt (nn) + nr);
              else
                {
                  const double dnew = dev + eps * (cA * sqrt (nn) + nr);
                  rep = dev <= kReplaceThreshold * nr_prev && dnew > kReplaceThreshold * nr && dnew > 1.1 * dev0;
                  dev = dnew;
                }
              nr_prev = nr;
              reset = rep;
            }
          sc.b = beta;
          sc.c = nb > 0.0 ? sqrt (rr) / nb : 0.0;
          sc.status = st;
          sc.rep = rep;
        }
      __syncthreads ();
      if (sc.status)
        {
          o.status = sc.status;
          o.rec_rel = sc.c;
          break;
        }
      if constexpr (RR)
        if (sc.rep)
          {
            // Group update, then r = b - A x: every thread folds its own
            // elements; the product reads everyone's, after the barrier.
            double gg = 0.0;
            for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
              {
                const T gi = x[i] + xp[i];
                x[i] = gi;
                xp[i] = 0;
                gg = fma ((double) gi, (double) gi, gg);
              }
            cl.sync ();
            EpiReplaceT er{ bt, S.r, S.rh };
            Op::run (S, ix, x, S.t, er);
            double d4[3] = { er.rhr, er.rr, gg }, nr4[3];
            team_sum<3> (cl, d4, nr4);
            rho = nr4[0];
            rr = nr4[1];
            nn = nr4[2];
            if (reps)
              (*reps)++;
            continue; // convergence is checked on the replaced residual
          }
      const T tb = (T) sc.b, tw = (T) omega;
      for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
        S.p[i] = S.r[i] + tb * (S.p[i] - tw * S.v[i]);
      cl.sync ();
      EpiDotT<T> e2{ S.rh };
      Op::run (S, ix, S.p, S.v, e2);
      double d1[1] = { e2.acc }, rhv[1];
      team_sum<1> (cl, d1, rhv);
      if (threadIdx.x == 0)
        {
          sc.a = rho / rhv[0];
          sc.status = (rhv[0] == 0.0 || !isfinite (sc.a)) ? 3 : 0;
        }
      __syncthreads ();
      if (sc.status)
        {
          o.status = 3;
          o.rec_rel = nb > 0.0 ? sqrt (rr) / nb : 0.0;
          break;
        }
      alpha = sc.a;
      const T ta = (T) alpha;
      for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
        S.s[i] = S.r[i] - ta * S.v[i];
      cl.sync ();
      EpiTST<T> e4{ S.s };
      Op::run (S, ix, S.s, S.t, e4);
      double d2[2] = { e4.ts, e4.tt }, tst[2];
      team_sum<2> (cl, d2, tst);
      if (threadIdx.x == 0)
        {
          const double w = tst[1] != 0.0 ? tst[0] / tst[1] : 0.0;
          sc.a = w;
          sc.status = isfinite (w) ? 0 : 3;
        }
      __syncthreads ();
      if (sc.status)
        {
          o.status = 3;
          o.rec_rel = nb > 0.0 ? sqrt (rr) / nb : 0.0;
          break;
        }
      omega = sc.a;
      const T tw2 = (T) omega;
      double rhr = 0.0, rrn = 0.0, xx = 0.0;
      T *xu = RR ? xp : x; // the vector the iteration updates
      for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
        {
          const T xn = xu[i] + ta * S.p[i] + tw2 * S.s[i];
          xu[i] = xn;
          const T ri = S.s[i] - tw2 * S.t[i];
          S.r[i] = ri;
          rhr = fma ((double) S.rh[i], (double) ri, rhr);
          rrn = fma ((double) ri, (double) ri, rrn);
          if (RR)
            xx = fma ((double) xn, (double) xn, xx);
        }
      double d3[3] = { rhr, rrn, xx }, nx[3];
      team_sum<3> (cl, d3, nx);
      rho_prev = rho;
      rho = nx[0];
      rr = nx[1];
      nn = nx[2];
      o.iters++;
    }
  if (snap && o.status != 1 && snap_rr < INFINITY && !(rr <= snap_rr))
    {
      for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
        {
          x[i] = snap[i];
          if (RR)
            xp[i] = 0;
        }
      o.rec_rel = nb > 0.0 ? sqrt (snap_rr) / nb : 0.0;
    }
  if (RR)
    for (int64_t i = ix.elem0; i < S.n; i += ix.elem_stride)
      {
        x[i] = x[i] + xp[i];
        xp[i] = 0;
      }
  cl.sync (); // x, r complete before anyone reads them
  return o;
}

// r = b - A x in FP64 over the team; returns (||r||^2, ||b||^2).
template <int OP>
__device__ void team_residual (cg::cluster_group &cl, const TeamSys<double> &S, const double *b, const double *x,
                               double *r, double &rr, double &bb)
{
  using Op = TeamOp<double, OP>;
  const TeamIdx ix = team_index<Op::G> (cl);
  EpiResid e{ b, r };
  Op::run (S, ix, x, S.t, e); // y lands in t (scratch)
  double d[2] = { e.rr, e.bb }, out[2];
  team_sum<2> (cl, d, out);
  rr = out[0];
  bb = out[1];
}

struct Fp64Result
{
  int iters = 0, status = 0, restarts = 0, replacements = 0;
  double rel = 0.0, rec = 0.0;
};

// FP64 BiCGStab with true-residual restarts: from x = 0 (first) or from the
// current x with its residual in r64. Restarts continue while each one at
// least halves the true residual (after a breakdown: lowers it at all; at
// most 8); each aims at half the one it
// starts from (a restart asked only for the tolerance again, from just above
// it, moves x by a hair and the true residual with it). Near FP64's
// attainable accuracy a restart can leave x worse, so the best iterate is
// kept (xb) and restored.
template <int OP>
__device__ Fp64Result fp64_restarted (cg::cluster_group &cl, const TeamSys<double> &S64, const BatchDesc &D,
                                      const BatchParams &P, bool first, int budget, double norm_b, double *r64,
                                      double cA)
{
  __shared__ double sh_rel, sh_nb;
  const TeamIdx ix = team_index<1> (cl);
  double *xb = D.w64 + 7 * D.n;
  double *snap = D.w64 + 8 * D.n;
  double *xp = D.w64 + 9 * D.n;
  Fp64Result f;
  double best = INFINITY;
  double target = P.tol; // a restart aims at half the true residual it starts from
  bool shadow = false;   // restart after a breakdown: perturbed shadow residual
  for (;;)
    {
      const SolveOut o = team_bicgstab<double, OP, true> (cl, S64, first ? D.b : r64, D.x, first, target,
                                                          budget - f.iters, norm_b, snap, 0, D.b, xp, cA,
                                                          &f.replacements, shadow);
      shadow = o.status == 3;
      f.iters += o.iters;
      double rr, bb;
      team_residual<OP> (cl, S64, D.b, D.x, r64, rr, bb);
      if (threadIdx.x == 0)
        {
          sh_rel = bb > 0 ? sqrt (rr / bb) : 0.0;
          sh_nb = sqrt (bb);
        }
      __syncthreads ();
      const double rel = sh_rel;
      norm_b = sh_nb;
      if (!(rel < best))
        {
          if (f.restarts > 0)
            {
              // This restart made x worse: go back to the best iterate.
              for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
                D.x[i] = xb[i];
              cl.sync ();
            }
          else
            {
              f.rel = rel;
              f.status = o.status;
              f.rec = o.rec_rel;
            }
          break;
        }
      // A restart that met its recursive tolerance but did not at least
      // halve the true residual met FP64's floor (u ||A| |x|| / ||b||):
      // keep its x, stop. Runs that broke down keep restarting while they
      // improve at all.
      const bool halved = rel <= 0.5 * best || o.status != 1;
      best = rel;
      f.rel = rel;
      f.status = o.status;
      f.rec = o.rec_rel;
      // A breakdown restarts too (fresh shadow residual); the iteration
      // limit ends the loop.
      if (rel < P.tol || o.status == 2 || f.iters >= budget || f.restarts >= 8 || (f.restarts > 0 && !halved))
        break;
      for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
        xb[i] = D.x[i];
      cl.sync ();
      first = false;
      f.restarts++;
      target = fmin (P.tol, 0.5 * rel);
    }
  return f;
}

template <int PREC, int OP>
__device__ void solve_system (cg::cluster_group &cl, const BatchDesc &D, const BatchParams &P, BatchOut &res)
{
  TeamSys<double> S64{ D.nbr, D.bs, D.n, D.rp, D.cols, D.vals64,
                       D.w64, D.w64 + D.n, D.w64 + 2 * D.n, D.w64 + 3 * D.n, D.w64 + 4 * D.n, D.w64 + 5 * D.n };
  const TeamIdx ix = team_index<1> (cl);
  __shared__ double sh_rel, sh_scale;
  int iters64 = 0, iters32 = 0, refinements = 0, fallback = 0, status = 0, restarts = 0, replacements = 0;
  double rel = 0.0, rec = 0.0;
  double *r64 = D.w64 + 6 * D.n; // FP64 residual of the refinement / restart loop
  // Replacement bound of the FP64 runs (one pass over the matrix).
  const double cA = PREC == BMFP_SOLVE_FP32 ? 0.0 : team_matrix_bound<double> (cl, S64);
  if constexpr (PREC == BMFP_SOLVE_FP32)
    {
      TeamSys<float> S32{ D.nbr, D.bs, D.n, D.rp, D.cols, D.vals32,
                          D.w32, D.w32 + D.n, D.w32 + 2 * D.n, D.w32 + 3 * D.n, D.w32 + 4 * D.n, D.w32 + 5 * D.n };
      float *x32 = D.w32 + 6 * D.n, *b32 = D.w32 + 7 * D.n;
      for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
        b32[i] = (float) D.b[i];
      cl.sync ();
      const SolveOut o = team_bicgstab<float, OP> (cl, S32, b32, x32, true, P.tol, P.max_it, -1.0);
      for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
        D.x[i] = (double) x32[i];
      cl.sync ();
      iters32 = o.iters;
      status = o.status;
      rec = o.rec_rel;
      double rr, bb;
      team_residual<OP> (cl, S64, D.b, D.x, r64, rr, bb);
      rel = bb > 0 ? sqrt (rr / bb) : 0.0;
    }
  else if constexpr (PREC == BMFP_SOLVE_FP64)
    {
      const Fp64Result f = fp64_restarted<OP> (cl, S64, D, P, true, P.max_it, -1.0, r64, cA);
      iters64 = f.iters;
      status = f.status;
      restarts = f.restarts;
      replacements = f.replacements;
      rel = f.rel;
      rec = f.rec;
    }
  else
    {
      // MIXED: FP32 inner solves, FP64 residual, update and norm; an FP64
      // finish (with restarts) when a step gains < 4x, from the current x or,
      // when the FP32 steps gained less than 100x in all, from x = 0.
      TeamSys<float> S32{ D.nbr, D.bs, D.n, D.rp, D.cols, D.vals32,
                          D.w32, D.w32 + D.n, D.w32 + 2 * D.n, D.w32 + 3 * D.n, D.w32 + 4 * D.n, D.w32 + 5 * D.n };
      float *x32 = D.w32 + 6 * D.n, *r32 = D.w32 + 7 * D.n;
      for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
        D.x[i] = 0.0;
      cl.sync ();
      double prev = INFINITY;
      for (int k = 0;; k++)
        {
          double rr, bb;
          team_residual<OP> (cl, S64, D.b, D.x, r64, rr, bb);
          if (threadIdx.x == 0)
            {
              sh_rel = bb > 0 ? sqrt (rr / bb) : 0.0;
              sh_scale = sqrt (rr);
            }
          __syncthreads ();
          rel = sh_rel;
          rec = rel;
          if (rel < P.tol)
            {
              status = 1;
              break;
            }
          const bool budget = iters32 + iters64 < P.max_it && k < P.max_ref;
          const bool stalled = k > 0 && rel > prev / 4;
          if (!budget || (stalled && P.fallback))
            {
              if (!P.fallback || iters32 + iters64 >= P.max_it)
                {
                  status = 2;
                  break;
                }
              fallback = 1;
              const double nb = rel > 0 ? sh_scale / rel : 0.0; // ||b||
              // FP32 steps that gained less than 100x leave an iterate from
              // which FP64 BiCGStab measured 1.1-1.8x the iterations it needs
              // from x = 0 (elasticity family): start over from zero then,
              // exactly as the FP64 solve does (same ||b||, same bits).
              const bool fresh = rel > 1e-2;
              const Fp64Result f
                = fp64_restarted<OP> (cl, S64, D, P, fresh, P.max_it - iters32, fresh ? -1.0 : nb, r64, cA);
              iters64 += f.iters;
              status = f.status;
              restarts = f.restarts;
              replacements = f.replacements;
              rel = f.rel;
              rec = f.rec;
              break;
            }
          prev = rel;
          const double inv = 1.0 / sh_scale;
          const double scale = sh_scale;
          for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
            r32[i] = (float) (r64[i] * inv);
          cl.sync ();
          const int cap = min (P.inner_max, P.max_it - iters32 - iters64);
          const SolveOut o = team_bicgstab<float, OP> (cl, S32, r32, x32, true, P.inner_tol, cap, -1.0,
                                                       nullptr, P.inner_stall);
          iters32 += o.iters;
          refinements = k + 1;
          if (!(o.rec_rel < 0.5))
            {
              // The inner solve did not halve its residual (stagnation,
              // breakdown or blow-up): discard it and fall back next pass.
              prev = 0.0;
              continue;
            }
          for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
            D.x[i] = D.x[i] + scale * (double) x32[i];
          cl.sync ();
        }
    }
  if (D.x_out)
    {
      for (int64_t i = ix.elem0; i < D.n; i += ix.elem_stride)
        D.x_out[i] = D.x[i];
      __threadfence_system ();
      cl.sync (); // every team thread's part of x is out before done is set
    }
  if (cl.block_rank () == 0 && threadIdx.x == 0)
    {
      // Converged means the FP64 true residual met the tolerance; a solve
      // whose recursive residual did (status 1) but whose true residual did
      // not is reported as not converged.
      res.status = rel < P.tol ? 1 : (status == 1 ? 2 : status);
      res.iterations = iters32 + iters64;
      res.iterations_fp32 = iters32;
      res.refinements = refinements;
      res.restarts = restarts;
      res.replacements = replacements;
      res.fallback = fallback;
      res.true_rel = rel;
      res.rec_rel = rec;
      __threadfence_system ();
      *reinterpret_cast<volatile int *> (&res.done) = 1;
    }
}

// Two CTAs of 512 threads per SM (64 registers a thread, some spilled): two
// teams share each SM's FP64 pipe and hide each other's latency. On the
// uneven elasticity batch (FP64, cluster 8 x 512) 0.66 s against 0.92 s at
// one CTA per SM and 128 registers, and the best configuration of either
// bound: 0.66 against 0.76 s.
template <int PREC, int OP>
__global__ void __launch_bounds__ (512, 2) batch_kernel (BatchParams P)
{
  cg::cluster_group cl = cg::this_cluster ();
  __shared__ int sh_sys;
  for (;;)
    {
      if (cl.block_rank () == 0 && threadIdx.x == 0)
        sh_sys = atomicAdd (P.counter, 1);
      cl.sync ();
      const int k = *cl.map_shared_rank (&sh_sys, 0);
      cl.sync ();
      if (k >= P.n_systems)
        break;
      const int sys = P.order[k];
      const BatchDesc D = P.desc[sys];
      solve_system<PREC, OP> (cl, D, P, P.out[sys]);
    }
}

using KernelFn = void (*) (BatchParams);

KernelFn kernel_for (int precision, int op)
{
#define BMFP_K(PR, OP)                                                                                               \
  if (precision == PR && op == OP)                                                                                   \
    return batch_kernel<PR, OP>;
  BMFP_K (BMFP_SOLVE_FP64, kOpFlat2) BMFP_K (BMFP_SOLVE_FP64, kOpCsr) BMFP_K (BMFP_SOLVE_FP64, kOpTpr)
  BMFP_K (BMFP_SOLVE_FP32, kOpFlat2) BMFP_K (BMFP_SOLVE_FP32, kOpCsr) BMFP_K (BMFP_SOLVE_FP32, kOpTpr)
  BMFP_K (BMFP_SOLVE_MIXED, kOpFlat2) BMFP_K (BMFP_SOLVE_MIXED, kOpCsr) BMFP_K (BMFP_SOLVE_MIXED, kOpTpr)
#undef BMFP_K
  return nullptr;
}
} // namespace

// ------------------------------------------------------------ raw launch
// Used by the serving loop for its micro-batches (serve.cpp).

int batch_op_for (const bmfp_matrix_s *A)
{
  if (A->bs == 2)
    return kOpFlat2;
  return (A->bs == 0 || A->bs == 1) ? kOpCsr : kOpTpr;
}

int batch_launch (int precision, int op, const BatchParams &P, int cluster, int threads, int grid, cudaStream_t s)
{
  KernelFn k = kernel_for (precision, op);
  if (!k)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "no batched kernel for precision %d / routine %d", precision, op);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3 ((unsigned) grid);
  cfg.blockDim = dim3 ((unsigned) threads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned) cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BMFP_CUDA (cudaLaunchKernelEx (&cfg, k, P));
  return BMFP_SUCCESS;
}

int batch_max_clusters (int precision, int op, int cluster, int threads, int *clusters)
{
  KernelFn k = kernel_for (precision, op);
  if (!k)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "no batched kernel for precision %d / routine %d", precision, op);
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3 ((unsigned) threads);
  cfg.gridDim = dim3 ((unsigned) cluster);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned) cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BMFP_CUDA (cudaOccupancyMaxActiveClusters (clusters, k, &cfg));
  return BMFP_SUCCESS;
}

// ------------------------------------------------------------ host side

BatchEngine::~BatchEngine ()
{
  if (graph_)
    cudaGraphExecDestroy (graph_);
  if (capture_stream_)
    cudaStreamDestroy (capture_stream_);
  cudaFree (d_desc_);
  cudaFree (d_out_);
  cudaFree (d_counter_);
  cudaFree (d_order_);
  cudaFree (w64_);
  cudaFree (w32_);
  for (void *v : vals32_)
    cudaFree (v);
  if (h_desc_)
    cudaFreeHost (h_desc_);
  if (h_out_)
    cudaFreeHost (h_out_);
}

int BatchEngine::init (int n, const bmfp_matrix_s *const *mats, const bmfp_solver_options &o, cudaStream_t s)
{
  n_ = n;
  opts_ = o;
  std::vector<int64_t> rows (n);
  int64_t total = 0;
  for (int i = 0; i < n; i++)
    {
      const bmfp_matrix_s *A = mats[i];
      if (!A || A->dtype != BMFP_R64F)
        return fail (BMFP_ERROR_INVALID_VALUE, "batch system %d: needs an FP64 matrix handle", i);
      const int bs = A->bs ? A->bs : 1;
      if (A->n_rows != A->n_cols)
        return fail (BMFP_ERROR_INVALID_VALUE, "batch system %d is not square", i);
      if (bs > 32)
        return fail (BMFP_ERROR_NOT_SUPPORTED, "batch system %d: bs %d > 32", i, bs);
      rows[i] = (int64_t) A->n_rows * bs;
      total += rows[i];
    }
  const bool lowp = o.precision != BMFP_SOLVE_FP64;
  BMFP_CUDA (cudaMalloc (&w64_, sizeof (double) * (size_t) std::max<int64_t> (kBatchW64 * total, 1)));
  if (lowp)
    BMFP_CUDA (cudaMalloc (&w32_, sizeof (float) * (size_t) std::max<int64_t> (8 * total, 1)));
  BMFP_CUDA (cudaMallocHost (&h_desc_, sizeof (BatchDesc) * (size_t) std::max (n, 1)));
  BMFP_CUDA (cudaMallocHost (&h_out_, sizeof (BatchOut) * (size_t) std::max (n, 1)));
  BMFP_CUDA (cudaMalloc (&d_desc_, sizeof (BatchDesc) * (size_t) std::max (n, 1)));
  BMFP_CUDA (cudaMalloc (&d_out_, sizeof (BatchOut) * (size_t) std::max (n, 1)));
  BMFP_CUDA (cudaMalloc (&d_counter_, sizeof (int)));
  BMFP_CUDA (cudaMalloc (&d_order_, sizeof (int) * (size_t) std::max (n, 1)));
  vals32_.assign (n, nullptr);
  int64_t off = 0;
  for (int i = 0; i < n; i++)
    {
      const bmfp_matrix_s *A = mats[i];
      // The page-locked array comes back uninitialised (or holding an
      // earlier engine's bytes): start every descriptor from its defaults,
      // so fields this engine does not use (x_out) are null.
      BatchDesc &D = h_desc_[i];
      D = BatchDesc{};
      D.nbr = A->n_rows;
      D.bs = A->bs ? A->bs : 1;
      D.n = rows[i];
      D.rp = A->d_row_ptr;
      D.cols = A->d_cols;
      D.vals64 = (const double *) A->d_vals;
      D.op = (A->bs == 2) ? kOpFlat2 : (D.bs == 1 ? kOpCsr : kOpTpr);
      if (i == 0)
        op_ = D.op;
      else if (op_ != D.op)
        op_ = kOpTpr; // mixed block sizes: the generic warp-per-block-row routine
      D.w64 = (double *) w64_ + kBatchW64 * off;
      D.w32 = lowp ? (float *) w32_ + 8 * off : nullptr;
      D.vals32 = nullptr;
      if (lowp)
        {
          const int64_t nv = A->bs ? A->nnz * A->bs * A->bs : A->nnz;
          BMFP_CUDA (cudaMalloc (&vals32_[i], sizeof (float) * (size_t) std::max<int64_t> (nv, 1)));
          int st = convert_values (BMFP_R64F, BMFP_R32F, nv, A->d_vals, vals32_[i], s);
          if (st != BMFP_SUCCESS)
            return st;
          D.vals32 = (const float *) vals32_[i];
        }
      D.b = nullptr;
      D.x = nullptr;
      off += rows[i];
    }
  // One kernel per (precision, row routine); a batch of mixed block sizes
  // uses the generic routine for every system.
  for (int i = 0; i < n; i++)
    h_desc_[i].op = op_;
  kernel_ = (void *) kernel_for (o.precision, op_);
  if (!kernel_)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "no batched kernel for this configuration");
  // Largest systems first (their solves are the longest).
  std::vector<int> order (n);
  std::iota (order.begin (), order.end (), 0);
  std::stable_sort (order.begin (), order.end (), [&] (int a, int b) { return rows[a] > rows[b]; });
  BMFP_CUDA (cudaMemcpyAsync (d_order_, order.data (), sizeof (int) * (size_t) n, cudaMemcpyHostToDevice, s));
  BMFP_CUDA (cudaStreamCreateWithFlags (&capture_stream_, cudaStreamNonBlocking));
  BMFP_CUDA (cudaStreamSynchronize (s));
  return configure (cluster_, threads_);
}

int BatchEngine::launch (cudaStream_t s, int max_it_override)
{
  BatchParams P;
  P.n_systems = n_;
  P.desc = d_desc_;
  P.out = d_out_;
  P.counter = d_counter_;
  P.order = d_order_;
  P.precision = opts_.precision;
  P.tol = opts_.tolerance;
  P.max_it = max_it_override > 0 ? max_it_override : opts_.max_iterations;
  P.inner_tol = opts_.inner_tolerance;
  P.inner_max = opts_.inner_max_iterations;
  P.inner_stall = opts_.inner_stall_iterations;
  P.max_ref = opts_.max_refinements;
  P.fallback = opts_.fallback_fp64;
  BMFP_CUDA (cudaMemsetAsync (d_counter_, 0, sizeof (int), s));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3 ((unsigned) grid_);
  cfg.blockDim = dim3 ((unsigned) threads_);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned) cluster_;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BMFP_CUDA (cudaLaunchKernelEx (&cfg, (KernelFn) kernel_, P));
  return BMFP_SUCCESS;
}

int BatchEngine::configure (int cluster, int threads)
{
  if (cluster < 1 || cluster > 8 || (cluster & (cluster - 1)) || threads < 64 || threads > kLaunchThreads
      || threads % 64)
    return fail (BMFP_ERROR_INVALID_VALUE, "invalid batch configuration (cluster %d, threads %d)", cluster, threads);
  cluster_ = cluster;
  threads_ = threads;
  // As many whole clusters as can be co-resident (the kernel is persistent).
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3 ((unsigned) threads);
  cfg.gridDim = dim3 ((unsigned) cluster);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned) cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  BMFP_CUDA (cudaOccupancyMaxActiveClusters (&clusters, (KernelFn) kernel_, &cfg));
  if (clusters < 1)
    return fail (BMFP_ERROR_NOT_SUPPORTED, "no cluster of %d x %d threads fits on this GPU", cluster, threads);
  grid_ = std::min (clusters, std::max (n_, 1)) * cluster;
  if (graph_)
    {
      cudaGraphExecDestroy (graph_);
      graph_ = nullptr;
    }
  cudaGraph_t g = nullptr;
  BMFP_CUDA (cudaStreamBeginCapture (capture_stream_, cudaStreamCaptureModeThreadLocal));
  const int st = launch (capture_stream_, 0);
  cudaError_t e = cudaStreamEndCapture (capture_stream_, &g);
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

int BatchEngine::set_vectors (const void *const *d_b, void *const *d_x, cudaStream_t s)
{
  for (int i = 0; i < n_; i++)
    {
      if (!d_b[i] || !d_x[i])
        return fail (BMFP_ERROR_INVALID_VALUE, "batch system %d: null b or x", i);
      h_desc_[i].b = (const double *) d_b[i];
      h_desc_[i].x = (double *) d_x[i];
    }
  BMFP_CUDA (cudaMemcpyAsync (d_desc_, h_desc_, sizeof (BatchDesc) * (size_t) n_, cudaMemcpyHostToDevice, s));
  return BMFP_SUCCESS;
}

int BatchEngine::solve (const void *const *d_b, void *const *d_x, bmfp_solve_info *infos, cudaStream_t s)
{
  const auto t0 = std::chrono::steady_clock::now ();
  int rc = set_vectors (d_b, d_x, s);
  if (rc != BMFP_SUCCESS)
    return rc;
  BMFP_CUDA (cudaGraphLaunch (graph_, s));
  BMFP_CUDA (cudaMemcpyAsync (h_out_, d_out_, sizeof (BatchOut) * (size_t) n_, cudaMemcpyDeviceToHost, s));
  BMFP_CUDA (cudaStreamSynchronize (s));
  const double secs = std::chrono::duration<double> (std::chrono::steady_clock::now () - t0).count ();
  int worst = BMFP_SUCCESS;
  for (int i = 0; i < n_; i++)
    {
      const BatchOut &o = h_out_[i];
      bmfp_solve_info &f = infos[i];
      f = bmfp_solve_info{};
      f.status = o.status == 1 ? BMFP_SUCCESS : (o.status == 3 ? BMFP_ERROR_BREAKDOWN : BMFP_ERROR_NOT_CONVERGED);
      f.iterations = o.iterations;
      f.iterations_fp32 = o.iterations_fp32;
      f.refinements = o.refinements;
      f.restarts = o.restarts;
      f.replacements = o.replacements;
      f.used_fp64_fallback = o.fallback;
      f.true_rel_residual = o.true_rel;
      f.recursive_rel_residual = o.rec_rel;
      f.seconds = secs;
      if (f.status != BMFP_SUCCESS && worst == BMFP_SUCCESS)
        worst = f.status;
    }
  return worst;
}

int BatchEngine::autotune (const void *const *d_b, void *const *d_x, cudaStream_t s, int probe_iterations)
{
  // Time each (cluster, threads) candidate on the real batch with every
  // system capped at probe_iterations, keep the fastest. Teams of 1 or 2
  // CTAs are never the fastest on these batches (their largest systems take
  // the longest). The cap decides what is timed: on the uneven elasticity
  // batch caps of 128-256 iterations time the small systems and pick
  // 8 x 256 (0.88 s for the full solve), caps of 512 (FP64) or 1024 (mixed)
  // and more pick 8 x 512 (0.63 s), as the full solves rank them.
  static const int clusters[] = { 4, 8 };
  static const int threads[] = { 256, 512 };
  int rc = set_vectors (d_b, d_x, s);
  if (rc != BMFP_SUCCESS)
    return rc;
  cudaEvent_t a, b;
  BMFP_CUDA (cudaEventCreate (&a));
  BMFP_CUDA (cudaEventCreate (&b));
  float best = 1e30f;
  int best_c = cluster_, best_t = threads_;
  for (int c : clusters)
    for (int t : threads)
      {
        if (configure (c, t) != BMFP_SUCCESS)
          continue;
        if (launch (s, std::min (probe_iterations, 4)) != BMFP_SUCCESS)
          continue;
        cudaEventRecord (a, s);
        int ok = launch (s, probe_iterations);
        cudaEventRecord (b, s);
        if (cudaEventSynchronize (b) != cudaSuccess || ok != BMFP_SUCCESS)
          continue;
        float ms = 0;
        cudaEventElapsedTime (&ms, a, b);
        if (ms < best)
          {
            best = ms;
            best_c = c;
            best_t = t;
          }
      }
  cudaEventDestroy (a);
  cudaEventDestroy (b);
  return configure (best_c, best_t);
}
} // namespace bmfp
