// fvc_krylov.cu -- persistent Krylov solvers and SpMV kernels (sm_103a).
//
// One cooperative (co-resident) launch runs a whole solve: the Krylov loop,
// its reductions and its stopping test stay on the device, with a bounded
// grid barrier between phases.  Each block owns a contiguous range of SELL-32
// slices; each warp lane owns one row of a slice, the same row in every
// phase, so vector updates touch only rows the thread itself produced.
//
// FP64 kernels restate src/Iterativos.f step by step:
//   pcg        Iterativos.f:29-106   (2 grid barriers per iteration: the
//              search-direction update p = z + beta*p of iteration j+1 is
//              fused into the SpMV of iteration j+1, double-buffering p)
//   pbicgstab  Iterativos.f:140-234  (3 grid reductions per iteration)
//   gmres      Iterativos.f:271-446  (restarted, k = 15, modified
//              Gram-Schmidt, Givens rotations)
// The arithmetic follows the Fortran statements term by term, with two
// GB300-motivated substitutions: products and sums are fused (FMA), and the
// Jacobi division r/m is a multiplication by 1/m computed once per matrix.
// GB300 executes FP64 at ~1/64 of its FP32 rate, and these two changes
// roughly halve the FP64 instructions per row; they move results only at
// rounding level, like the dot products, which are tree sums in a fixed
// (deterministic) order instead of the reference's sequential sums.
// BiCGSTAB adds one thing the reference lacks: where one of its
// denominators is exactly zero (the reference goes on with Inf/NaN), the
// recurrence restarts from the current residual, or the solve ends with
// FVC_ERR_BREAKDOWN when it has just restarted (bicgstab_run).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fvc_device.cuh"
#include "fvc_internal.h"

namespace fvc {

namespace {

struct KArgs {
  SellView<double> A;
  const double *m;
  const double *minv;
  const double *b;
  double *x;
  double *v0, *v1, *v2, *v3, *v4, *v5, *v6, *v7;
  double *v8, *v9;  // batched BiCGSTAB: z = p/m and z' = s'/m stored once per row
  double *g;  // GMRES basis
  GridSync gs;
  double tol;
  int maxit;
  int init;
  int stop_rule;
  double *result;  // [0] energy [1] conv [2] final_crit [3] |b-Ax|^2 [4] |b|^2
  int *iresult;    // [0] iterations [1] status [2] inner iterations
};

// Slice range of this block and the lane/warp decomposition.
struct Part {
  int lane, warp, nwarps, sb, se, n;
  __device__ Part(int nslices, int nrows) {
    lane = threadIdx.x & 31;
    warp = threadIdx.x >> 5;
    nwarps = blockDim.x >> 5;
    const int spb = (nslices + gridDim.x - 1) / gridDim.x;
    sb = blockIdx.x * spb;
    se = min(nslices, sb + spb);
    n = nrows;
  }
  // slices [s0, s1) of one system of a batch, shared by nb blocks; this
  // block is the rank-th of them
  __device__ Part(int s0, int s1, int nrows, int rank, int nb) {
    lane = threadIdx.x & 31;
    warp = threadIdx.x >> 5;
    nwarps = blockDim.x >> 5;
    const int spb = (s1 - s0 + nb - 1) / nb;
    sb = s0 + rank * spb;
    se = min(s1, sb + spb);
    n = nrows;
  }
};

#define FOR_ROWS(P)                                          \
  for (int s_ = (P).sb + (P).warp; s_ < (P).se; s_ += (P).nwarps) \
    for (int row = s_ * 32 + (P).lane, once_ = 1; once_ && row < (P).n; once_ = 0)

template <int NV>
__device__ __forceinline__ bool reduce(const KArgs &a, unsigned int &ep, double (&v)[NV],
                                       double *red) {
  return grid_allreduce<NV>(a.gs, ep, v, red);
}

__device__ __forceinline__ void finish_to(double *result, int *iresult, bool lead, int iters,
                                          int status, double conv, double crit, int inner) {
  if (lead && threadIdx.x == 0) {
    iresult[0] = iters;
    iresult[1] = status;
    iresult[2] = inner;
    result[1] = conv;
    result[2] = crit;
  }
}

__device__ __forceinline__ void finish(const KArgs &a, int iters, int status,
                                       double conv, double crit, int inner) {
  finish_to(a.result, a.iresult, blockIdx.x == 0, iters, status, conv, crit, inner);
}

// Energy norm x.Ax and the FP64 residual ||b-Ax||^2, ||b||^2 in one pass
// over the rows of P (x must be complete at every row: called right after
// a synchronisation of gs); the lead block writes result[0, 3, 4].
template <bool kT = false>
__device__ __forceinline__ bool epilogue_to(const KArgs &a, const Part &P, const GridSync &gs,
                                            double *result, bool lead, unsigned int &ep,
                                            double *red, bool energy_xb) {
  double acc[3] = {0.0, 0.0, 0.0};
  const double *x = a.x;
  FOR_ROWS(P) {
    double ax = row_fma<kT>(a.A, s_, P.lane, row, [&](int k) { return x[k]; });
    double xi = x[row], bi = a.b[row];
    double rr = bi - ax;
    acc[0] = fma(xi, energy_xb ? bi : ax, acc[0]);
    acc[1] = fma(rr, rr, acc[1]);
    acc[2] = fma(bi, bi, acc[2]);
  }
  if (!grid_allreduce<3>(gs, ep, acc, red)) return false;
  if (lead && threadIdx.x == 0) {
    result[0] = acc[0];
    result[3] = acc[1];
    result[4] = acc[2];
  }
  return true;
}

__device__ __forceinline__ bool epilogue(const KArgs &a, unsigned int &ep, double *red,
                                         bool energy_xb) {
  return epilogue_to(a, Part(a.A.nslices, a.A.n), a.gs, a.result, blockIdx.x == 0, ep, red,
                     energy_xb);
}

// ---------------------------------------------------------------------
// PCG (Iterativos.f:29-106).  v0 = r, v1 = z, v2/v3 = p (double buffer),
// v4 = q (the reference's z = A p).
// ---------------------------------------------------------------------
// The iteration over the rows of P, synchronising through gs; the lead
// block writes result / iresult.  pcg_f64 runs it over the whole matrix,
// krylov_batched over one system of a batch per group of blocks.
// kStoreP: p = z + beta p is formed once per row in place and published by a
// grid barrier before the SpMV (one FP64 FMA per row instead of one per
// gathered neighbour -- 4 of the 16 FP64 instructions of a row-iteration on
// quadrilaterals); otherwise it is formed at every read from the previous p
// and z, which saves the barrier.  Both give the same bits.
// kMaxT: the most threads per block the kernel is launched with (the
// reductions' staging buffer holds that many values per reduced quantity).
template <bool kStoreP, int kMaxT = 1024>
__device__ __forceinline__ void pcg_run(const KArgs &a, const Part &P, const GridSync &gs,
                                        double *result, int *iresult, bool lead) {
  __shared__ double red[kMaxNV * 32];
  __shared__ double buf[2 * kMaxT];
  // scalars of the recurrence, updated by lane 0 of warp 0 inside the
  // all-reduces and read by every thread after them
  __shared__ struct {
    double d, alpha, beta, conv, crit;
    int stop;  // 0 go on, 1 converged, 2 NaN/Inf
  } sh;
  double *r = a.v0, *z = a.v1, *q = a.v4, *x = a.x;
  const double *minv = a.minv, *b = a.b;
  const bool rule0 = a.stop_rule == 0;
  unsigned int ep = 0;

  // r = b - A x ; z = r/m ; p = z ; d = r.z  (x = 0 when init)
  double acc[2] = {0.0, 0.0};
  FOR_ROWS(P) {
    double ax;
    if (a.init) {
      ax = 0.0;
      x[row] = 0.0;
    } else {
      ax = sell_row_fma(a.A, s_, P.lane, row, [&](int k) { return x[k]; });
    }
    const double ri = b[row] - ax;
    const double zi = ri * minv[row];
    r[row] = ri;
    a.v2[row] = zi;
    acc[0] = fma(ri, zi, acc[0]);
    acc[1] = fma(b[row], b[row], acc[1]);
  }
  if (!grid_allreduce_d<2>(gs, ep, acc, buf, [&](const double *t) {
        sh.d = t[0];
        sh.conv = rule0 ? a.tol * sqrt(fabs(t[0])) : a.tol * sqrt(t[1]);
        sh.beta = 0.0;
        sh.crit = 0.0;
        sh.stop = 0;
      }))
    return;

  double *pprev = a.v2, *pcur = a.v2;
  double beta = 0.0;
  int j, status = FVC_OK;
  for (j = 1; j <= a.maxit; ++j) {
    // q = A p  (p = z + beta*p formed on the fly for j >= 2); p.q
    double pq[1] = {0.0};
    if (kStoreP && j > 1) {
      FOR_ROWS(P) pcur[row] = fma(beta, pcur[row], z[row]);
      if (!grid_barrier(gs, ep)) return;
    }
    if (j == 1 || kStoreP) {
      FOR_ROWS(P) {
        const double *pc = pcur;
        const double qi = sell_row_fma(a.A, s_, P.lane, row, [&](int k) { return pc[k]; });
        q[row] = qi;
        pq[0] = fma(pc[row], qi, pq[0]);
      }
    } else {
      FOR_ROWS(P) {
        const double *pp = pprev;
        auto pf = [&](int k) { return fma(beta, pp[k], z[k]); };
        const double pi = pf(row);
        pcur[row] = pi;
        const double qi = sell_row_fma(a.A, s_, P.lane, row, pf);
        q[row] = qi;
        pq[0] = fma(pi, qi, pq[0]);
      }
    }
    if (!grid_allreduce_d<1>(gs, ep, pq, buf,
                             [&](const double *t) { sh.alpha = sh.d / t[0]; }))
      return;
    const double alpha = sh.alpha;
    // x += alpha p ; r -= alpha q ; z = r/m ; r.z (and r.r for stop_rule 1)
    double rz[1] = {0.0}, rr2[2] = {0.0, 0.0};
    FOR_ROWS(P) {
      x[row] = fma(alpha, pcur[row], x[row]);
      const double ri = fma(-alpha, q[row], r[row]);
      const double zi = ri * minv[row];
      r[row] = ri;
      z[row] = zi;
      if (rule0) {
        rz[0] = fma(ri, zi, rz[0]);
      } else {
        rr2[0] = fma(ri, zi, rr2[0]);
        rr2[1] = fma(ri, ri, rr2[1]);
      }
    }
    // beta = r.z / d ; d = beta d ; the reference's stopping test
    auto step = [&](const double *t) {
      sh.beta = t[0] / sh.d;
      sh.d = sh.beta * sh.d;
      sh.crit = rule0 ? sqrt(fabs(sh.d)) : sqrt(t[1]);
      sh.stop = (!(sh.crit == sh.crit) || isinf(sh.d)) ? 2 : (sh.crit < sh.conv ? 1 : 0);
    };
    const bool ok = rule0 ? grid_allreduce_d<1>(gs, ep, rz, buf, step)
                          : grid_allreduce_d<2>(gs, ep, rr2, buf, step);
    if (!ok) return;
    if (sh.stop == 2) {
      status = FVC_ERR_NAN;
      break;
    }
    if (sh.stop == 1) break;
    beta = sh.beta;
    if (!kStoreP) {
      pprev = pcur;
      pcur = (pcur == a.v2) ? a.v3 : a.v2;
    }
  }
  if (j > a.maxit) {
    j = a.maxit;
    status = FVC_ERR_NOCONV;
  }
  finish_to(result, iresult, lead, j, status, sh.conv, sh.crit, 0);
  epilogue_to(a, P, gs, result, lead, ep, red, false);
}

constexpr int kStorePRows = 262144;

template <bool kStoreP>
__global__ void __launch_bounds__(1024, 1) pcg_f64(KArgs a) {
  pcg_run<kStoreP>(a, Part(a.A.nslices, a.A.n), a.gs, a.result, a.iresult, blockIdx.x == 0);
}


// ---------------------------------------------------------------------


// ---------------------------------------------------------------------
// BiCGSTAB (Iterativos.f:140-234) in three grid synchronisations per
// iteration instead of five: the preconditioned vectors the two SpMVs
// gather (z = p/m and z = s/m) are formed on the fly from vectors the
// previous all-reduce finalised, as each neighbour is read, so no barrier
// publishes them.  Forming them needs the previous p, v and s while the
// new ones are written, so p, v and s are double-buffered.  The per-row
// arithmetic and its order are those of the reference recurrence:
//   phase 1  p = s + beta (p - w v) ; v = A (p/m) ; s.r ; v.r   -> alpha
//   phase 2  s' = s - alpha v ; t = A (s'/m) ; t.s' ; t.t       -> w
//   phase 3  x += alpha p/m ; x += w s'/m ; s'' = s' - w t ;
//            s''.(s'/m) ; r.s'' ; s''.s''                       -> beta, stop
// v0 = r (shadow r0), v1/v2 = s, v3/v4 = p, v5/v6 = v, v7 = t.
// ---------------------------------------------------------------------
// kT: solve A^T x = b through the transposed row sums (sell_row_fma_t).
// kStoreZ (batched solves, bound by GB300's FP64 rate rather than by their
// barriers): p and s' are formed once per row with z = p/m and z' = s'/m
// (a.v8, a.v9) and published by a barrier before the SpMV that gathers
// them -- five synchronisations per iteration instead of three, about half
// the FP64 instructions (a gathered neighbour costs one FMA instead of
// three or two), the same bits.
template <int kMaxT = 1024, bool kT = false, bool kStoreZ = false>
__device__ __forceinline__ void bicgstab_run(const KArgs &a, const Part &P, const GridSync &gs,
                                             double *result, int *iresult, bool lead) {
  __shared__ double red[kMaxNV * 32];
  __shared__ double buf[3 * kMaxT];
  __shared__ struct {
    double d, conv, rr0, alpha, w, beta, crit;
    int stop;     // 0 go on, 1 converged, 2 NaN/Inf, 3 breakdown
    int restart;  // a breakdown: the next iteration restarts from s
    int fresh;    // this iteration started from r0 = s (the start or a restart)
    int brk;      // r.v = 0 or r.s = 0 in phase 1 (alpha = 0 this iteration)
  } sh;
  double *r = a.v0, *t = a.v7, *x = a.x;
  double *scur = a.v1, *snxt = a.v2, *pold = a.v3, *pnew = a.v4, *vold = a.v5, *vnew = a.v6;
  const double *minv = a.minv, *b = a.b;
  const bool rule0 = a.stop_rule == 0;
  unsigned int ep = 0;

  // r = b - A x ; p = s = r ; d = r.(r/m)   (x = 0 when init)
  double acc[2] = {0.0, 0.0}, acc3[3];
  FOR_ROWS(P) {
    double ax;
    if (a.init) {
      ax = 0.0;
      x[row] = 0.0;
    } else {
      ax = row_fma<kT>(a.A, s_, P.lane, row, [&](int k) { return x[k]; });
    }
    const double ri = b[row] - ax;
    r[row] = ri;
    pnew[row] = ri;
    scur[row] = ri;
    acc[0] = fma(ri, ri * minv[row], acc[0]);
    acc[1] = fma(b[row], b[row], acc[1]);
  }
  if (!grid_allreduce_d<2>(gs, ep, acc, buf, [&](const double *q) {
        sh.d = q[0];
        sh.conv = rule0 ? a.tol * sqrt(fabs(q[0])) : a.tol * sqrt(q[1]);
        sh.crit = 0.0;
        sh.stop = 0;
        sh.restart = 0;
        sh.fresh = 1;
      }))
    return;
  int j, status = FVC_OK;
  double alpha = 0.0, w = 0.0, beta = 0.0;
  bool restart = false;
  for (j = 1; j <= a.maxit; ++j) {
    // phase 1: v = A z with z = p/m, p formed from the previous p, v, s
    acc[0] = 0.0;
    acc[1] = 0.0;
    if (kStoreZ) {
      double *zp = a.v8;
      FOR_ROWS(P) {
        if (restart) r[row] = scur[row];
        const double pi =
            (j == 1) ? pnew[row] : fma(beta, fma(-w, vold[row], pold[row]), scur[row]);
        pnew[row] = pi;
        zp[row] = pi * minv[row];
      }
      if (!grid_barrier(gs, ep)) return;
      FOR_ROWS(P) {
        const double vi = row_fma<kT>(a.A, s_, P.lane, row, [&](int k) { return zp[k]; });
        vnew[row] = vi;
        const double ri = r[row];
        acc[0] = fma(scur[row], ri, acc[0]);
        acc[1] = fma(vi, ri, acc[1]);
      }
    } else if (j == 1) {
      FOR_ROWS(P) {
        const double *pc = pnew;
        const double vi =
            row_fma<kT>(a.A, s_, P.lane, row, [&](int k) { return pc[k] * minv[k]; });
        vnew[row] = vi;
        const double ri = r[row];
        acc[0] = fma(scur[row], ri, acc[0]);
        acc[1] = fma(vi, ri, acc[1]);
      }
    } else {
      FOR_ROWS(P) {
        const double *po = pold, *vo = vold, *sc = scur;
        // after a breakdown beta = 0 (p = s) and the shadow residual is s:
        // each row rewrites its own r before it reads it
        if (restart) r[row] = sc[row];
        auto pf = [&](int k) { return fma(beta, fma(-w, vo[k], po[k]), sc[k]); };
        pnew[row] = pf(row);
        const double vi =
            row_fma<kT>(a.A, s_, P.lane, row, [&](int k) { return pf(k) * minv[k]; });
        vnew[row] = vi;
        const double ri = r[row];
        acc[0] = fma(sc[row], ri, acc[0]);
        acc[1] = fma(vi, ri, acc[1]);
      }
    }
    // r.v = 0 (the reference's alpha = r.s/0) or r.s = 0 (alpha = 0, no
    // progress): alpha = 0, the iteration takes only its w step, and the
    // next one restarts
    if (!grid_allreduce_d<2>(gs, ep, acc, buf, [&](const double *q) {
          sh.rr0 = q[0];
          sh.brk = (q[0] == 0.0 || q[1] == 0.0) ? 1 : 0;
          sh.alpha = sh.brk ? 0.0 : q[0] / q[1];
        }))
      return;
    alpha = sh.alpha;
    // phase 2: s' = s - alpha v ; t = A z with z = s'/m
    acc[0] = 0.0;
    acc[1] = 0.0;
    if (kStoreZ) {
      double *zs = a.v9;
      FOR_ROWS(P) {
        const double s1 = fma(-alpha, vnew[row], scur[row]);
        snxt[row] = s1;
        zs[row] = s1 * minv[row];
      }
      if (!grid_barrier(gs, ep)) return;
      FOR_ROWS(P) {
        const double ti = row_fma<kT>(a.A, s_, P.lane, row, [&](int k) { return zs[k]; });
        t[row] = ti;
        acc[0] = fma(ti, snxt[row], acc[0]);
        acc[1] = fma(ti, ti, acc[1]);
      }
    } else {
      FOR_ROWS(P) {
        const double *sc = scur, *vn = vnew;
        auto sf = [&](int k) { return fma(-alpha, vn[k], sc[k]); };
        snxt[row] = sf(row);
        const double ti =
            row_fma<kT>(a.A, s_, P.lane, row, [&](int k) { return sf(k) * minv[k]; });
        t[row] = ti;
        acc[0] = fma(ti, snxt[row], acc[0]);
        acc[1] = fma(ti, ti, acc[1]);
      }
    }
    // t = 0 exactly: s' = 0, the alpha step solved the system (the
    // reference's 0/0 there gives NaN); w = 0 keeps x and s' as they are
    if (!grid_allreduce_d<2>(gs, ep, acc, buf,
                             [&](const double *q) { sh.w = (q[1] != 0.0) ? q[0] / q[1] : 0.0; }))
      return;
    w = sh.w;
    // phase 3: x += alpha z ; x += w z' ; s'' = s' - w t ; s''.z' ; r.s'' ; s''.s''
    acc3[0] = 0.0;
    acc3[1] = 0.0;
    acc3[2] = 0.0;
    FOR_ROWS(P) {
      const double mi = minv[row];
      const double s1 = snxt[row];
      const double z1 = kStoreZ ? a.v9[row] : s1 * mi;
      double xi = fma(alpha, kStoreZ ? a.v8[row] : pnew[row] * mi, x[row]);
      x[row] = fma(w, z1, xi);
      const double si = fma(-w, t[row], s1);
      snxt[row] = si;
      acc3[0] = fma(si, z1, acc3[0]);
      acc3[1] = fma(r[row], si, acc3[1]);
      acc3[2] = fma(si, si, acc3[2]);
    }
    if (!grid_allreduce_d<3>(gs, ep, acc3, buf, [&](const double *q) {
          const double b0 = q[0] / sh.d;
          sh.crit = rule0 ? sqrt(fabs(b0)) : sqrt(q[2]);
          sh.stop = (!(sh.crit == sh.crit) || !(sh.w == sh.w)) ? 2 : (sh.crit < sh.conv ? 1 : 0);
          sh.beta = (q[1] / sh.rr0) * (sh.alpha / sh.w);
          // breakdown guard (where the reference's recurrence divides by
          // zero and goes on with Inf/NaN): w = 0, r.s'' = 0 or a beta that
          // is not finite restart the iteration from the current residual
          // (shadow residual and p := s''); a breakdown in an iteration that
          // itself started from its residual ends the solve (FVC_ERR_BREAKDOWN).
          // Iterations without a breakdown are unchanged.
          const bool broke = sh.stop == 0 &&
                             (sh.brk || sh.w == 0.0 || q[1] == 0.0 || !isfinite(sh.beta));
          sh.restart = 0;
          if (broke && sh.fresh) {
            sh.stop = 3;
          } else if (broke) {
            sh.restart = 1;
            sh.beta = 0.0;
          }
          sh.fresh = sh.restart;
        }))
      return;
    if (sh.stop >= 2) {
      status = (sh.stop == 2) ? FVC_ERR_NAN : FVC_ERR_BREAKDOWN;
      break;
    }
    if (sh.stop == 1) break;
    beta = sh.beta;
    restart = sh.restart != 0;
    double *tmp = scur;
    scur = snxt;
    snxt = tmp;
    tmp = pold;
    pold = pnew;
    pnew = tmp;
    tmp = vold;
    vold = vnew;
    vnew = tmp;
  }
  if (j > a.maxit) {
    j = a.maxit;
    status = FVC_ERR_NOCONV;
  }
  finish_to(result, iresult, lead, j, status, sh.conv, sh.crit, 0);
  epilogue_to<kT>(a, P, gs, result, lead, ep, red, false);
}

__global__ void __launch_bounds__(1024, 1) bicgstab_f64(KArgs a) {
  bicgstab_run(a, Part(a.A.nslices, a.A.n), a.gs, a.result, a.iresult, blockIdx.x == 0);
}

// A small system's BiCGSTAB on one thread-block cluster: the same body, its
// reductions and barriers through the cluster (GridSync.cluster), its
// vectors in global memory (L2-resident at these sizes)
__global__ void __launch_bounds__(256) bicgstab_cl(KArgs a) {
  bicgstab_run<256>(a, Part(a.A.nslices, a.A.n), a.gs, a.result, a.iresult, blockIdx.x == 0);
  cluster_close(a.gs);
}

// The same with z = p/m and z' = s'/m stored once per row (kStoreZ): for
// systems large enough that the FP64 rate, not the barriers, bounds the
// iteration
__global__ void __launch_bounds__(1024, 1) bicgstab_f64_z(KArgs a) {
  bicgstab_run<1024, false, true>(a, Part(a.A.nslices, a.A.n), a.gs, a.result, a.iresult,
                                  blockIdx.x == 0);
}

// BiCGSTAB on A^T x = b over A's storage (a.A.mirror set)
__global__ void __launch_bounds__(1024, 1) bicgstab_f64_t(KArgs a) {
  bicgstab_run<1024, true>(a, Part(a.A.nslices, a.A.n), a.gs, a.result, a.iresult,
                           blockIdx.x == 0);
}

// Batched PCG / BiCGSTAB: the matrix is block diagonal, each system
// starting at a slice boundary; every block belongs to one system
// (sys_of_block) and synchronises only with that system's blocks, so each
// system iterates with its own solver and stops on its own inside one
// cooperative launch.  PCG stores p (most groups are one block, where
// publishing p is a __syncthreads).  With d.gs.cluster each system's blocks
// are one thread-block cluster (an ordinary launch of many clusters: no
// co-residency needed, the hardware starts clusters as SMs free up).
template <int kMaxT>
__global__ void __launch_bounds__(kMaxT, 1024 / kMaxT) krylov_batched(KArgs a, const BatchSys *__restrict__ sys,
                                                        const int *__restrict__ sys_of_block) {
  const BatchSys d = sys[sys_of_block[blockIdx.x]];
  const int rank = (int)(blockIdx.x - d.gs.base);
  if (batch_masked(d, rank == 0)) return;
  const Part P(d.s0, d.s1, a.A.n, rank, (int)d.gs.nblocks);
  KArgs ak = a;
  ak.tol = d.tol;
  ak.init = d.init;
  if (d.code == 2)
    bicgstab_run<kMaxT, false, true>(ak, P, d.gs, d.result, d.iresult, rank == 0);
  else
    pcg_run<true, kMaxT>(ak, P, d.gs, d.result, d.iresult, rank == 0);
  cluster_close(d.gs);
}

// ---------------------------------------------------------------------
// GMRES(k) (Iterativos.f:271-446).  g holds k+1 basis vectors of length n;
// the small Hessenberg problem is solved redundantly by every block from
// the same totals (identical bits, no broadcast).
// ---------------------------------------------------------------------
constexpr int kGmresK = 15;

__global__ void __launch_bounds__(1024, 1) gmres_f64(KArgs a) {
  __shared__ double red[kMaxNV * 32];
  __shared__ double h[(kGmresK + 1) * kGmresK];
  __shared__ double cc[kGmresK], ss[kGmresK], e[kGmresK + 1], y[kGmresK];
  const Part P(a.A.nslices, a.A.n);
  const int n = a.A.n;
  const int k = kGmresK;
  double *x = a.x;
  const double *minv = a.minv, *b = a.b;
  auto G = [&](int i) { return a.g + (size_t)(i - 1) * n; };  // 1-based column
  auto H = [&](int i, int jj) -> double & { return h[(i - 1) + (jj - 1) * (k + 1)]; };
  unsigned int ep = 0;
  double acc[1];

  // x = 0 ; econv = tol*||b||
  acc[0] = 0.0;
  FOR_ROWS(P) {
    x[row] = 0.0;
    acc[0] = fma(b[row], b[row], acc[0]);
  }
  if (!reduce<1>(a, ep, acc, red)) return;
  const double econv = a.tol * sqrt(acc[0]);
  int l, nit = 0, ni = 0, status = FVC_OK;
  double crit = 0.0;
  for (l = 1; l <= a.maxit; ++l) {
    // g1 = (b - A x)/m ; e1 = ||g1||
    acc[0] = 0.0;
    double *g1 = G(1);
    FOR_ROWS(P) {
      const double ax = sell_row_fma(a.A, s_, P.lane, row, [&](int kk) { return x[kk]; });
      const double gi = (b[row] - ax) * minv[row];
      g1[row] = gi;
      acc[0] = fma(gi, gi, acc[0]);
    }
    if (!reduce<1>(a, ep, acc, red)) return;
    if (threadIdx.x == 0) e[0] = sqrt(acc[0]);
    __syncthreads();
    const double e1inv = 1.0 / e[0];
    FOR_ROWS(P) { g1[row] = g1[row] * e1inv; }
    if (!grid_barrier(a.gs, ep)) return;
    ni = 0;
    for (int i = 1; i <= k; ++i) {
      ++nit;
      ++ni;
      double *gi = G(i), *gn = G(i + 1);
      // g(i+1) = A g(i) / m ; first MGS dot with g(1)
      acc[0] = 0.0;
      const double *g1c = G(1);
      FOR_ROWS(P) {
        const double av = sell_row_fma(a.A, s_, P.lane, row, [&](int kk) { return gi[kk]; });
        const double vi = av * minv[row];
        gn[row] = vi;
        acc[0] = fma(vi, g1c[row], acc[0]);
      }
      if (!reduce<1>(a, ep, acc, red)) return;
      double beta = acc[0];
      if (threadIdx.x == 0) H(1, i) = beta;
      // modified Gram-Schmidt: subtract, then dot with the next vector
      for (int jj = 1; jj <= i; ++jj) {
        const double *gj = G(jj);
        const double *gnext = G(jj + 1);
        acc[0] = 0.0;
        FOR_ROWS(P) {
          const double vi = fma(-beta, gj[row], gn[row]);
          gn[row] = vi;
          acc[0] = fma(vi, (jj < i) ? gnext[row] : vi, acc[0]);
        }
        if (!reduce<1>(a, ep, acc, red)) return;
        beta = acc[0];
        if (jj < i && threadIdx.x == 0) H(jj + 1, i) = beta;
      }
      const double norm = sqrt(beta);
      const double ninv = 1.0 / norm;
      FOR_ROWS(P) { gn[row] = gn[row] * ninv; }
      if (threadIdx.x == 0) {
        H(i + 1, i) = norm;
        for (int jj = 1; jj <= i - 1; ++jj) {
          const double aux1 = cc[jj - 1] * H(jj, i) + ss[jj - 1] * H(jj + 1, i);
          const double aux2 = -ss[jj - 1] * H(jj, i) + cc[jj - 1] * H(jj + 1, i);
          H(jj, i) = aux1;
          H(jj + 1, i) = aux2;
        }
        const double rr = sqrt(H(i, i) * H(i, i) + H(i + 1, i) * H(i + 1, i));
        cc[i - 1] = H(i, i) / rr;
        ss[i - 1] = H(i + 1, i) / rr;
        H(i, i) = rr;
        H(i + 1, i) = 0.0;
        e[i] = -ss[i - 1] * e[i - 1];
        e[i - 1] = cc[i - 1] * e[i - 1];
      }
      if (!grid_barrier(a.gs, ep)) return;  // also publishes g(i+1) and h
      if (!(e[i] == e[i])) {
        status = FVC_ERR_NAN;
        break;
      }
      if (fabs(e[i]) <= econv) break;
    }
    if (status != FVC_OK) break;
    // back substitution h y = e
    if (threadIdx.x == 0) {
      y[ni - 1] = e[ni - 1] / H(ni, ni);
      for (int i = ni - 1; i >= 1; --i) {
        double yi = 0.0;
        for (int jj = i + 1; jj <= ni; ++jj) yi = yi - H(i, jj) * y[jj - 1];
        y[i - 1] = (yi + e[i - 1]) / H(i, i);
      }
    }
    __syncthreads();
    FOR_ROWS(P) {
      double xi = x[row];
      for (int jj = 1; jj <= ni; ++jj) xi = fma(y[jj - 1], G(jj)[row], xi);
      x[row] = xi;
    }
    if (!grid_barrier(a.gs, ep)) return;
    crit = fabs(e[ni]);
    if (crit <= econv) break;
  }
  if (l > a.maxit) {
    l = a.maxit;
    if (status == FVC_OK) status = FVC_ERR_NOCONV;
  }
  finish(a, l, status, econv, crit, nit);
  epilogue(a, ep, red, true);
}

// ---------------------------------------------------------------------
// Plain SpMV kernels (one warp per slice, grid-stride over slices)
// ---------------------------------------------------------------------
template <bool kFused>
__global__ void __launch_bounds__(256) spmv_f64(SellView<double> A, const double *__restrict__ x,
                                                double *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < A.nslices; s += nw) {
    const int row = s * 32 + lane;
    if (row >= A.n) continue;
    auto xf = [&](int k) { return __ldg(x + k); };
    y[row] = kFused ? sell_row_fma(A, s, lane, row, xf) : sell_row_f64(A, s, lane, row, xf);
  }
}

// y = A x in the FP32 difference form, y_i = e_i x_i + sum_k w_ik (x_i - x_k).
// kW = 4: the weights and 16-bit column offsets laid out 4 slots per slice
// row-major (one 16-byte and one 8-byte load per row); kW = 3: 3 slots per
// slice column-major (three coalesced 4-byte and three 2-byte loads, all
// issued before the gathers); kW = 0: SELL-32 with the FP64 matrix's
// columns.  Padding slots have weight 0 and add exactly 0.
template <int kW>
__global__ void __launch_bounds__(256) spmv_f32(int n, int nslices, const int64_t *__restrict__ sptr,
                                                const int *__restrict__ col,
                                                const int16_t *__restrict__ col16,
                                                const float *__restrict__ w32,
                                                const float *__restrict__ e32,
                                                const float *__restrict__ x, float *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += nw) {
    const int row = s * 32 + lane;
    if (row >= n) continue;
    const float xi = __ldg(x + row);
    float t = ld_stream(e32 + row) * xi;
    if (kW == 4) {
      const int64_t base = (int64_t)s * 128 + 4 * lane;
      const float4 w = ld_stream4(w32 + base);
      const uint2 c = ld_stream_u2(col16 + base);
      int k4[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        k4[k] = row + off16(c, k);
        FVC_CHK((unsigned)k4[k] < (unsigned)n, (int *)nullptr, kChkOffset, k4[k] = row);
      }
      t = fmaf(w.x, xi - __ldg(x + k4[0]), t);
      t = fmaf(w.y, xi - __ldg(x + k4[1]), t);
      t = fmaf(w.z, xi - __ldg(x + k4[2]), t);
      t = fmaf(w.w, xi - __ldg(x + k4[3]), t);
    } else if (kW == 3) {
      const int64_t base = (int64_t)s * 96 + lane;
      float w[3];
      int c[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        w[k] = ld_stream(w32 + base + 32 * k);
        c[k] = row + (int)ld_stream16(col16 + base + 32 * k);
        FVC_CHK((unsigned)c[k] < (unsigned)n, (int *)nullptr, kChkOffset, c[k] = row);
      }
      float xv[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) xv[k] = __ldg(x + c[k]);
#pragma unroll
      for (int k = 0; k < 3; ++k) t = fmaf(w[k], xi - xv[k], t);
    } else {
      const int64_t base = sptr[s];
      const int w = (int)((sptr[s + 1] - base) >> 5);
      for (int kk = 0; kk < w; ++kk) {
        int c = ld_stream(col + base + 32 * kk + lane);
        FVC_CHK((unsigned)c < (unsigned)n, (int *)nullptr, kChkColumn, c = row);
        t = fmaf(ld_stream(w32 + base + 32 * kk + lane), xi - __ldg(x + c), t);
      }
    }
    y[row] = t;
  }
}

__global__ void reciprocal_kernel(int n, const double *__restrict__ m, double *__restrict__ minv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) minv[i] = 1.0 / m[i];
}

SellView<double> view64(const DeviceMatrix &A) {
  SellView<double> v;
  v.n = A.n;
  v.nslices = A.nslices;
  v.sptr = A.sptr;
  v.col = A.col;
  v.val = A.val;
  v.diag = A.diag;
  v.diag_mode = A.diag_mode;
  v.mirror = A.mirror;
  return v;
}

int sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

// Co-resident grid for a persistent kernel: at most occupancy x SMs blocks,
// and no more blocks than there are slices to hand one per warp.
template <typename K>
Launch persistent_launch(K kernel, const DeviceMatrix &A, const fvc_opts &o) {
  Launch L;
  // 128..1024 threads in multiples of 128 (the block reductions assume it)
  L.threads = block_threads_for(o.block_threads, A.nslices, sm_count());
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, L.threads, 0);
  if (occ <= 0) occ = 1;
  if (o.blocks_per_sm > 0 && o.blocks_per_sm < occ) occ = o.blocks_per_sm;
  const int warps = L.threads / 32;
  const int need = (A.nslices + warps - 1) / warps;
  L.blocks = std::max(1, std::min(occ * sm_count(), need));
  if (o.max_blocks > 0) L.blocks = std::min(L.blocks, o.max_blocks);
  return L;
}

int32_t ensure_vectors(Scratch &S, size_t n, int nvec, size_t nblocks, bool gmres) {
  if (S.n < n) {
    for (int i = 0; i < Scratch::kVec; ++i) {
      if (S.v[i]) cudaFree(S.v[i]);
      S.v[i] = nullptr;
    }
    S.n = n;
  }
  for (int i = 0; i < nvec; ++i)
    if (!S.v[i] && cudaMalloc(&S.v[i], sizeof(double) * (n + 32)) != cudaSuccess) return FVC_ERR_CUDA;
  if (gmres && S.ngmres < n) {
    if (S.g) cudaFree(S.g);
    S.g = nullptr;
    if (cudaMalloc(&S.g, sizeof(double) * (size_t)(kGmresK + 1) * n) != cudaSuccess) return FVC_ERR_CUDA;
    S.ngmres = n;
  }
  return ensure_sync(S, nblocks);
}

// Enqueues one persistent solve on `stream` and returns without waiting:
// the scratch exists afterwards, so a second call of the same shape makes
// no allocation and may run inside a stream capture.  launch = false stops
// after the allocations.
template <typename K>
int32_t enqueue_persistent(K kernel, const DeviceMatrix &A, Scratch &S, const double *b,
                           double *x, double tol, int maxit, int init, const fvc_opts &o,
                           cudaStream_t stream, int nvec, bool gmres, bool launch = true) {
  if (A.n <= 0) return FVC_ERR_ARG;
  Launch L = persistent_launch(kernel, A, o);
  int32_t rc = ensure_vectors(S, (size_t)A.n, nvec, (size_t)L.blocks, gmres);
  if (rc != FVC_OK || !launch) return rc;
  reset_sync(S, stream);
  KArgs a{};
  a.A = view64(A);
  a.A.chk = check_word(S);
  a.m = A.jac;
  a.minv = A.jinv;
  a.b = b;
  a.x = x;
  a.v0 = S.v[0];
  a.v1 = S.v[1];
  a.v2 = S.v[2];
  a.v3 = S.v[3];
  a.v4 = S.v[4];
  a.v5 = S.v[5];
  a.v6 = S.v[6];
  a.v7 = S.v[7];
  a.v8 = S.v[8];
  a.v9 = S.v[9];
  a.g = S.g;
  a.gs = make_sync(S, L.blocks);
  a.tol = tol;
  a.maxit = maxit;
  a.init = init;
  a.stop_rule = o.stop_rule;
  a.result = S.result;
  a.iresult = S.iresult;
  void *args[] = {&a};
  cudaError_t ce = cudaLaunchCooperativeKernel((const void *)kernel, dim3(L.blocks), dim3(L.threads),
                                               args, 0, stream);
  count_launch();
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: cooperative launch failed: %s\n", cudaGetErrorString(ce));
    return FVC_ERR_CUDA;
  }
  return FVC_OK;
}

// The solver's scalars after a synchronous solve (the kernel has ended).
int32_t read_stats(const Scratch &S, cudaStream_t stream, cudaEvent_t e0, cudaEvent_t e1,
                   bool have_err, fvc_stats *st) {
  double res[16];
  int ires[16], err = 0;
  cudaMemcpyAsync(res, S.result, sizeof(res), cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(ires, S.iresult, sizeof(ires), cudaMemcpyDeviceToHost, stream);
  if (have_err) cudaMemcpyAsync(&err, S.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
  cudaError_t ce = cudaStreamSynchronize(stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: solver kernel failed: %s\n", cudaGetErrorString(ce));
    return FVC_ERR_CUDA;
  }
  if (err != 0) return FVC_ERR_TIMEOUT;
  if (const int32_t c = check_word_status(S, stream); c != FVC_OK) return c;
  if (st) {
    st->status = ires[1];
    st->iterations = ires[0];
    st->inner_iterations = ires[2];
    st->refinements = 0;
    st->energy = res[0];
    st->conv = res[1];
    st->final_crit = res[2];
    st->rel_residual = (res[4] > 0) ? std::sqrt(res[3] / res[4]) : std::sqrt(res[3]);
    st->solve_ms = ms;
  }
  return ires[1];
}

template <typename K>
int32_t run_persistent(K kernel, const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                       double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                       fvc_stats *st, int nvec, bool gmres) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream);
  const int32_t rc =
      enqueue_persistent(kernel, A, S, b, x, tol, maxit, init, o, stream, nvec, gmres);
  cudaEventRecord(e1, stream);
  if (rc != FVC_OK) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  return read_stats(S, stream, e0, e1, true, st);
}

// status, iterations, inner iterations and the timeout flag of the solve
// that ran last on this scratch, copied where a captured graph can read them
__global__ void solve_status_kernel(const int *iresult, const int *err, int32_t *out, int mixed) {
#ifdef FVC_CHECK
  if (err[0] == 0 && err[8] != 0) {  // a failed device check (check builds)
    out[0] = FVC_ERR_ARG;
    out[1] = 0;
    out[2] = 0;
    out[3] = err[8];
    return;
  }
#endif
  out[0] = (*err != 0) ? (int32_t)FVC_ERR_TIMEOUT : iresult[1];
  out[1] = mixed ? iresult[2] : iresult[0];
  out[2] = iresult[2];
  out[3] = *err;
}

}  // namespace

int32_t check_word_status(const Scratch &S, cudaStream_t stream) {
#ifdef FVC_CHECK
  int w = 0;
  int *cw = check_word(S);
  if (!cw) return FVC_OK;
  if (cudaMemcpyAsync(&w, cw, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (w != 0) {
    const char *what = w == kChkColumn       ? "SELL column outside [0, n)"
                       : w == kChkSliceWidth ? "slice width outside [0, n]"
                       : w == kChkOffset     ? "FP32 operator row + offset outside [0, n)"
                       : w == kChkMirror     ? "transposed-solve mirror slot outside the slots"
                       : w == kChkCluster    ? "cluster PCG column outside [0, n)"
                                             : "unknown check";
    fprintf(stderr, "fvcgpu: device check failed: %s (code %d); the solve's result is void\n",
            what, w);
    return FVC_ERR_ARG;
  }
#else
  (void)S;
  (void)stream;
#endif
  return FVC_OK;
}

int32_t run_pcg(const DeviceMatrix &A, Scratch &S, const double *b, double *x, double tol,
                int maxit, int init, const fvc_opts &o, cudaStream_t stream, fvc_stats *st) {
  // a system that fits one thread-block cluster runs there (fvc_cluster.cu)
  // unless the caller fixed the launch shape of the grid-wide kernel
  if (o.block_threads == 0 && o.blocks_per_sm == 0 && o.max_blocks == 0) {
    const int32_t rc = run_pcg_cluster(A, S, b, x, tol, maxit, init, o, stream, st);
    if (rc != FVC_ERR_UNSUPPORTED) return rc;
  }
  // p stored from 262144 rows on: per iteration on GB300 (same bits either
  // way) 98k rows 14.5 vs 13.0 us, 393k 23.0 vs 23.5, 1.57M 58.8 vs 66.2,
  // 4.19M 146 vs 161 us (stored vs formed at every read)
  if (A.n >= kStorePRows)
    return run_persistent(pcg_f64<true>, A, S, b, x, tol, maxit, init, o, stream, st, 5, false);
  return run_persistent(pcg_f64<false>, A, S, b, x, tol, maxit, init, o, stream, st, 5, false);
}

// FP64 BiCGSTAB with z stored once per row from this many rows on (below,
// the two extra grid barriers cost more than the FP64 they save; the 262k-
// row enthalpy solves of a 512^2 natural-convection loop gain: 30 outer
// iterations 2.93 -> 2.77 s; the 65k-row ones of a 256^2 loop lose: 200
// outer iterations 6.26 -> 6.55 s)
constexpr int kStoreZRows = 131072;

// BiCGSTAB on one cluster up to this many rows (a block of 256 threads per
// eight slices, at most 16 blocks): the grid-wide kernel's grid waits cost
// more than a cluster's FP64 throughput there.  Per iteration on GB300,
// cluster against grid-wide: 2025 rows 15.3 vs 18.3 us, 4096 rows 15.3 vs
// 18.3, 8100 rows 19.9 vs 19.4, 16384 rows 28.8 vs 21.9
constexpr int kBcgClusterRows = 8192;

// Enqueues the cluster BiCGSTAB when the system is small enough, the caller
// left the launch shape automatic and one cluster fits; FVC_ERR_UNSUPPORTED,
// with nothing enqueued, otherwise.  launch = false only prepares the scratch.
int32_t enqueue_bicgstab_cluster(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                                 double tol, int maxit, int init, const fvc_opts &o,
                                 cudaStream_t stream, bool launch) {
  if (A.n <= 0 || A.n > kBcgClusterRows || o.block_threads != 0 || o.blocks_per_sm != 0 ||
      o.max_blocks != 0)
    return FVC_ERR_UNSUPPORTED;
  constexpr int threads = 256;
  const int csize = std::min(16, std::max(1, (A.nslices + 7) / 8));
  static bool attrs_set = false;
  if (!attrs_set) {
    cudaFuncSetAttribute((const void *)bicgstab_cl,
                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    attrs_set = true;
  }
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[1];
  cluster_config(cfg, at, csize, threads, stream);
  int ncl = 0;
  if (cudaOccupancyMaxActiveClusters(&ncl, (const void *)bicgstab_cl, &cfg) != cudaSuccess ||
      ncl < 1) {
    cudaGetLastError();
    return FVC_ERR_UNSUPPORTED;
  }
  int32_t rc = ensure_vectors(S, (size_t)A.n, 8, 1, false);
  if (rc != FVC_OK || !launch) return rc;
  // the error block (wait and check words) and the result slots start at zero
  cudaMemsetAsync(S.err, 0, 64, stream);
  cudaMemsetAsync(S.iresult, 0, 16 * sizeof(int), stream);
  cudaMemsetAsync(S.result, 0, 16 * sizeof(double), stream);
  KArgs a{};
  a.A = view64(A);
  a.A.chk = check_word(S);
  a.m = A.jac;
  a.minv = A.jinv;
  a.b = b;
  a.x = x;
  a.v0 = S.v[0];
  a.v1 = S.v[1];
  a.v2 = S.v[2];
  a.v3 = S.v[3];
  a.v4 = S.v[4];
  a.v5 = S.v[5];
  a.v6 = S.v[6];
  a.v7 = S.v[7];
  a.gs = make_sync(S, 1);
  a.gs.nblocks = (unsigned int)csize;
  a.gs.cluster = csize > 1 ? 1 : 0;
  a.tol = tol;
  a.maxit = maxit;
  a.init = init;
  a.stop_rule = o.stop_rule;
  a.result = S.result;
  a.iresult = S.iresult;
  void *args[] = {&a};
  const cudaError_t ce = launch_groups((const void *)bicgstab_cl, csize, threads, csize, args, stream);
  count_launch();
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: cluster BiCGSTAB launch failed: %s\n", cudaGetErrorString(ce));
    cudaGetLastError();
    return FVC_ERR_CUDA;
  }
  return FVC_OK;
}

int32_t run_bicgstab(const DeviceMatrix &A, Scratch &S, const double *b, double *x, double tol,
                     int maxit, int init, const fvc_opts &o, cudaStream_t stream, fvc_stats *st) {
  if (enqueue_bicgstab_cluster(A, S, b, x, tol, maxit, init, o, stream, false) == FVC_OK) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, stream);
    const int32_t rc = enqueue_bicgstab_cluster(A, S, b, x, tol, maxit, init, o, stream, true);
    cudaEventRecord(e1, stream);
    if (rc != FVC_OK) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    return read_stats(S, stream, e0, e1, true, st);
  }
  if (A.n >= kStoreZRows)
    return run_persistent(bicgstab_f64_z, A, S, b, x, tol, maxit, init, o, stream, st, 10, false);
  return run_persistent(bicgstab_f64, A, S, b, x, tol, maxit, init, o, stream, st, 8, false);
}

int32_t run_bicgstab_transposed(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                                double tol, int maxit, int init, const fvc_opts &o,
                                cudaStream_t stream, fvc_stats *st) {
  if (!A.mirror) return FVC_ERR_UNSUPPORTED;
  return run_persistent(bicgstab_f64_t, A, S, b, x, tol, maxit, init, o, stream, st, 8, false);
}

int32_t run_gmres(const DeviceMatrix &A, Scratch &S, const double *b, double *x, double tol,
                  int maxit, const fvc_opts &o, cudaStream_t stream, fvc_stats *st) {
  return run_persistent(gmres_f64, A, S, b, x, tol, maxit, 1, o, stream, st, 0, true);
}

int32_t enqueue_solve(const DeviceMatrix &A, Scratch &S, int code, const double *b, double *x,
                      double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                      bool launch) {
  if (code == 1) {
    if (o.block_threads == 0 && o.blocks_per_sm == 0 && o.max_blocks == 0) {
      const int32_t rc = enqueue_pcg_cluster(A, S, b, x, tol, maxit, init, o, stream, launch);
      if (rc != FVC_ERR_UNSUPPORTED) return rc;
    }
    if (A.n >= kStorePRows)
      return enqueue_persistent(pcg_f64<true>, A, S, b, x, tol, maxit, init, o, stream, 5, false,
                                launch);
    return enqueue_persistent(pcg_f64<false>, A, S, b, x, tol, maxit, init, o, stream, 5, false,
                              launch);
  }
  if (code == 2) {
    const int32_t rc = enqueue_bicgstab_cluster(A, S, b, x, tol, maxit, init, o, stream, launch);
    if (rc != FVC_ERR_UNSUPPORTED) return rc;
  }
  if (code == 2)
    return A.n >= kStoreZRows
               ? enqueue_persistent(bicgstab_f64_z, A, S, b, x, tol, maxit, init, o, stream, 10,
                                    false, launch)
               : enqueue_persistent(bicgstab_f64, A, S, b, x, tol, maxit, init, o, stream, 8,
                                    false, launch);
  if (code == 3)
    return enqueue_persistent(gmres_f64, A, S, b, x, tol, maxit, 1, o, stream, 0, true, launch);
  return FVC_ERR_UNSUPPORTED;
}

int32_t launch_solve_status(const Scratch &S, int32_t *out, cudaStream_t stream, bool mixed) {
  if (!S.iresult || !S.err || !out) return FVC_ERR_ARG;
  solve_status_kernel<<<1, 1, 0, stream>>>(S.iresult, S.err, out, mixed ? 1 : 0);
  count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

const void *krylov_batched_kernel(int threads) {
  return threads <= 128   ? (const void *)krylov_batched<128>
         : threads <= 256 ? (const void *)krylov_batched<256>
                          : (const void *)krylov_batched<1024>;
}

void cluster_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *at, int csize, int threads,
                    cudaStream_t stream) {
  cfg = cudaLaunchConfig_t{};
  cfg.blockDim = dim3((unsigned)threads);
  cfg.gridDim = dim3((unsigned)csize);
  cfg.stream = stream;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
}

cudaError_t launch_groups(const void *kern, int blocks, int threads, int csize, void **args,
                          cudaStream_t stream) {
  if (csize <= 0)
    return cudaLaunchCooperativeKernel(kern, dim3((unsigned)blocks), dim3((unsigned)threads),
                                       args, 0, stream);
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[1];
  cluster_config(cfg, at, csize, threads, stream);
  cfg.gridDim = dim3((unsigned)blocks);
  return cudaLaunchKernelExC(&cfg, kern, args);
}

int32_t plan_batched(DeviceMatrix &A, Scratch &S, int nsys, const int32_t *row_start,
                     const int32_t *codes, const double *tols, const double *its_hint,
                     const int32_t *inits, const int32_t *run, double tol, const fvc_opts &o,
                     cudaStream_t stream, bool persistent, BatchPlan &P) {
  if (nsys < 1 || !row_start || !inits || row_start[0] != 0 || row_start[nsys] != A.n)
    return FVC_ERR_ARG;
  bool any_bicg = false;
  for (int s = 0; s < nsys; ++s) {
    if (row_start[s] % 32 != 0 || row_start[s + 1] <= row_start[s]) return FVC_ERR_ARG;
    const int code = codes ? codes[s] : 1;
    if (code != 1 && code != 2) return FVC_ERR_UNSUPPORTED;
    any_bicg = any_bicg || code == 2;
  }
  const bool mixed = o.precision == FVC_PREC_MIXED;
  // one thread-block cluster per system, or groups of blocks of one
  // cooperative launch (csize 0).  The p' and enthalpy systems of 256
  // SIMPLE cases (32^2 to 254^2 cells, 4.0M rows a stage), frozen, to
  // ||r|| <= 1e-8 ||b||: FP64 p' 152 ms in groups, 129 ms on clusters sized
  // per system; enthalpy 219 / 176 ms
  if (o.cluster_size < -1 || o.cluster_size > 16) return FVC_ERR_ARG;
  // csize: the largest cluster (fixed sizes: all of them); adaptive (-1, the
  // automatic choice): each system's cluster sized to it,
  // ceil(rows / (the largest system's rows / 16)) blocks, so that every block
  // has about as many rows and the per-iteration times line up
  bool adaptive = o.cluster_size <= 0;
  if (o.cluster_size == 0) {
    // automatic: clusters sized per system when their blocks fill the
    // device, else groups, where a large system can spread over more than
    // 16 blocks (the enthalpy systems of those SIMPLE cases in FP64: 256
    // cases 184 ms on clusters against 233 ms in groups; 64 cases 83
    // against 52 ms)
    int most_rows = 0;
    for (int s = 0; s < nsys; ++s)
      most_rows = std::max(most_rows, row_start[s + 1] - row_start[s]);
    const long per = std::max(1024, (most_rows + 15) / 16);
    long want = 0;
    for (int s = 0; s < nsys; ++s)
      want += std::min<long>(16, std::max<long>(1, (row_start[s + 1] - row_start[s] + per - 1) / per));
    int occ256 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ256, mixed ? mixed_batched_kernel(256) : krylov_batched_kernel(256), 256, 0);
    if (want < (long)std::max(occ256, 1) * sm_count()) adaptive = false;
  }
  int csize = (o.cluster_size == 1)   ? 0
              : (o.cluster_size >= 2) ? o.cluster_size
              : adaptive              ? 16
                                      : 0;
  // groups: 128-thread blocks by default, twice the co-resident blocks of
  // 256, so the one-block minimum of the small systems takes a smaller share
  // (the u, v, T and p' systems of 256 heated cavities, 1024 systems: 184 ms
  // at 128 threads, 215 at 256, 386 at 512); clusters: 256
  auto threads_for = [&](int cs) {
    return (o.block_threads > 0) ? block_threads_for(o.block_threads, 0, 1) : cs > 0 ? 256 : 128;
  };
  int threads = threads_for(csize);
  if (mixed) {
    int32_t rc = build_f32_copy(A, stream, o.fp32_layout);
    if (rc == FVC_OK) rc = ensure_f32_vectors(S, (size_t)A.n);
    if (rc != FVC_OK) return rc;
  }
  int occ = 0;
  // PCG stores p: most groups of a batch are one block, where publishing p
  // is a __syncthreads (the same 1024 systems: 159 ms vs 184 ms)
  const void *kern = mixed ? mixed_batched_kernel(threads) : krylov_batched_kernel(threads);
  int cap = 0;
  if (csize > 0) {
    // ordinary launches of one cluster per system: no co-residency bound,
    // but one cluster of the largest size must fit on the device
    bool fits = csize <= 8 ||
                cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                    cudaSuccess;
    int ncl = 0;
    if (fits) {
      cudaLaunchConfig_t cfg{};
      cudaLaunchAttribute at[1];
      cluster_config(cfg, at, csize, threads, stream);
      fits = cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg) == cudaSuccess && ncl >= 1;
    }
    if (!fits) {
      cudaGetLastError();
      if (o.cluster_size != 0) {
        fprintf(stderr, "fvcgpu: no cluster of %d blocks of %d threads fits the device\n",
                csize, threads);
        return FVC_ERR_UNSUPPORTED;
      }
      // the automatic choice falls back to groups
      csize = 0;
      adaptive = false;
      threads = threads_for(0);
      kern = mixed ? mixed_batched_kernel(threads) : krylov_batched_kernel(threads);
    }
  }
  if (csize == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, 0);
    if (occ <= 0) occ = 1;
    if (o.blocks_per_sm > 0 && o.blocks_per_sm < occ) occ = o.blocks_per_sm;
    cap = occ * sm_count();
    if (o.max_blocks > 0) cap = std::min(cap, o.max_blocks);
    if (nsys > cap) {
      fprintf(stderr, "fvcgpu: %d systems exceed the %d co-resident blocks of one launch\n", nsys,
              cap);
      return FVC_ERR_ARG;
    }
  }
  // blocks per system in proportion to its work: slices x the expected
  // iterations (the caller's hint, else sqrt(rows), the growth of the
  // iteration count with the mesh size) x the SpMVs per iteration (2 for
  // BiCGSTAB); at most one slice per warp.  Water-filling: a system whose share is
  // below one block gets one, the others share the rest, and blocks left
  // over by rounding go to the largest remainders.
  const int warps = threads / 32;
  std::vector<int> nb(nsys, 0), slices(nsys), most(nsys);
  std::vector<double> wt(nsys), frac(nsys, 0.0);
  std::vector<char> fixed(nsys, 0);
  double wleft = 0.0;
  for (int s = 0; s < nsys; ++s) {
    const int rows = row_start[s + 1] - row_start[s];
    slices[s] = (rows + 31) / 32;
    most[s] = (slices[s] + warps - 1) / warps;
    const double its = (its_hint && its_hint[s] > 0.0) ? its_hint[s] : std::sqrt((double)rows);
    wt[s] = slices[s] * its * ((codes && codes[s] == 2) ? 2.0 : 1.0);
    wleft += wt[s];
  }
  // clusters: csize blocks each (adaptive: each system's own size), one
  // launch per size, the heaviest systems first within it (the hardware
  // starts clusters roughly in launch order, so the long solves begin at once)
  std::vector<int> order(nsys);
  for (int s = 0; s < nsys; ++s) order[s] = s;
  int nseg = 0, seg_csize[BatchPlan::kMaxSeg] = {}, seg_blocks[BatchPlan::kMaxSeg] = {},
      seg_off[BatchPlan::kMaxSeg] = {};
  if (csize > 0) {
    if (adaptive) {
      int most_rows = 0;
      for (int s = 0; s < nsys; ++s) most_rows = std::max(most_rows, slices[s] * 32);
      const int per = std::max(1024, (most_rows + 15) / 16);
      for (int s = 0; s < nsys; ++s)
        nb[s] = (int)std::min<long>(16, std::max<long>(1, ((long)slices[s] * 32 + per - 1) / per));
    } else {
      std::fill(nb.begin(), nb.end(), csize);
    }
    // segments by cluster size, largest first; within one, heaviest first
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
      return nb[p] != nb[q] ? nb[p] > nb[q] : wt[p] > wt[q];
    });
    for (int i = 0; i < nsys; ++i) {
      const int c = nb[order[i]];
      if (nseg == 0 || seg_csize[nseg - 1] != c) {
        seg_csize[nseg] = c;
        seg_off[nseg] = (nseg == 0) ? 0 : seg_off[nseg - 1] + seg_blocks[nseg - 1];
        ++nseg;
      }
      seg_blocks[nseg - 1] += c;
    }
    std::fill(fixed.begin(), fixed.end(), 1);
    wleft = 0.0;
  }
  long capleft = cap;
  for (bool changed = csize == 0; changed;) {
    changed = false;
    for (int s = 0; s < nsys; ++s) {
      if (fixed[s]) continue;
      const double share = capleft * wt[s] / wleft;
      if (share < 1.0 || share >= most[s]) {
        nb[s] = share < 1.0 ? 1 : most[s];
        fixed[s] = 1;
        capleft -= nb[s];
        wleft -= wt[s];
        changed = true;
      }
    }
    if (wleft <= 0.0) break;
  }
  long total = 0;
  for (int s = 0; s < nsys; ++s) {
    if (!fixed[s]) {
      const double share = capleft * wt[s] / wleft;
      nb[s] = std::max(1, (int)std::floor(share));
      frac[s] = share - nb[s];
    }
    total += nb[s];
  }
  while (csize == 0 && total < cap) {  // rounding leftovers: largest remainder first
    int k = -1;
    for (int s = 0; s < nsys; ++s)
      if (!fixed[s] && nb[s] < most[s] && (k < 0 || frac[s] > frac[k])) k = s;
    if (k < 0 || frac[k] <= 0.0) break;
    ++nb[k];
    frac[k] = 0.0;
    ++total;
  }
  while (csize == 0 && total > cap) {  // trim the largest shares (nsys <= cap keeps one each)
    int k = 0;
    for (int s = 1; s < nsys; ++s)
      if (nb[s] > nb[k]) k = s;
    --nb[k];
    --total;
  }
  // one device buffer: per system a 64-byte counter sector, partials and
  // totals, results; then the error word, descriptors and block map
  size_t part_doubles = 0;
  for (int s = 0; s < nsys; ++s) part_doubles += (size_t)4 * kMaxNV * (nb[s] + 1);
  const size_t ctr_bytes = (size_t)nsys * 64 + 64;
  const size_t res_bytes = (size_t)nsys * 16 * sizeof(double);
  const size_t ires_bytes = (size_t)nsys * 16 * sizeof(int);
  const size_t sys_bytes = (size_t)nsys * sizeof(BatchSys);
  const size_t sob_bytes = (size_t)total * sizeof(int);
  const size_t bytes =
      ctr_bytes + part_doubles * sizeof(double) + res_bytes + ires_bytes + sys_bytes + sob_bytes;
  char *buf = nullptr;
  if (persistent ? cudaMalloc((void **)&buf, bytes) != cudaSuccess
                 : cudaMallocAsync((void **)&buf, bytes, stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  unsigned int *ctr = reinterpret_cast<unsigned int *>(buf);
  int *err = reinterpret_cast<int *>(buf + (size_t)nsys * 64);
  double *part = reinterpret_cast<double *>(buf + ctr_bytes);
  double *res = part + part_doubles;
  int *ires = reinterpret_cast<int *>(res + (size_t)nsys * 16);
  BatchSys *dsys = reinterpret_cast<BatchSys *>(reinterpret_cast<char *>(ires) + ires_bytes);
  int *dsob = reinterpret_cast<int *>(reinterpret_cast<char *>(dsys) + sys_bytes);
  std::vector<BatchSys> hsys(nsys);
  std::vector<int> hsob((size_t)total);
  size_t poff = 0;
  int b0 = 0, seg = 0;
  for (int i = 0; i < nsys; ++i) {
    const int s = order[i];
    BatchSys &d = hsys[s];
    while (csize > 0 && seg + 1 < nseg && b0 >= seg_off[seg + 1]) ++seg;
    d.s0 = row_start[s] / 32;
    d.s1 = d.s0 + slices[s];
    d.code = codes ? codes[s] : 1;
    d.init = inits[s];
    d.tol = tols ? tols[s] : tol;
    // mixed precision: FP32 reduction per reliable update (CG) or per
    // defect-correction sweep (BiCGSTAB), as in a single solve
    d.inner_tol = (o.inner_tol > 0) ? o.inner_tol : kInnerTolDefault;
    d.gs.count = ctr + (size_t)s * 16;
    d.gs.flag = ctr + (size_t)s * 16 + 8;
    d.gs.err = err;
    d.gs.partials = part + poff;
    d.gs.totals = part + poff + (size_t)4 * kMaxNV * nb[s];
    d.gs.nblocks = (unsigned int)nb[s];
    // a cluster launch numbers its blocks from 0: the base within the segment
    d.gs.base = (unsigned int)(csize > 0 ? b0 - seg_off[seg] : b0);
    // a one-block cluster needs no cluster barrier: the block's own sums
    d.gs.cluster = (csize > 0 && nb[s] > 1) ? 1 : 0;
    d.result = res + (size_t)s * 16;
    d.iresult = ires + (size_t)s * 16;
    d.run = run ? run + s : nullptr;
    poff += (size_t)4 * kMaxNV * (nb[s] + 1);
    for (int k = 0; k < nb[s]; ++k) hsob[(size_t)b0 + k] = s;
    b0 += nb[s];
  }
  int32_t rc = mixed ? FVC_OK : ensure_vectors(S, (size_t)A.n, any_bicg ? 10 : 5, 1, false);
#ifdef FVC_CHECK
  // the check word lives in the scratch's error block (check builds)
  if (rc == FVC_OK) rc = ensure_sync(S, 1);
  if (rc == FVC_OK) cudaMemsetAsync(S.err, 0, 64, stream);
#endif
  if (rc != FVC_OK) {
    if (persistent)
      cudaFree(buf);
    else
      cudaFreeAsync(buf, stream);
    return rc;
  }
  cudaMemcpyAsync(dsys, hsys.data(), sys_bytes, cudaMemcpyHostToDevice, stream);
  cudaMemcpyAsync(dsob, hsob.data(), sob_bytes, cudaMemcpyHostToDevice, stream);
  if (persistent && cudaStreamSynchronize(stream) != cudaSuccess) {  // host vectors die here
    cudaFree(buf);
    return FVC_ERR_CUDA;
  }
  P.nsys = nsys;
  P.total = (int)total;
  P.threads = threads;
  P.cluster = csize;
  if (csize == 0) {  // groups: one cooperative launch of every block
    nseg = 1;
    seg_csize[0] = 0;
    seg_blocks[0] = (int)total;
    seg_off[0] = 0;
  }
  P.nseg = nseg;
  for (int k = 0; k < nseg; ++k) {
    P.seg_csize[k] = seg_csize[k];
    P.seg_blocks[k] = seg_blocks[k];
    P.seg_off[k] = seg_off[k];
  }
  P.mixed = mixed;
  P.kern = kern;
  P.buf = buf;
  P.persistent = persistent;
  P.ctr_bytes = ctr_bytes;
  P.res_bytes = res_bytes;
  P.ires_bytes = ires_bytes;
  P.err = err;
  P.res = res;
  P.ires = ires;
  P.dsys = dsys;
  P.dsob = dsob;
  P.tol = tol;
  P.fp32_layout = o.fp32_layout;
  // the segments after the first run on their own streams
  if (nseg > 1) {
    bool ok = cudaEventCreateWithFlags(&P.fork, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 1; k < nseg && ok; ++k)
      ok = cudaStreamCreateWithFlags(&P.aux[k], cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&P.join[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      free_batched(P, stream);
      return FVC_ERR_CUDA;
    }
  }
  return FVC_OK;
}

// The plan's launches: one (groups, or clusters of one size), or one per
// cluster size, the first on the caller's stream and the others on the
// plan's streams, forked from it after everything enqueued so far and
// joined back into it (event waits: stream-ordered and capturable).
template <typename L>
int32_t launch_segments(const BatchPlan &P, cudaStream_t stream, L &&launch) {
  if (P.nseg <= 1) return launch(0, stream);
  if (cudaEventRecord(P.fork, stream) != cudaSuccess) return FVC_ERR_CUDA;
  for (int k = 1; k < P.nseg; ++k)
    if (cudaStreamWaitEvent(P.aux[k], P.fork, 0) != cudaSuccess) return FVC_ERR_CUDA;
  int32_t rc = FVC_OK;
  for (int k = 0; k < P.nseg; ++k) {
    const int32_t r = launch(k, k == 0 ? stream : P.aux[k]);
    if (r != FVC_OK && rc == FVC_OK) rc = r;
  }
  for (int k = 1; k < P.nseg; ++k) {
    if (cudaEventRecord(P.join[k], P.aux[k]) != cudaSuccess ||
        cudaStreamWaitEvent(stream, P.join[k], 0) != cudaSuccess)
      rc = FVC_ERR_CUDA;
  }
  return rc;
}

int32_t enqueue_batched(DeviceMatrix &A, Scratch &S, const BatchPlan &P, const double *b,
                        double *x, int maxit, const fvc_opts &o, cudaStream_t stream) {
  // counters, the error word and every system's result slots start at zero
  if (cudaMemsetAsync(P.buf, 0, P.ctr_bytes, stream) != cudaSuccess ||
      cudaMemsetAsync(P.res, 0, P.res_bytes + P.ires_bytes, stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (P.mixed) {
    // the FP32 operator of the current values (stream-ordered once its
    // layout is decided, which planning did)
    int32_t rc = build_f32_copy(A, stream, P.fp32_layout);
    if (rc != FVC_OK) return rc;
    return launch_segments(P, stream, [&](int k, cudaStream_t st) {
      return launch_mixed_batched(A, S, P.dsys, P.dsob + P.seg_off[k], P.seg_blocks[k],
                                  P.threads, P.seg_csize[k], b, x, maxit, o, st);
    });
  }
  KArgs a{};
  a.A = view64(A);
  a.A.chk = check_word(S);
  a.m = A.jac;
  a.minv = A.jinv;
  a.b = b;
  a.x = x;
  a.v0 = S.v[0];
  a.v1 = S.v[1];
  a.v2 = S.v[2];
  a.v3 = S.v[3];
  a.v4 = S.v[4];
  a.v5 = S.v[5];
  a.v6 = S.v[6];
  a.v7 = S.v[7];
  a.v8 = S.v[8];
  a.v9 = S.v[9];
  a.tol = P.tol;
  a.maxit = maxit;
  a.init = 1;
  a.stop_rule = o.stop_rule;
  return launch_segments(P, stream, [&](int k, cudaStream_t st) {
    const BatchSys *psys = P.dsys;
    const int *psob = P.dsob + P.seg_off[k];
    void *args[] = {&a, &psys, &psob};
    const cudaError_t ce =
        launch_groups(P.kern, P.seg_blocks[k], P.threads, P.seg_csize[k], args, st);
    count_launch();
    if (ce != cudaSuccess) {
      fprintf(stderr, "fvcgpu: batched launch failed: %s\n", cudaGetErrorString(ce));
      return FVC_ERR_CUDA;
    }
    return FVC_OK;
  });
}

void free_batched(BatchPlan &P, cudaStream_t stream) {
  if (P.buf) {
    if (P.persistent)
      cudaFree(P.buf);
    else
      cudaFreeAsync(P.buf, stream);
  }
  // (a stream destroyed with work pending finishes that work first)
  for (int k = 0; k < BatchPlan::kMaxSeg; ++k) {
    if (P.aux[k]) cudaStreamDestroy(P.aux[k]);
    if (P.join[k]) cudaEventDestroy(P.join[k]);
  }
  if (P.fork) cudaEventDestroy(P.fork);
  P = BatchPlan();
}

int32_t run_krylov_batched(DeviceMatrix &A, Scratch &S, int nsys,
                           const int32_t *row_start, const int32_t *codes, const double *tols,
                           const double *its_hint, const int32_t *inits, const double *b,
                           double *x, double tol, int maxit, const fvc_opts &o,
                           cudaStream_t stream, fvc_stats *st) {
  BatchPlan P;
  int32_t rc = plan_batched(A, S, nsys, row_start, codes, tols, its_hint, inits, nullptr, tol, o,
                            stream, false, P);
  if (rc != FVC_OK) return rc;
  const bool mixed = P.mixed;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream);
  rc = enqueue_batched(A, S, P, b, x, maxit, o, stream);
  cudaEventRecord(e1, stream);
  std::vector<double> hres((size_t)nsys * 16);
  std::vector<int> hires((size_t)nsys * 16);
  int herr = 0;
  if (rc == FVC_OK) {
    cudaMemcpyAsync(hres.data(), P.res, P.res_bytes, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(hires.data(), P.ires, P.ires_bytes, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(&herr, P.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
  }
  free_batched(P, stream);
  cudaError_t ce2 = cudaStreamSynchronize(stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != FVC_OK) return rc;
  if (ce2 != cudaSuccess) return FVC_ERR_CUDA;
  if (herr != 0) return FVC_ERR_TIMEOUT;
  if (const int32_t c = check_word_status(S, stream); c != FVC_OK) return c;
  // mixed BiCGSTAB systems whose FP32 sweeps stalled (the kernel's stall
  // rule: FVC_ERR_NOCONV below max_refine sweeps and maxit iterations) are
  // finished in FP64 from their iterate, on ||r|| <= tol ||b||, in one more
  // batched launch over those systems alone -- as a single mixed solve does
  std::vector<char> fin((size_t)nsys, 0);
  std::vector<double> hres64;
  std::vector<int> hires64;
  if (mixed) {
    const int max_refine = (o.max_refine > 0) ? o.max_refine : 30;
    std::vector<int32_t> run2((size_t)nsys, 0);
    int nfin = 0;
    for (int s = 0; s < nsys; ++s) {
      const int *ir = &hires[(size_t)s * 16];
      if (codes && codes[s] == 2 && ir[1] == FVC_ERR_NOCONV && ir[0] < max_refine &&
          ir[2] < maxit) {
        run2[s] = 1;
        fin[s] = 1;
        ++nfin;
      }
    }
    if (nfin > 0) {
      fvc_opts f = o;
      f.precision = FVC_PREC_FP64;
      f.stop_rule = 1;
      const std::vector<int32_t> warm((size_t)nsys, 0);
      int32_t *run2_d = nullptr;
      if (cudaMallocAsync((void **)&run2_d, sizeof(int32_t) * nsys, stream) != cudaSuccess)
        return FVC_ERR_CUDA;
      cudaMemcpyAsync(run2_d, run2.data(), sizeof(int32_t) * nsys, cudaMemcpyHostToDevice,
                      stream);
      BatchPlan P64;
      rc = plan_batched(A, S, nsys, row_start, codes, tols, nullptr, warm.data(), run2_d, tol, f,
                        stream, false, P64);
      if (rc == FVC_OK) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, stream);
        rc = enqueue_batched(A, S, P64, b, x, maxit, f, stream);
        cudaEventRecord(e1, stream);
        hres64.resize((size_t)nsys * 16);
        hires64.resize((size_t)nsys * 16);
        if (rc == FVC_OK) {
          cudaMemcpyAsync(hres64.data(), P64.res, P64.res_bytes, cudaMemcpyDeviceToHost, stream);
          cudaMemcpyAsync(hires64.data(), P64.ires, P64.ires_bytes, cudaMemcpyDeviceToHost,
                          stream);
          cudaMemcpyAsync(&herr, P64.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
        }
        free_batched(P64, stream);
        cudaFreeAsync(run2_d, stream);
        ce2 = cudaStreamSynchronize(stream);
        float ms2 = 0.f;
        cudaEventElapsedTime(&ms2, e0, e1);
        ms += ms2;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc == FVC_OK && ce2 != cudaSuccess) rc = FVC_ERR_CUDA;
        if (rc == FVC_OK && herr != 0) rc = FVC_ERR_TIMEOUT;
      } else {
        cudaFreeAsync(run2_d, stream);
      }
      if (rc != FVC_OK) return rc;
    }
  }
  int32_t worst = FVC_OK;
  for (int s = 0; s < nsys; ++s) {
    const double *r = &hres[(size_t)s * 16];
    const int *ir = &hires[(size_t)s * 16];
    int its64 = 0;
    if (fin[s]) {  // the FP64 finish's status and residual, its iterations
      const int *i2 = &hires64[(size_t)s * 16];
      hires[(size_t)s * 16 + 1] = i2[1];
      its64 = i2[0];
      hres[(size_t)s * 16 + 3] = hres64[(size_t)s * 16 + 3];
      hres[(size_t)s * 16 + 4] = hres64[(size_t)s * 16 + 4];
    }
    if (ir[1] == FVC_ERR_NAN) worst = FVC_ERR_NAN;
    else if (ir[1] != FVC_OK && worst == FVC_OK) worst = ir[1];
    if (st) {
      fvc_stats &t = st[s];
      memset(&t, 0, sizeof(t));
      t.status = ir[1];
      // mixed: FP32 iterations (plus those of an FP64 finish), FP32
      // iterations, and reliable updates / sweeps
      t.iterations = mixed ? ir[2] + its64 : ir[0];
      t.inner_iterations = mixed ? ir[2] : 0;
      t.refinements = mixed ? ir[0] : 0;
      t.energy = mixed ? 0.0 : r[0];
      t.conv = r[1];
      t.final_crit = r[2];
      t.rel_residual = (r[4] > 0) ? std::sqrt(r[3] / r[4]) : std::sqrt(r[3]);
      t.solve_ms = ms;
    }
  }
  return worst;
}

int32_t launch_spmv(const DeviceMatrix &A, const double *x, double *y, cudaStream_t stream,
                    bool fused) {
  if (A.n <= 0) return FVC_ERR_ARG;
  const int threads = 256;
  int blocks = (A.nslices + 7) / 8;
  blocks = std::max(1, std::min(blocks, sm_count() * 8));
  if (fused)
    spmv_f64<true><<<blocks, threads, 0, stream>>>(view64(A), x, y);
  else
    spmv_f64<false><<<blocks, threads, 0, stream>>>(view64(A), x, y);
  count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t launch_spmv_f32(const DeviceMatrix &A, const float *x, float *y, cudaStream_t stream) {
  if (A.n <= 0 || !A.have32) return FVC_ERR_ARG;
  const int threads = 256;
  int blocks = (A.nslices + 7) / 8;
  blocks = std::max(1, std::min(blocks, sm_count() * 8));
  if (A.ell_w == 4)
    spmv_f32<4><<<blocks, threads, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.col16,
                                                A.val32, A.diag32, x, y);
  else if (A.ell_w == 3)
    spmv_f32<3><<<blocks, threads, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.col16,
                                                A.val32, A.diag32, x, y);
  else
    spmv_f32<0><<<blocks, threads, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.col16,
                                                A.val32, A.diag32, x, y);
  count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t launch_reciprocal(const DeviceMatrix &A, cudaStream_t stream) {
  if (A.n <= 0 || !A.jac || !A.jinv) return FVC_ERR_ARG;
  reciprocal_kernel<<<(A.n + 255) / 256, 256, 0, stream>>>(A.n, A.jac, A.jinv);
  count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

}  // namespace fvc
