// fvc_mixed.cu -- mixed-precision solves: FP32 Krylov iterations with the
// solution and the true residual kept in FP64, one persistent launch.
//
// FP32 operator.  The matrix is stored for the FP32 iterations in
// difference form
//     (A x)_i = e_i x_i + sum_k w_ik (x_i - x_k),
//     w_ik = -a_ik (FP32 per slot),  e_i = a_ii - sum_k w_ik (FP32 per row),
// an exact identity for any matrix.  For the finite-volume matrices of the
// reference the rows of a Neumann pressure-correction system sum to zero
// (e_i = 0) and FP32 rounding of the weights then perturbs the operator only
// relatively, so its near-null space (the lowest eigenvalues, O(1e-7) at a
// few million cells) survives; rounding a_ii and a_ik separately would shift
// those eigenvalues by a comparable absolute amount and stall the solve.
// The Jacobi preconditioner m = ad (src/Solver.f:84) is applied as an FP32
// reciprocal.  A row whose m lies beyond FP32 range (the 1e60 pressure pin
// of src/CellibPressure.f:557) gets 1/m = 0 there and is moved only by the
// FP64 Jacobi step of each reliable update (fold_correction).
//
// CG (code 1): Jacobi-PCG with reliable updates (residual replacement): the
// correction e accumulates alpha*p as an unevaluated FP32 pair (hi + lo,
// products split exactly with FMA, sums by TwoSum), which keeps it as
// accurate as FP64 with FP32 arithmetic -- rounding it to one FP32 number
// would add a residual error of order eps32 * cond(A) per update cycle and
// stall the solve at a few million cells.  Whenever the FP32 residual has
// dropped by a factor inner_tol (default 0.1) since the last update, or
// looks converged, x += e in FP64, the true residual b - A x is recomputed
// with the FP64 matrix, and replaces the FP32 residual.  The search
// direction survives updates, so the iteration count stays close to the
// FP64 PCG count while the iterations stream FP32 data.
// BiCGSTAB (code 2): the reference's Jacobi BiCGSTAB (src/Iterativos.f:
// 140-234) in FP32 on the correction equation, restarted from the FP64
// residual (defect correction) after each inner reduction by inner_tol
// (default 1e-4).
// Both stop on ||b - A x||2 <= refine_tol * ||b||2 recomputed in FP64.  Dot
// products and norms: each thread sums its rows with compensated FP32
// (TwoSum), the per-thread pairs are combined in FP64.  GB300 executes FP64
// at ~1/64 of its FP32 rate, so the iteration keeps the FP64 pipe idle.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "fvc_device.cuh"
#include "fvc_internal.h"

namespace fvc {

namespace {

constexpr double kF32Clamp = 1.0e30;

// Compensated FP32 sum (TwoSum per term); value() folds it to FP64.  The
// _rn intrinsics keep the compiler from contracting the error terms.
struct CSum {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float v) {
    const float t = __fadd_rn(s, v);
    const float bp = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(v, bp)));
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// (hi, lo) += alpha * p with alpha given as an FP32 pair (ah, al): the
// product ah*p is split exactly with an FMA, the sum uses TwoSum and a
// final Fast2Sum renormalisation.
__device__ __forceinline__ float2 df_axpy(float2 e, float ah, float al, float p) {
  const float th = __fmul_rn(ah, p);
  const float terr = fmaf(ah, p, -th);
  const float tl = fmaf(al, p, terr);
  const float s = __fadd_rn(e.x, th);
  const float bp = __fsub_rn(s, e.x);
  const float err = __fadd_rn(__fsub_rn(e.x, __fsub_rn(s, bp)), __fsub_rn(th, bp));
  const float lo = __fadd_rn(__fadd_rn(e.y, tl), err);
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// e_i (FP64 sum, rounded once), Jacobi 1/m, and the FP32 weights.
__global__ void build_f32_operator(int n, int nslices, const int64_t *__restrict__ sptr,
                                   const int *__restrict__ col, const double *__restrict__ val,
                                   const double *__restrict__ jac, float *__restrict__ w32,
                                   float *__restrict__ e32, float *__restrict__ minv32) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += nw) {
    const int row = s * 32 + lane;
    const int64_t base = sptr[s];
    const int wd = (int)((sptr[s + 1] - base) >> 5);
    double off = 0.0;  // sum of a_ik over true off-diagonal slots
    for (int k = 0; k < wd; ++k) {
      const int64_t q = base + 32 * k + lane;
      const bool diag_slot = (row < n) && (col[q] == row);
      const double a = (row < n && !diag_slot) ? val[q] : 0.0;
      off += a;
      w32[q] = (float)(-a);
    }
    if (row < n) {
      const double m = jac[row];
      double e = m + off;
      e = fmin(fmax(e, -kF32Clamp), kF32Clamp);
      e32[row] = (float)e;
      minv32[row] = (fabs(m) > 1.0e37 || m == 0.0) ? 0.0f : (float)(1.0 / m);
    }
  }
}

struct MArgs {
  SellView<double> A;   // FP64 matrix (true residuals)
  const float *w32;     // weights per slot
  const float *e32;     // row excess
  const float *minv;    // Jacobi 1/m (0 on rows whose m is beyond FP32)
  const double *jac;    // m in FP64
  const double *b;
  double *x;
  float *rs, *pa, *pb, *q, *r0, *v, *t, *z;
  float *rsl;           // CG: low part of the residual (FP32 pair rs + rsl)
  float2 *e;            // correction, FP32 pair (hi, lo)
  GridSync gs;
  double target;        // refine tolerance on ||b-Ax||/||b||
  double inner_tol;
  int max_refine;
  int update_beta;      // 1: beta from the recursive residual at updates
  int maxit;            // cap on total inner iterations
  int init;
  double *result;
  int *iresult;
  double *trace;        // (iteration, relres) per residual replacement
};

// (A y)_row in FP32 difference form, y supplied by a functor.
template <typename YF>
__device__ __forceinline__ float arow32(const MArgs &a, int s, int lane, int row, YF yf) {
  const int64_t base = a.A.sptr[s];
  const int w = (int)((a.A.sptr[s + 1] - base) >> 5);
  const int *cp = a.A.col + base + lane;
  const float *vp = a.w32 + base + lane;
  const float yi = yf(row);
  float t = ld_stream(a.e32 + row) * yi;
  if (w <= 4) {
    int c[4];
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      c[k] = (k < w) ? ld_stream(cp + 32 * k) : row;
      v[k] = (k < w) ? ld_stream(vp + 32 * k) : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < w) t = fmaf(v[k], yi - yf(c[k]), t);
    return t;
  }
  for (int k = 0; k < w; ++k) t = fmaf(ld_stream(vp + 32 * k), yi - yf(ld_stream(cp + 32 * k)), t);
  return t;
}

struct MPart {
  int lane, warp, nwarps, sb, se, n;
  __device__ MPart(int nslices, int nrows) {
    lane = threadIdx.x & 31;
    warp = threadIdx.x >> 5;
    nwarps = blockDim.x >> 5;
    const int spb = (nslices + gridDim.x - 1) / gridDim.x;
    sb = blockIdx.x * spb;
    se = min(nslices, sb + spb);
    n = nrows;
  }
};

#define MFOR_ROWS(P)                                               \
  for (int s_ = (P).sb + (P).warp; s_ < (P).se; s_ += (P).nwarps) \
    for (int row = s_ * 32 + (P).lane, once_ = 1; once_ && row < (P).n; once_ = 0)

// FP64 residual sweep: rs = b - A x rounded to FP32.  Returns ||b-Ax||^2,
// ||b||^2, rs.(rs/m) and ||b-Ax||^2 over the rows the FP32 iteration moves
// (FP64 sums).
__device__ __forceinline__ bool residual_sweep(const MArgs &a, unsigned int &ep, bool zero_x,
                                               double (&out)[4], double *red) {
  const MPart P(a.A.nslices, a.A.n);
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const double *x = a.x;
  MFOR_ROWS(P) {
    double ax = zero_x ? 0.0 : sell_row_fma(a.A, s_, P.lane, row, [&](int k) { return x[k]; });
    if (zero_x) a.x[row] = 0.0;
    const double bi = a.b[row];
    const double ri = bi - ax;
    const float rsi = (float)ri;
    a.rs[row] = rsi;
    if (a.rsl) a.rsl[row] = (float)(ri - (double)rsi);
    acc[0] = fma(ri, ri, acc[0]);
    acc[1] = fma(bi, bi, acc[1]);
    const float mi = a.minv[row];
    a.z[row] = rsi * mi;
    acc[2] = fma((double)rsi, (double)(rsi * mi), acc[2]);
    if (mi != 0.0f) acc[3] = fma(ri, ri, acc[3]);
  }
  if (!grid_allreduce<4>(a.gs, ep, acc, red)) return false;
  out[0] = acc[0];
  out[1] = acc[1];
  out[2] = acc[2];
  out[3] = acc[3];
  return true;
}

// x += e (FP64) and e = 0, own rows; a barrier must follow.  Rows whose
// diagonal is beyond FP32 range (1/m = 0: the pressure pin) are frozen in
// the FP32 iteration; they take one FP64 Jacobi step on their current
// residual estimate instead, which solves such a row to FP64 accuracy.
__device__ __forceinline__ void fold_correction(const MArgs &a) {
  const MPart P(a.A.nslices, a.A.n);
  MFOR_ROWS(P) {
    const float2 ev = a.e[row];
    double dx = (double)ev.x + (double)ev.y;
    const double m = a.jac[row];
    if (a.minv[row] == 0.0f && m != 0.0) dx += (double)a.rs[row] / m;
    a.x[row] = a.x[row] + dx;
    a.e[row] = make_float2(0.0f, 0.0f);
  }
}

// CG phase A: p = z + beta p_prev (formed on the fly at the neighbours),
// q = A p, returns p.q.  Each warp handles two slices per step and issues
// every load of both before any arithmetic, so two slices' streams and
// gathers are in flight per warp (the loop is latency-bound otherwise).
template <bool kFirst>
__device__ __forceinline__ double cg_phase_a(const MArgs &a, const MPart &P, float beta,
                                             const float *__restrict__ z,
                                             const float *__restrict__ pp,
                                             float *__restrict__ pcur, float *__restrict__ q,
                                             float2 *__restrict__ e) {
  CSum cpq;
  const int n = P.n;
  const int64_t *__restrict__ sptr = a.A.sptr;
  const int *__restrict__ col = a.A.col;
  const float *__restrict__ w32 = a.w32;
  const float *__restrict__ e32 = a.e32;
  for (int s0 = P.sb + P.warp; s0 < P.se; s0 += 2 * P.nwarps) {
    int row[2], wd[2];
    bool ok[2];
    int64_t base[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int sl = s0 + u * P.nwarps;
      row[u] = sl * 32 + P.lane;
      ok[u] = (sl < P.se) && (row[u] < n);
      base[u] = 0;
      wd[u] = 0;
      if (sl < P.se) {
        base[u] = sptr[sl];
        wd[u] = (int)((sptr[sl + 1] - base[u]) >> 5);
      }
    }
    if (wd[0] > 4 || wd[1] > 4) {  // wide slices: one row at a time
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (!ok[u]) continue;
        auto pf = [&](int k) { return kFirst ? z[k] : fmaf(beta, pp[k], z[k]); };
        const float pi = pf(row[u]);
        const float t = arow32(a, s0 + u * P.nwarps, P.lane, row[u], pf);
        pcur[row[u]] = pi;
        q[row[u]] = t;
        if (kFirst) e[row[u]] = make_float2(0.0f, 0.0f);
        cpq.add(pi * t);
      }
      continue;
    }
    int c[2][4];
    float w[2][4], ex[2], zo[2], po[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const bool use = ok[u] && k < wd[u];
        c[u][k] = use ? ld_stream(col + base[u] + 32 * k + P.lane) : (ok[u] ? row[u] : 0);
        w[u][k] = use ? ld_stream(w32 + base[u] + 32 * k + P.lane) : 0.0f;
      }
      ex[u] = ok[u] ? ld_stream(e32 + row[u]) : 0.0f;
      zo[u] = ok[u] ? z[row[u]] : 0.0f;
      po[u] = (!kFirst && ok[u]) ? pp[row[u]] : 0.0f;
    }
    float nb[2][4];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int ck = c[u][k];
        nb[u][k] = kFirst ? z[ck] : fmaf(beta, pp[ck], z[ck]);
      }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (!ok[u]) continue;
      const float pi = kFirst ? zo[u] : fmaf(beta, po[u], zo[u]);
      float t = ex[u] * pi;
#pragma unroll
      for (int k = 0; k < 4; ++k) t = fmaf(w[u][k], pi - nb[u][k], t);
      pcur[row[u]] = pi;
      q[row[u]] = t;
      if (kFirst) e[row[u]] = make_float2(0.0f, 0.0f);
      cpq.add(pi * t);
    }
  }
  return cpq.value();
}

// CG phase B: e += alpha p (FP32 pair), rs -= alpha q, z = rs/m; sums
// rs.z and rs.rs (over the rows the FP32 iteration moves).  kUB slices
// per warp step, loads first.  With kPair the residual is carried as an
// FP32 pair (rs + rsl): rounding the residual recurrence to one FP32
// number delays the last decades of convergence (the lowest eigenvalues of
// the Jacobi-scaled matrix approach the FP32 rounding level), so the pair
// is switched on below kPairFrom relative residual; earlier iterations
// stream the high part only (the two parts live in separate arrays).
// Measured (and emulated in numpy): promoting the residual only late does
// not help -- the lost orthogonality dates from the first iterations -- so
// the pair runs from the start unless the caller opts out.
constexpr int kUB = 2;
constexpr double kPairFrom = 1.0e300;  // always
template <bool kPair>
__device__ __forceinline__ void cg_phase_b(const MPart &P, float alpha, float alpha_lo,
                                           const float *__restrict__ pcur,
                                           const float *__restrict__ q, float *__restrict__ rs,
                                           float *__restrict__ rsl, float *__restrict__ z,
                                           float2 *__restrict__ e,
                                           const float *__restrict__ minv, CSum &crz,
                                           CSum &crr) {
  const int n = P.n;
  for (int s0 = P.sb + P.warp; s0 < P.se; s0 += kUB * P.nwarps) {
    int row[kUB];
    bool ok[kUB];
    float2 ev[kUB];
    float pv[kUB], qv[kUB], rv[kUB], rl[kUB], mv[kUB];
#pragma unroll
    for (int u = 0; u < kUB; ++u) {
      const int sl = s0 + u * P.nwarps;
      row[u] = sl * 32 + P.lane;
      ok[u] = (sl < P.se) && (row[u] < n);
      if (ok[u]) {
        ev[u] = e[row[u]];
        pv[u] = pcur[row[u]];
        qv[u] = q[row[u]];
        rv[u] = rs[row[u]];
        rl[u] = kPair ? rsl[row[u]] : 0.0f;
        mv[u] = minv[row[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < kUB; ++u) {
      if (!ok[u]) continue;
      e[row[u]] = df_axpy(ev[u], alpha, alpha_lo, pv[u]);
      float r;
      if (kPair) {
        const float2 rp = df_axpy(make_float2(rv[u], rl[u]), -alpha, -alpha_lo, qv[u]);
        r = rp.x;
        rsl[row[u]] = rp.y;
      } else {
        r = fmaf(-alpha, qv[u], rv[u]);
      }
      const float zz = r * mv[u];
      rs[row[u]] = r;
      z[row[u]] = zz;
      crz.add(r * zz);
      if (mv[u] != 0.0f) crr.add(r * r);
    }
  }
}

__global__ void __launch_bounds__(1024, 1) mixed_cg(MArgs a) {
  __shared__ double red[kMaxNV * 32];
  const MPart P(a.A.nslices, a.A.n);
  unsigned int ep = 0;
  int status = FVC_ERR_NOCONV, updates = 0, it = 0;
  double res[4];
  if (!residual_sweep(a, ep, a.init != 0, res, red)) return;
  const double bnorm2 = res[1];
  const double scale = (bnorm2 > 0.0) ? bnorm2 : 1.0;
  double relres = sqrt(res[0] / scale);
  double rz = res[2];
  double rr_upd = res[3];  // ||r||^2 (moving rows) at the last reliable update
  const double delta2 = a.inner_tol * a.inner_tol;
  const double target2 = a.target * a.target * scale;
  float beta = 0.0f;
  float *pprev = a.pb, *pcur = a.pa;
  bool pair = relres <= kPairFrom;
  if (!(relres == relres)) status = FVC_ERR_NAN;
  else if (relres <= a.target) status = FVC_OK;
  while (status == FVC_ERR_NOCONV && it < a.maxit) {
    ++it;
    // p = z + beta p_prev (formed on the fly at the neighbours); q = A p; p.q
    double pq[1];
    if (it == 1)
      pq[0] = cg_phase_a<true>(a, P, beta, a.z, pprev, pcur, a.q, a.e);
    else
      pq[0] = cg_phase_a<false>(a, P, beta, a.z, pprev, pcur, a.q, a.e);
    if (!grid_allreduce<1>(a.gs, ep, pq, red)) return;
    const double alpha_d = rz / pq[0];
    const float alpha = (float)alpha_d;
    const float alpha_lo = (float)(alpha_d - (double)alpha);
    // e += alpha p (FP32 pair) ; rs -= alpha q ; z = rs/m ; rs.z ; rs.rs
    CSum crz, crr;
    if (pair)
      cg_phase_b<true>(P, alpha, alpha_lo, pcur, a.q, a.rs, a.rsl, a.z, a.e, a.minv, crz, crr);
    else
      cg_phase_b<false>(P, alpha, alpha_lo, pcur, a.q, a.rs, a.rsl, a.z, a.e, a.minv, crz, crr);
    double acc[2] = {crz.value(), crr.value()};
    if (!grid_allreduce<2>(a.gs, ep, acc, red)) return;
    double rz_new = acc[0];
    if (!(rz_new == rz_new)) {
      status = FVC_ERR_NAN;
      break;
    }
    if (acc[1] <= delta2 * rr_upd || acc[1] <= target2 || it >= a.maxit) {
      // reliable update: fold e into x, recompute the true residual in FP64
      fold_correction(a);
      if (!grid_barrier(a.gs, ep)) return;
      if (!residual_sweep(a, ep, false, res, red)) return;
      ++updates;
      relres = sqrt(res[0] / scale);
      if (blockIdx.x == 0 && threadIdx.x == 0 && updates <= kTraceMax) {
        a.trace[2 * (updates - 1)] = (double)it;
        a.trace[2 * (updates - 1) + 1] = relres;
      }
      if (!(relres == relres)) {
        status = FVC_ERR_NAN;
        break;
      }
      if (relres <= a.target) {
        status = FVC_OK;
        break;
      }
      if (relres <= kPairFrom) pair = true;  // the sweep wrote both parts
      rr_upd = res[3];
      if (a.update_beta) {
        // beta from the recursive residual, the next alpha from the true one
        beta = (float)(rz_new / rz);
        rz = res[2];
        float *tmp = pprev;
        pprev = pcur;
        pcur = tmp;
        continue;
      }
      rz_new = res[2];
    }
    beta = (float)(rz_new / rz);
    rz = rz_new;
    float *tmp = pprev;
    pprev = pcur;
    pcur = tmp;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.iresult[0] = updates;
    a.iresult[1] = status;
    a.iresult[2] = it;
    a.result[2] = relres;
    a.result[3] = res[0];
    a.result[4] = bnorm2;
  }
}

// The reference's Jacobi BiCGSTAB (Iterativos.f:140-234) in FP32 on the
// correction equation A e = r, inside FP64 defect correction.
__global__ void __launch_bounds__(1024, 1) mixed_bicgstab(MArgs a) {
  __shared__ double red[kMaxNV * 32];
  const MPart P(a.A.nslices, a.A.n);
  unsigned int ep = 0;
  int sweep = 0, inner_total = 0, status = FVC_ERR_NOCONV;
  double res[4];
  double relres = 0.0, bnorm2 = 0.0;
  bool zero_x = a.init != 0;
  float *sv = a.rs, *p = a.pa, *v = a.q, *t = a.t, *r0 = a.r0, *z = a.z;
  float2 *e = a.e;
  const float *minv = a.minv;
  for (sweep = 0; sweep <= a.max_refine; ++sweep) {
    if (!residual_sweep(a, ep, zero_x, res, red)) return;
    zero_x = false;
    if (sweep == 0) bnorm2 = res[1];
    relres = (bnorm2 > 0.0) ? sqrt(res[0] / bnorm2) : sqrt(res[0]);
    if (!(relres == relres)) {
      status = FVC_ERR_NAN;
      break;
    }
    if (relres <= a.target) {
      status = FVC_OK;
      break;
    }
    if (sweep == a.max_refine || inner_total >= a.maxit) break;
    const double d = res[2];  // r.z with z = r/m
    const double stop2 = a.inner_tol * a.inner_tol * fabs(d);
    MFOR_ROWS(P) {
      const float si = sv[row];
      r0[row] = si;
      p[row] = si;
      z[row] = si * minv[row];
      e[row] = make_float2(0.0f, 0.0f);
    }
    if (!grid_barrier(a.gs, ep)) return;
    int it = 0;
    for (;;) {
      ++it;
      // v = A z ; rr0 = s.r0 ; v.r0
      CSum c0, c1;
      MFOR_ROWS(P) {
        const float vi = arow32(a, s_, P.lane, row, [&](int k) { return z[k]; });
        v[row] = vi;
        const float r0i = r0[row];
        c0.add(sv[row] * r0i);
        c1.add(vi * r0i);
      }
      double acc[2] = {c0.value(), c1.value()};
      if (!grid_allreduce<2>(a.gs, ep, acc, red)) return;
      const double rr0 = acc[0];
      const float alpha = (float)(rr0 / acc[1]);
      // e += alpha z ; s -= alpha v ; z = s/m
      MFOR_ROWS(P) {
        e[row] = df_axpy(e[row], alpha, 0.0f, z[row]);
        const float si = fmaf(-alpha, v[row], sv[row]);
        sv[row] = si;
        z[row] = si * minv[row];
      }
      if (!grid_barrier(a.gs, ep)) return;
      // t = A z ; t.s ; t.t
      CSum c2, c3;
      MFOR_ROWS(P) {
        const float ti = arow32(a, s_, P.lane, row, [&](int k) { return z[k]; });
        t[row] = ti;
        c2.add(ti * sv[row]);
        c3.add(ti * ti);
      }
      acc[0] = c2.value();
      acc[1] = c3.value();
      if (!grid_allreduce<2>(a.gs, ep, acc, red)) return;
      const float omega = (acc[1] > 0.0) ? (float)(acc[0] / acc[1]) : 0.0f;
      // e += w z ; s -= w t ; s.z ; r0.s
      CSum c4, c5;
      MFOR_ROWS(P) {
        const float zi = z[row];
        e[row] = df_axpy(e[row], omega, 0.0f, zi);
        const float sn = fmaf(-omega, t[row], sv[row]);
        sv[row] = sn;
        c4.add(sn * zi);
        c5.add(r0[row] * sn);
      }
      double acc2[2] = {c4.value(), c5.value()};
      if (!grid_allreduce<2>(a.gs, ep, acc2, red)) return;
      if (!(acc2[0] == acc2[0]) || fabs(acc2[0]) <= stop2 || inner_total + it >= a.maxit ||
          omega == 0.0f)
        break;
      const float beta = (float)((acc2[1] / rr0) * ((double)alpha / (double)omega));
      // p = s + beta (p - w v) ; z = p/m
      MFOR_ROWS(P) {
        const float pi = fmaf(beta, fmaf(-omega, v[row], p[row]), sv[row]);
        p[row] = pi;
        z[row] = pi * minv[row];
      }
      if (!grid_barrier(a.gs, ep)) return;
    }
    inner_total += it;
    fold_correction(a);
    if (!grid_barrier(a.gs, ep)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.iresult[0] = sweep;
    a.iresult[1] = status;
    a.iresult[2] = inner_total;
    a.result[2] = relres;
    a.result[3] = res[0];
    a.result[4] = bnorm2;
  }
}

int sm_count_m() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

}  // namespace

int32_t build_f32_copy(DeviceMatrix &A, cudaStream_t stream) {
  if (A.have32) return FVC_OK;
  const size_t sl = (size_t)std::max<int64_t>(A.slots, 1);
  if (!A.val32 && cudaMalloc(&A.val32, sizeof(float) * sl) != cudaSuccess) return FVC_ERR_CUDA;
  if (!A.diag32 && cudaMalloc(&A.diag32, sizeof(float) * (size_t)A.n) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (!A.minv32 && cudaMalloc(&A.minv32, sizeof(float) * (size_t)A.n) != cudaSuccess)
    return FVC_ERR_CUDA;
  int blocks = std::max(1, std::min((A.nslices + 7) / 8, sm_count_m() * 8));
  build_f32_operator<<<blocks, 256, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.val, A.jac,
                                                 A.val32, A.diag32, A.minv32);
  count_launch();
  if (cudaStreamSynchronize(stream) != cudaSuccess) return FVC_ERR_CUDA;
  A.have32 = true;
  return FVC_OK;
}

int32_t run_mixed(const DeviceMatrix &A0, Scratch &S, int code, const double *b, double *x,
                  double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                  fvc_stats *st) {
  DeviceMatrix &A = const_cast<DeviceMatrix &>(A0);
  if (code != 1 && code != 2) return FVC_ERR_UNSUPPORTED;
  int32_t rc = build_f32_copy(A, stream);
  if (rc != FVC_OK) return rc;
  const size_t n = (size_t)A.n;
  if (S.nf < n) {
    for (int i = 0; i < 10; ++i) {
      if (S.f[i]) cudaFree(S.f[i]);
      S.f[i] = nullptr;
    }
    S.nf = n;
  }
  for (int i = 0; i < 10; ++i)  // f[4] holds the float2 correction
    if (!S.f[i] && cudaMalloc(&S.f[i], sizeof(float) * (i == 4 ? 2 : 1) * (n + 64)) != cudaSuccess)
      return FVC_ERR_CUDA;
  auto kern = (code == 1) ? mixed_cg : mixed_bicgstab;
  const int threads = (o.block_threads > 0) ? o.block_threads : 1024;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, 0);
  if (occ <= 0) occ = 1;
  if (o.blocks_per_sm > 0 && o.blocks_per_sm < occ) occ = o.blocks_per_sm;
  const int warps = threads / 32;
  int blocks = std::max(1, std::min(occ * sm_count_m(), (A.nslices + warps - 1) / warps));
  if (ensure_sync(S, (size_t)blocks) != FVC_OK) return FVC_ERR_CUDA;
  reset_sync(S, stream);
  MArgs a{};
  a.A.n = A.n;
  a.A.nslices = A.nslices;
  a.A.sptr = A.sptr;
  a.A.col = A.col;
  a.A.val = A.val;
  a.A.diag = A.diag;
  a.A.diag_mode = A.diag_mode;
  a.w32 = A.val32;
  a.e32 = A.diag32;
  a.minv = A.minv32;
  a.jac = A.jac;
  a.b = b;
  a.x = x;
  a.rs = S.f[0];
  a.pa = S.f[1];
  a.pb = S.f[2];
  a.q = S.f[3];
  a.e = reinterpret_cast<float2 *>(S.f[4]);
  a.r0 = S.f[5];
  a.t = S.f[6];
  a.v = S.f[7];
  a.z = S.f[8];
  a.rsl = (code == 1) ? S.f[9] : nullptr;
  a.gs = make_sync(S, blocks);
  a.target = (o.refine_tol > 0) ? o.refine_tol : tol;
  a.inner_tol = (o.inner_tol > 0) ? o.inner_tol : (code == 1 ? 0.1 : 1e-4);
  a.max_refine = (o.max_refine > 0) ? o.max_refine : 30;
  a.update_beta = o.update_beta;
  a.maxit = maxit;
  a.init = init;
  a.result = S.result;
  a.iresult = S.iresult;
  a.trace = S.trace;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream);
  void *args[] = {&a};
  cudaError_t ce =
      cudaLaunchCooperativeKernel((const void *)kern, dim3(blocks), dim3(threads), args, 0, stream);
  count_launch();
  cudaEventRecord(e1, stream);
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: cooperative launch failed: %s\n", cudaGetErrorString(ce));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return FVC_ERR_CUDA;
  }
  double res[16];
  int ires[16], err = 0;
  cudaMemcpyAsync(res, S.result, sizeof(res), cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(ires, S.iresult, sizeof(ires), cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(&err, S.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
  ce = cudaStreamSynchronize(stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) return FVC_ERR_CUDA;
  if (err != 0) return FVC_ERR_TIMEOUT;
  if (st) {
    st->status = ires[1];
    st->iterations = ires[2];
    st->inner_iterations = ires[2];
    st->refinements = ires[0];  // CG: reliable updates; BiCGSTAB: sweeps
    st->energy = 0.0;
    st->conv = a.target;
    st->final_crit = res[2];
    st->rel_residual = res[2];
    st->solve_ms = ms;
  }
  return ires[1];
}

}  // namespace fvc
